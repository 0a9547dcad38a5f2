// tc_gemm.cu -- diagnostic: C[M][N] = A[M][K] * B[N][K]^T (B K-major) or A[M][K] * B[K][N]
// (B MN-major) with BF16 operands and FP32 accumulation on the 5th-generation tensor cores
// (TMA -> SW128 shared tiles -> tcgen05.mma -> TMEM -> tcgen05.ld).  It exercises the exact
// descriptor, pipeline and TMEM conventions the fused LCA kernels use, on a plain GEMM that a
// test compares with a host reference.  One CTA per 128-row tile, all N (<= 256) columns;
// 2-stage TMA ring.
#include "pvgpu_internal.cuh"
#include "tc_ptx.cuh"
#include "tmap.cuh"

namespace {

using namespace pvgpu::tc;

constexpr int kBM = 128, kBK = 64;

// BMN: B is [K][N] in global memory; each 64-deep K chunk lands as N / 64 tiles of 64 K rows x
// 128 B, 8 KB apart -- the layout of a K-major weight tile read as the MN-major operand.
template <bool BMN>
__global__ void __launch_bounds__(128) tc_gemm_kernel(const __grid_constant__ CUtensorMap tmA,
                                                      const __grid_constant__ CUtensorMap tmB, float *__restrict__ C,
                                                      int M, int N, int K, int *__restrict__ err) {
   extern __shared__ uint8_t smem_raw[];
   uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
   const int bytesA = kBM * kBK * 2, bytesB = N * kBK * 2;
   uint8_t *sA[2] = {smem, smem + bytesA + bytesB};
   uint8_t *sB[2] = {smem + bytesA, smem + 2 * bytesA + bytesB};
   __shared__ __align__(8) uint64_t full[2], empty[2], done;
   __shared__ uint32_t tmemBase;
   __shared__ int failed;

   const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
   const int m0 = blockIdx.x * kBM;
   const uint32_t ncols = N <= 32 ? 32 : (N <= 64 ? 64 : (N <= 128 ? 128 : 256));
   if (threadIdx.x == 0) {
      mbar_init(&full[0], 1);
      mbar_init(&full[1], 1);
      mbar_init(&empty[0], 1);
      mbar_init(&empty[1], 1);
      mbar_init(&done, 1);
      fence_mbar_init();
      failed = 0;
      prefetch_tmap(&tmA);
      prefetch_tmap(&tmB);
   }
   if (warp == 0) tmem_alloc(&tmemBase, ncols);
   tc_fence_before();
   __syncthreads();
   tc_fence_after();
   const uint32_t tmem = tmemBase;

   const int nk = K / kBK;
   if (threadIdx.x == 0) {
      const uint32_t idesc = BMN ? idesc_bf16_bmn(kBM, N) : idesc_bf16(kBM, N);
      int issued = 0, consumed = 0;  // TMA stage loads issued / waited for
      auto load_b = [&](int s, int kc) {
         if (BMN) {
            for (int j = 0; j < N / 64; j++) tma_load_2d(sB[s] + j * 8192, &tmB, &full[s], j * 64, kc * kBK);
         } else {
            tma_load_2d(sB[s], &tmB, &full[s], kc * kBK, 0);
         }
      };
      for (int kc = 0; kc < nk && kc < 2; kc++, issued++) {
         mbar_arrive_expect_tx(&full[kc], bytesA + bytesB);
         tma_load_2d(sA[kc], &tmA, &full[kc], kc * kBK, m0);
         load_b(kc, kc);
      }
      bool ok = true;
      for (int kc = 0; kc < nk && ok; kc++) {
         const int s = kc & 1;
         const uint32_t ph = (kc >> 1) & 1;
         if (!mbar_wait(&full[s], ph)) { ok = false; break; }
         consumed++;
         tc_fence_after();
         const uint32_t a0 = smem_u32(sA[s]), b0 = smem_u32(sB[s]);
#pragma unroll
         for (int k = 0; k < kBK / 16; k++)
            mma_bf16(tmem, sdesc_sw128(a0 + k * 32), BMN ? sdesc_sw128_mn(b0 + k * 2048, 8192) : sdesc_sw128(b0 + k * 32),
                     idesc, (kc | k) != 0);
         mma_commit(&empty[s]);
         if (kc + 2 < nk) {
            if (!mbar_wait(&empty[s], ph)) { ok = false; break; }
            mbar_arrive_expect_tx(&full[s], bytesA + bytesB);
            tma_load_2d(sA[s], &tmA, &full[s], (kc + 2) * kBK, m0);
            load_b(s, kc + 2);
            issued++;
         }
      }
      mma_commit(&done);
      if (!ok) {
         failed = 1;
         // let the copies still in flight land before the CTA's shared memory goes away
         for (int i = consumed; i < issued; i++) mbar_wait(&full[i & 1], (i >> 1) & 1);
      }
   }
   __syncthreads();
   bool ok = __syncthreads_and(failed == 0 && mbar_wait(&done, 0));
   tc_fence_after();
   if (ok) {
      const int row = m0 + warp * 32 + lane;
      for (int c = 0; c < N; c += 32) {
         float v[32];
         tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + c, v);
         if (row < M) {
#pragma unroll
            for (int j = 0; j < 32; j++)
               if (c + j < N) C[(size_t)row * N + c + j] = v[j];
         }
      }
   } else if (threadIdx.x == 0) {
      atomicExch(err, 1);
   }
   tc_fence_before();
   __syncthreads();
   if (warp == 0) tmem_dealloc(tmem, ncols);
}

}  // namespace

namespace {

pvgpu_status tc_gemm(const void *A, const void *B, float *C, int M, int N, int K, int *errFlag, void *stream, bool bmn) {
   if (!A || !B || !C || !errFlag || M <= 0 || N < 16 || N > 256 || (N % 16) || K < 64 || (K % 64) || (M % 128) ||
       (bmn && N % 64))
      return PVGPU_ERR_BAD_ARG;
   CUtensorMap tmA, tmB;
   if (!pvgpu::make_tmap_bf16_sw128(&tmA, A, M, K, K, kBM) ||
       !(bmn ? pvgpu::make_tmap_bf16_sw128(&tmB, B, K, N, N, kBK) : pvgpu::make_tmap_bf16_sw128(&tmB, B, N, K, K, N)))
      return PVGPU_ERR_BAD_ARG;
   size_t smem = 2 * (size_t)(kBM * kBK * 2 + N * kBK * 2) + 1024;
   auto fn = bmn ? tc_gemm_kernel<true> : tc_gemm_kernel<false>;
   cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
   if (e != cudaSuccess) return pvgpu::record_cuda_error(e, "tc_gemm attr");
   fn<<<M / kBM, 128, smem, pvgpu::as_stream(stream)>>>(tmA, tmB, C, M, N, K, errFlag);
   PVGPU_CHECK_LAUNCH("tc_gemm");
   return PVGPU_OK;
}

// A from tensor memory: each thread (row m of the 128-row tile) loads its row of A (BF16, K
// <= 256) from global memory and stores it into TMEM lane m, two K elements per column; B (K-
// major, [N][K]) by TMA into SW128 shared tiles, all of K at once; MMAs read A from TMEM.
__global__ void __launch_bounds__(128) tc_gemm_atmem_kernel(const __grid_constant__ CUtensorMap tmB,
                                                            const uint16_t *__restrict__ A, float *__restrict__ C,
                                                            int M, int N, int K, int *__restrict__ err) {
   extern __shared__ uint8_t smem_raw[];
   uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
   __shared__ __align__(8) uint64_t full, done;
   __shared__ uint32_t tmemBase;
   const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
   const int m0 = blockIdx.x * kBM, nk = K / kBK;
   if (threadIdx.x == 0) {
      mbar_init(&full, 1);
      mbar_init(&done, 1);
      fence_mbar_init();
      prefetch_tmap(&tmB);
   }
   if (warp == 0) tmem_alloc(&tmemBase, 512);
   tc_fence_before();
   __syncthreads();
   tc_fence_after();
   const uint32_t tmem = tmemBase, aCol = 256;  // D in columns 0..N-1, A from column 256
   if (threadIdx.x == 0) {
      mbar_arrive_expect_tx(&full, (uint32_t)(nk * N * kBK * 2));
      for (int kc = 0; kc < nk; kc++) tma_load_2d(smem + kc * N * kBK * 2, &tmB, &full, kc * kBK, 0);
   }
   // row m of A into lane m: columns aCol + k/2 hold (A[m][k], A[m][k+1])
   const int row = m0 + warp * 32 + lane;
   const uint32_t *arow = reinterpret_cast<const uint32_t *>(A + (size_t)row * K);
   for (int c = 0; c < K / 2; c += 8) {
      uint32_t r[8];
#pragma unroll
      for (int j = 0; j < 8; j++) r[j] = arow[c + j];
      tmem_st8(tmem + ((uint32_t)(warp * 32) << 16) + aCol + c, r);
   }
   tmem_wait_st();
   tc_fence_before();
   __syncthreads();
   tc_fence_after();
   int ok = 1;
   if (threadIdx.x == 0) {
      ok = mbar_wait(&full, 0);
      if (ok) {
         tc_fence_after();
         const uint32_t idesc = idesc_bf16(kBM, N);
         for (int kc = 0; kc < nk; kc++) {
            const uint32_t b0 = smem_u32(smem + kc * N * kBK * 2);
#pragma unroll
            for (int k = 0; k < kBK / 16; k++)
               mma_bf16_ta(tmem, tmem + aCol + (uint32_t)((kc * kBK + k * 16) / 2), sdesc_sw128(b0 + k * 32), idesc,
                           (kc | k) != 0);
         }
      }
      mma_commit(&done);
   }
   ok = __syncthreads_and(ok && mbar_wait(&done, 0));
   tc_fence_after();
   if (ok) {
      for (int c = 0; c < N; c += 32) {
         float v[32];
         tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + c, v);
         if (row < M) {
#pragma unroll
            for (int j = 0; j < 32; j++)
               if (c + j < N) C[(size_t)row * N + c + j] = v[j];
         }
      }
   } else if (threadIdx.x == 0) {
      atomicExch(err, 1);
   }
   tc_fence_before();
   __syncthreads();
   if (warp == 0) tmem_dealloc(tmem, 512);
}

}  // namespace

extern "C" pvgpu_status pvgpu_tc_gemm_bf16_atmem(const void *A, const void *B, float *C, int M, int N, int K,
                                                 int *errFlag, void *stream) {
   if (!A || !B || !C || !errFlag || M <= 0 || N < 16 || N > 256 || (N % 16) || K < 64 || K > 256 || (K % 64) ||
       (M % 128) || (reinterpret_cast<uintptr_t>(A) & 3))
      return PVGPU_ERR_BAD_ARG;
   CUtensorMap tmB;
   if (!pvgpu::make_tmap_bf16_sw128(&tmB, B, N, K, K, N)) return PVGPU_ERR_BAD_ARG;
   const size_t smem = (size_t)(K / kBK) * N * kBK * 2 + 1024;
   cudaError_t e = cudaFuncSetAttribute(tc_gemm_atmem_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
   if (e != cudaSuccess) return pvgpu::record_cuda_error(e, "tc_gemm attr");
   tc_gemm_atmem_kernel<<<M / kBM, 128, smem, pvgpu::as_stream(stream)>>>(tmB, static_cast<const uint16_t *>(A), C, M,
                                                                          N, K, errFlag);
   PVGPU_CHECK_LAUNCH("tc_gemm atmem");
   return PVGPU_OK;
}

extern "C" pvgpu_status pvgpu_tc_gemm_bf16(const void *A, const void *B, float *C, int M, int N, int K, int *errFlag,
                                           void *stream) {
   return tc_gemm(A, B, C, M, N, K, errFlag, stream, false);
}

extern "C" pvgpu_status pvgpu_tc_gemm_bf16_kn(const void *A, const void *B, float *C, int M, int N, int K,
                                              int *errFlag, void *stream) {
   return tc_gemm(A, B, C, M, N, K, errFlag, stream, true);
}

// ---------------------------------------------------------------------------------------------
// Diagnostic: the expiry path of a bounded device wait.  One CTA holds TMEM like the
// warp-specialised kernels do; warp 1 waits on an mbarrier that nothing arrives at, with the
// caller's time limit; when the wait gives up it raises the CTA's abort flag, which warp 2 (a
// role polling the flag between work items, like the load warps) sees and leaves its loop by.
// The CTA then frees its TMEM and reports {timed out, ns waited} -- the discipline every
// kernel of the library follows on a timeout, without a fault or a hang.
namespace {

__global__ void __launch_bounds__(96) wait_expiry_kernel(uint64_t limitNs, long long *out) {
   __shared__ __align__(8) uint64_t never;
   __shared__ uint32_t tmemBase;
   __shared__ volatile int abortFlag;
   const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
   if (threadIdx.x == 0) {
      mbar_init(&never, 1);
      abortFlag = 0;
      fence_mbar_init();
   }
   if (warp == 0) tmem_alloc(&tmemBase, 32);
   tc_fence_before();
   __syncthreads();
   tc_fence_after();
   long long waited = 0;
   if (warp == 1 && lane == 0) {
      const uint64_t t0 = global_ns();
      if (!mbar_wait(&never, 0, limitNs)) abortFlag = 1;
      waited = (long long)(global_ns() - t0);
   } else if (warp == 2) {
      // polls the abort flag; its own loop is bounded too (twice the wait's limit)
      const uint64_t t0 = global_ns();
      while (!abortFlag && global_ns() - t0 < 2 * limitNs) __nanosleep(1000);
   }
   __syncthreads();
   if (threadIdx.x == 32) {
      out[0] = abortFlag ? 1 : 0;
      out[1] = waited;
   }
   tc_fence_before();
   __syncthreads();
   if (warp == 0) tmem_dealloc(tmemBase, 32);
}

}  // namespace

extern "C" pvgpu_status pvgpu_selftest_wait_expiry(uint64_t limitNs, long long *hostOut2, void *stream) {
   if (!hostOut2 || limitNs == 0 || limitNs > 1000000000ull) return PVGPU_ERR_BAD_ARG;
   cudaStream_t s = pvgpu::as_stream(stream);
   long long *d = nullptr;
   cudaError_t e = cudaMallocAsync(&d, 2 * sizeof(long long), s);
   if (e != cudaSuccess) return pvgpu::record_cuda_error(e, "selftest_wait_expiry");
   wait_expiry_kernel<<<1, 96, 0, s>>>(limitNs, d);
   e = cudaGetLastError();
   if (e == cudaSuccess) e = cudaMemcpyAsync(hostOut2, d, 2 * sizeof(long long), cudaMemcpyDeviceToHost, s);
   cudaError_t f = cudaFreeAsync(d, s);
   if (e == cudaSuccess) e = f;
   if (e == cudaSuccess) e = cudaStreamSynchronize(s);
   if (e != cudaSuccess) return pvgpu::record_cuda_error(e, "selftest_wait_expiry");
   return hostOut2[0] ? PVGPU_ERR_TIMEOUT : PVGPU_OK;
}
