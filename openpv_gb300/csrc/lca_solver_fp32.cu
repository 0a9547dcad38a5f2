// lca_solver_fp32.cu -- the plain FP32 form of the batched LCA solver: the same two fused
// kernels per timestep as lca_solver.cu (reconstruction partials, then residual + post
// delivery + LCA update), with the two GEMMs on the FP32 pipes (SIMT, shared-memory
// tiles, register blocking) instead of tcgen05, and FP32 activity.  It is the baseline
// the BF16 tensor-core form is measured against.
#include "lca_common.cuh"

namespace {

using pvgpu::LcaGeom;
using pvgpu::rwin_cols;

constexpr int kThreads = 256;

// D[pos][k] = sum_f A[pos][f] * W[f][k] for 128 positions, then the tap-group fold (the same
// group order as the tensor-core kernel) into this block's partial reconstruction.
template <int S, int P, int C>
__global__ void __launch_bounds__(kThreads) recon32_kernel(LcaGeom g, const float *__restrict__ A32,
                                                           const float *__restrict__ Wt32,
                                                           float *__restrict__ partials) {
   constexpr int KP = P * P * C, E = (P - S) / 2, TK = KP / 16, KPAD = KP + 1;
   extern __shared__ float sm[];
   float *As = sm;               // [16][128]
   float *Ws = As + 16 * 128;    // [16][KP]
   float *D = Ws + 16 * KP;      // [128][KP + 1]
   float *recon = D + 128 * KPAD;
   const int tid = threadIdx.x, tr = tid >> 4, tc = tid & 15;
   const int b = blockIdx.x / g.MB, mb = blockIdx.x % g.MB;
   const size_t rowA = (size_t)b * g.Npos + mb * 128;

   float acc[8][TK];
#pragma unroll
   for (int i = 0; i < 8; i++)
#pragma unroll
      for (int j = 0; j < TK; j++) acc[i][j] = 0.0f;

   for (int f0 = 0; f0 < g.F; f0 += 16) {
      {  // A chunk: 128 positions x 16 features, two float4 per thread
         const int p = tid >> 1, h = (tid & 1) * 8;
         const float4 *src = reinterpret_cast<const float4 *>(A32 + (rowA + p) * g.F + f0 + h);
         float4 u = src[0], v = src[1];
         As[(h + 0) * 128 + p] = u.x;
         As[(h + 1) * 128 + p] = u.y;
         As[(h + 2) * 128 + p] = u.z;
         As[(h + 3) * 128 + p] = u.w;
         As[(h + 4) * 128 + p] = v.x;
         As[(h + 5) * 128 + p] = v.y;
         As[(h + 6) * 128 + p] = v.z;
         As[(h + 7) * 128 + p] = v.w;
      }
      for (int i = tid; i < KP * 16; i += kThreads) {  // W^T chunk: KP rows x 16 features
         const int k = i >> 4, kk = i & 15;
         Ws[kk * KP + k] = Wt32[(size_t)k * g.F + f0 + kk];
      }
      __syncthreads();
#pragma unroll 4
      for (int kk = 0; kk < 16; kk++) {
         float a[8], w[TK];
#pragma unroll
         for (int i = 0; i < 8; i++) a[i] = As[kk * 128 + tr + 16 * i];
#pragma unroll
         for (int j = 0; j < TK; j++) w[j] = Ws[kk * KP + tc + 16 * j];
#pragma unroll
         for (int i = 0; i < 8; i++)
#pragma unroll
            for (int j = 0; j < TK; j++) acc[i][j] = fmaf(a[i], w[j], acc[i][j]);
      }
      __syncthreads();
   }
#pragma unroll
   for (int i = 0; i < 8; i++)
#pragma unroll
      for (int j = 0; j < TK; j++) D[(tr + 16 * i) * KPAD + tc + 16 * j] = acc[i][j];
   const int nPix = g.inNx * g.inNy * C;
   for (int i = tid; i < nPix; i += kThreads) recon[i] = 0.0f;
   __syncthreads();

   // fold, thread = position (threads 128..255 only take part in the barriers)
   const int pos = mb * 128 + (tid & 127);
   const int y1 = pos / g.v1Nx, x1 = pos % g.v1Nx;
   const int py0 = S * y1 - E, px0 = S * x1 - E;
   const float *drow = D + (tid & 127) * KPAD;
   for (int ty = 0; ty < P / S; ty++) {
#pragma unroll
      for (int tx = 0; tx < P / S; tx++) {
         if (tid < 128) {
#pragma unroll
            for (int dy = 0; dy < S; dy++) {
               const int ky = S * ty + dy, py = py0 + ky;
#pragma unroll
               for (int dx = 0; dx < S; dx++) {
                  const int kx = S * tx + dx, px = px0 + kx;
                  if (py >= 0 && py < g.inNy && px >= 0 && px < g.inNx) {
                     float *rp = recon + (py * g.inNx + px) * C;
#pragma unroll
                     for (int c = 0; c < C; c++) rp[c] += drow[(ky * P + kx) * C + c];
                  }
               }
            }
         }
         __syncthreads();
      }
   }
   float *out = partials + ((size_t)b * g.MB + mb) * nPix;
   for (int i = tid; i < nPix; i += kThreads) out[i] = recon[i];
}

// Residual window, D[pos][f] = sum_k r[pos][k] W[f][k] for 128 positions x NT features,
// then the LCA update of those neurons.
template <int S, int P, int C, int NT>
__global__ void __launch_bounds__(kThreads) post32_kernel(LcaGeom g, const float *__restrict__ x,
                                                          const float *__restrict__ partials,
                                                          const float *__restrict__ Wt32, float *__restrict__ V,
                                                          float *__restrict__ A32) {
   constexpr int KP = P * P * C, TN = NT / 16;
   extern __shared__ float sm[];
   float *As = sm;              // [16][128]
   float *Ws = As + 16 * 128;   // [16][NT]
   float *rwin = Ws + 16 * NT;
   const int tid = threadIdx.x, tr = tid >> 4, tc = tid & 15;
   const int nTilesN = g.F / NT;
   const int b = blockIdx.x / (g.MB * nTilesN);
   const int rem = blockIdx.x % (g.MB * nTilesN);
   const int mb = rem / nTilesN, f0 = (rem % nTilesN) * NT;
   const int RWC = rwin_cols(S, P, g.v1Nx);
   pvgpu::build_residual_window<S, P, C, kThreads>(g, b, mb, x, partials, rwin);
   __syncthreads();

   float acc[8][TN];
#pragma unroll
   for (int i = 0; i < 8; i++)
#pragma unroll
      for (int j = 0; j < TN; j++) acc[i][j] = 0.0f;
   for (int k0 = 0; k0 < KP; k0 += 16) {
      for (int i = tid; i < 16 * 128; i += kThreads) {  // im2col chunk, gathered from the window
         const int kk = i >> 7, p = i & 127;
         const int k = k0 + kk, ky = k / (P * C), kr = k % (P * C);
         const int yl = p / g.v1Nx, x1 = p % g.v1Nx;
         As[kk * 128 + p] = rwin[((S * yl + ky) * RWC + S * x1) * C + kr];
      }
      for (int i = tid; i < 16 * NT; i += kThreads) {
         const int kk = i / NT, f = i % NT;
         Ws[kk * NT + f] = Wt32[(size_t)(k0 + kk) * g.F + f0 + f];
      }
      __syncthreads();
#pragma unroll 4
      for (int kk = 0; kk < 16; kk++) {
         float a[8], w[TN];
#pragma unroll
         for (int i = 0; i < 8; i++) a[i] = As[kk * 128 + tr + 16 * i];
#pragma unroll
         for (int j = 0; j < TN; j++) w[j] = Ws[kk * NT + tc + 16 * j];
#pragma unroll
         for (int i = 0; i < 8; i++)
#pragma unroll
            for (int j = 0; j < TN; j++) acc[i][j] = fmaf(a[i], w[j], acc[i][j]);
      }
      __syncthreads();
   }
   // HyPerLCAInternalStateBuffer.kpp:52-61 and the threshold, rounded as the CPU path rounds
   const float e = g.e, om = __fadd_rn(1.0f, -g.e);
#pragma unroll
   for (int i = 0; i < 8; i++) {
      const int pos = mb * 128 + tr + 16 * i;
      const size_t row = ((size_t)b * g.Npos + pos) * g.F + f0;
#pragma unroll
      for (int j = 0; j < TN; j++) {
         const int f = tc + 16 * j;
         const size_t vi = pvgpu::v_index(g, b, pos, f0 + f);
         const float vo = V[vi];
         const float ao = pvgpu::lca_thresh(vo, g);
         const float vn = __fadd_rn(__fmul_rn(e, vo), __fmul_rn(om, __fadd_rn(acc[i][j], __fmul_rn(g.si, ao))));
         V[vi] = vn;
         A32[row + f] = pvgpu::lca_thresh(vn, g);
      }
   }
}

template <int S, int P, int C>
pvgpu_status step(const LcaGeom &g, const float *x, const float *Wt32, float *partials, float *V, float *A32,
                  cudaStream_t st, cudaEvent_t mid) {
   constexpr int KP = P * P * C;
   const size_t rs = sizeof(float) * (16 * 128 + 16 * KP + 128 * (KP + 1) + (size_t)g.inNx * g.inNy * C);
   auto rk = recon32_kernel<S, P, C>;
   cudaError_t e = cudaFuncSetAttribute(rk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rs);
   if (e != cudaSuccess) return pvgpu::record_cuda_error(e, "lca32 recon attr");
   rk<<<g.nb * g.MB, kThreads, rs, st>>>(g, A32, Wt32, partials);
   PVGPU_CHECK_LAUNCH("lca32 recon");
   if (mid) cudaEventRecord(mid, st);
   const size_t win = (size_t)pvgpu::rwin_rows(S, P, g.rowsPerBlock) * rwin_cols(S, P, g.v1Nx) * C;
   if (g.NT == 128) {
      const size_t ps = sizeof(float) * (16 * 128 + 16 * 128 + win);
      auto pk = post32_kernel<S, P, C, 128>;
      e = cudaFuncSetAttribute(pk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ps);
      if (e != cudaSuccess) return pvgpu::record_cuda_error(e, "lca32 post attr");
      pk<<<g.nb * g.MB * (g.F / 128), kThreads, ps, st>>>(g, x, partials, Wt32, V, A32);
   } else {
      const size_t ps = sizeof(float) * (16 * 128 + 16 * 64 + win);
      auto pk = post32_kernel<S, P, C, 64>;
      e = cudaFuncSetAttribute(pk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ps);
      if (e != cudaSuccess) return pvgpu::record_cuda_error(e, "lca32 post attr");
      pk<<<g.nb * g.MB * (g.F / 64), kThreads, ps, st>>>(g, x, partials, Wt32, V, A32);
   }
   PVGPU_CHECK_LAUNCH("lca32 post");
   return PVGPU_OK;
}

}  // namespace

namespace pvgpu {

pvgpu_status lca_fp32_step(int S, int P, int C, const LcaGeom &g, const float *x, const float *W32, const float *Wt32,
                           float *partials, float *V, float *A32, cudaStream_t st, cudaEvent_t mid) {
   (void)W32;
   if (S == 2 && P == 8 && C == 1) return step<2, 8, 1>(g, x, Wt32, partials, V, A32, st, mid);
   if (S == 2 && P == 8 && C == 3) return step<2, 8, 3>(g, x, Wt32, partials, V, A32, st, mid);
   if (S == 4 && P == 16 && C == 1) return step<4, 16, 1>(g, x, Wt32, partials, V, A32, st, mid);
   return PVGPU_ERR_UNSUPPORTED_SHAPE;
}

}  // namespace pvgpu
