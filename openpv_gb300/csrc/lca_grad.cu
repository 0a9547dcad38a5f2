// lca_grad.cu -- the gradient of unrolled LCA (differentiable dictionary learning) on the device,
// behind the C ABI: L(W) = 0.5 ||x - W^T a_T||^2 + lambda ||a_T||_1 after T LCA timesteps from
// V = 0, with the soft threshold a = T(V) = max(V - VThresh, 0) (ANNActivityBuffer with AMin = 0,
// AShift = VThresh, VWidth = 0), V' = e V + (1 - e)(W r + a), r = x - W^T a, e = exp(-dt/tau)
// (HyPerLCAInternalStateBuffer.kpp:18-63 with selfInteract), and dL/dW.  The reference learns its
// dictionaries with the Hebbian rule (weightupdaters/HebbianUpdater.cpp:476-629): the gradient of
// the loss of a fixed activity a is minus that update (dWMax = 1); here the whole unrolled solve is
// differentiated, with a checkpoint every K timesteps.
//
// Both deliveries are GEMMs over the im2col'd operands.  Row-major, M = nbatch * positions:
//   recon:  D[M][KP] = A[M][F] . W[F][KP],  y = fold(D)   (patch k of position p adds to pixel
//           (S*py - E + ky, S*px - E + kx, c), E = (P - S) / 2 -- PatchGeometry's one-to-many start)
//   drive:  R[M][KP] = im2col(x - y),  Z[M][F] = R . W^T
// and their adjoints (the transpose delivery and the pre (x) post-error correlation):
//   gR = (1 - e) g . W,  gr = fold(gR),  gD = -im2col(gr),  gA = gD . W^T,
//   g <- e g + [V >= VThresh] ((1 - e) g + gA),   dW += (1 - e) g^T R + A^T gD
// where g = dL/dV of the later step; the correlations of a whole segment run as two GEMMs over all
// its steps' positions (K = steps x positions).  The final loss seeds g_T = [V_T >= VThresh](-Z_T + lambda [a_T > 0])
// and dW = -A_T^T R_T.
//
// The GEMMs are plain library GEMMs and run on cuBLAS in FP32 emulated on the BF16 tensor cores
// (CUBLAS_COMPUTE_32F_EMULATED_16BFX9: each operand split in three BF16 parts, FP32 accuracy), or
// in plain FP32 where that mode is refused.  cuBLAS is loaded at the first create, so the rest of
// the library does not depend on it.  Everything else -- fold, im2col, the update and its adjoint,
// the threshold mask, the loss -- is the kernels below.  A run is one CUDA graph (captured once
// per set of pointers, replayed on the caller's stream).
#include "pvgpu_internal.cuh"

#include <cublas_v2.h>
#include <dlfcn.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

namespace {

constexpr int kThreads = 256;

struct Geo {
   int nb, iny, inx, C, vy, vx, F, P, S, E, KP, Np;
   int64_t M;  // nb * Np
};

__device__ __forceinline__ float soft(float v, float vt) { return v >= vt ? v - vt : 0.0f; }

__global__ void threshold_kernel(int64_t n, float vt, const float *__restrict__ v, float *__restrict__ a) {
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
      a[i] = soft(v[i], vt);
}

// out[b][iy][ix][c] = (x ? x : 0) + sign * sum over the positions whose patch covers the pixel of
// D[b, p][k] (positions ascending in y, then x: a fixed order, no atomics).
__global__ void fold_kernel(Geo g, const float *__restrict__ D, const float *__restrict__ x, float sign,
                            float *__restrict__ out) {
   const int n = g.nb * g.iny * g.inx * g.C;
   for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
      const int c = i % g.C;
      const int ix = (i / g.C) % g.inx;
      const int iy = (i / (g.C * g.inx)) % g.iny;
      const int b = i / (g.C * g.inx * g.iny);
      // positions py with 0 <= iy - (S*py - E) < P
      const int pyLo = max(0, (iy + g.E - g.P + g.S) / g.S), pyHi = min(g.vy - 1, (iy + g.E) / g.S);
      const int pxLo = max(0, (ix + g.E - g.P + g.S) / g.S), pxHi = min(g.vx - 1, (ix + g.E) / g.S);
      float s = 0.0f;
      for (int py = pyLo; py <= pyHi; py++) {
         const int ky = iy - (g.S * py - g.E);
         for (int px = pxLo; px <= pxHi; px++) {
            const int kx = ix - (g.S * px - g.E);
            s += D[((int64_t)b * g.Np + py * g.vx + px) * g.KP + (ky * g.P + kx) * g.C + c];
         }
      }
      out[i] = (x ? x[i] : 0.0f) + sign * s;
   }
}

// R[b, p][k] = sign * img[b][S*py - E + ky][S*px - E + kx][c], 0 outside the image.  One block
// per row (b, p); the threads walk k.
__global__ void im2col_kernel(Geo g, const float *__restrict__ img, float sign, float *__restrict__ R) {
   const int row = blockIdx.x;
   const int p = row % g.Np, b = row / g.Np;
   const int iy0 = g.S * (p / g.vx) - g.E, ix0 = g.S * (p % g.vx) - g.E;
   const float *ib = img + (size_t)b * g.iny * g.inx * g.C;
   float *out = R + (size_t)row * g.KP;
   const int PC = g.P * g.C;
   for (int k = threadIdx.x; k < g.KP; k += blockDim.x) {
      const int ky = k / PC, r = k - ky * PC, kx = r / g.C, c = r - kx * g.C;
      const int iy = iy0 + ky, ix = ix0 + kx;
      float v = 0.0f;
      if (iy >= 0 && iy < g.iny && ix >= 0 && ix < g.inx) v = ib[(iy * g.inx + ix) * g.C + c];
      out[k] = sign * v;
   }
}

// WT[k][f] = W[f][k] (the weights as the K-major operand of the reconstruction GEMM).
__global__ void transpose_kernel(int F, int KP, const float *__restrict__ W, float *__restrict__ WT) {
   __shared__ float tile[32][33];
   const int f0 = blockIdx.y * 32, k0 = blockIdx.x * 32;
   for (int j = threadIdx.y; j < 32; j += blockDim.y)
      if (f0 + j < F && k0 + threadIdx.x < KP) tile[j][threadIdx.x] = W[(size_t)(f0 + j) * KP + k0 + threadIdx.x];
   __syncthreads();
   for (int j = threadIdx.y; j < 32; j += blockDim.y)
      if (k0 + j < KP && f0 + threadIdx.x < F) WT[(size_t)(k0 + j) * F + f0 + threadIdx.x] = tile[threadIdx.x][j];
}

// V' = e V + (1 - e)(Z + A), A' = T(V')
__global__ void update_kernel(int n, float e, float vt, const float *__restrict__ v, const float *__restrict__ a,
                              const float *__restrict__ z, float *__restrict__ vOut, float *__restrict__ aOut) {
   const float om = 1.0f - e;
   for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
      const float vn = e * v[i] + om * (z[i] + a[i]);
      vOut[i] = vn;
      aOut[i] = soft(vn, vt);
   }
}

// gOut = e g + [V >= vt] ((1 - e) g + gA)
__global__ void adjoint_update_kernel(int n, float e, float vt, const float *__restrict__ v,
                                      const float *__restrict__ gA, const float *__restrict__ g,
                                      float *__restrict__ gOut) {
   const float om = 1.0f - e;
   for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
      const float gv = g[i];
      gOut[i] = e * gv + (v[i] >= vt ? om * gv + gA[i] : 0.0f);
   }
}

// g_T = [V_T >= vt] (lambda [A_T > 0] - Z_T)
__global__ void seed_kernel(int64_t n, float vt, float lambda, const float *__restrict__ v,
                            const float *__restrict__ a, const float *__restrict__ z, float *__restrict__ gV) {
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
      gV[i] = v[i] >= vt ? (a[i] > 0.0f ? lambda : 0.0f) - z[i] : 0.0f;
}

// Per-block partial sums of 0.5 r^2 (r: nr values) + lambda |a| (a: na values), in FP64; then
// one block adds the partials in block order (deterministic).
constexpr int kLossBlocks = 256;
__global__ void loss_partial_kernel(int64_t nr, const float *__restrict__ r, int64_t na, const float *__restrict__ a,
                                    double lambda, double *__restrict__ partial) {
   double s = 0.0;
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nr; i += (int64_t)gridDim.x * blockDim.x)
      s += 0.5 * (double)r[i] * (double)r[i];
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < na; i += (int64_t)gridDim.x * blockDim.x)
      s += lambda * fabs((double)a[i]);
   __shared__ double red[kThreads];
   red[threadIdx.x] = s;
   __syncthreads();
   for (int w = kThreads / 2; w > 0; w >>= 1) {
      if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
      __syncthreads();
   }
   if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void loss_final_kernel(const double *__restrict__ partial, int n, double *__restrict__ out) {
   if (threadIdx.x == 0 && blockIdx.x == 0) {
      double s = 0.0;
      for (int i = 0; i < n; i++) s += partial[i];
      *out = s;
   }
}

// ---- cuBLAS, loaded at first use --------------------------------------------------------------
struct Blas {
   void *so = nullptr;
   cublasStatus_t (*create)(cublasHandle_t *) = nullptr;
   cublasStatus_t (*destroy)(cublasHandle_t) = nullptr;
   cublasStatus_t (*setStream)(cublasHandle_t, cudaStream_t) = nullptr;
   cublasStatus_t (*setWorkspace)(cublasHandle_t, void *, size_t) = nullptr;
   cublasStatus_t (*gemmEx)(cublasHandle_t, cublasOperation_t, cublasOperation_t, int, int, int, const void *,
                            const void *, cudaDataType, int, const void *, cudaDataType, int, const void *, void *,
                            cudaDataType, int, cublasComputeType_t, cublasGemmAlgo_t) = nullptr;
   cublasStatus_t (*setSpecialValues)(cublasHandle_t, cudaEmulationSpecialValuesSupport) = nullptr;  // optional
   bool ok = false;
};

Blas g_blas;
std::once_flag g_blas_once;

void load_blas() {
   const char *env = getenv("PVGPU_CUBLAS");
   const char *names[] = {env, "libcublas.so.13", "/usr/local/cuda/lib64/libcublas.so.13",
                          "/usr/local/cuda/lib64/libcublas.so", "libcublas.so"};
   for (const char *n : names) {
      if (!n) continue;
      g_blas.so = dlopen(n, RTLD_NOW | RTLD_GLOBAL);
      if (g_blas.so) break;
   }
   if (!g_blas.so) return;
   g_blas.create = reinterpret_cast<decltype(g_blas.create)>(dlsym(g_blas.so, "cublasCreate_v2"));
   g_blas.destroy = reinterpret_cast<decltype(g_blas.destroy)>(dlsym(g_blas.so, "cublasDestroy_v2"));
   g_blas.setStream = reinterpret_cast<decltype(g_blas.setStream)>(dlsym(g_blas.so, "cublasSetStream_v2"));
   g_blas.setWorkspace = reinterpret_cast<decltype(g_blas.setWorkspace)>(dlsym(g_blas.so, "cublasSetWorkspace_v2"));
   g_blas.gemmEx = reinterpret_cast<decltype(g_blas.gemmEx)>(dlsym(g_blas.so, "cublasGemmEx"));
   g_blas.setSpecialValues = reinterpret_cast<decltype(g_blas.setSpecialValues)>(
         dlsym(g_blas.so, "cublasSetEmulationSpecialValuesSupport"));
   g_blas.ok = g_blas.create && g_blas.destroy && g_blas.setStream && g_blas.setWorkspace && g_blas.gemmEx;
}

unsigned grid_for(int64_t n) {
   int64_t b = (n + kThreads - 1) / kThreads;
   return (unsigned)(b > 152 * 32 ? 152 * 32 : (b < 1 ? 1 : b));
}

}  // namespace

struct pvgpu_lca_grad {
   pvgpu_lca_grad_desc d;
   Geo g;
   float e = 0.f;
   int nseg = 0;
   cublasHandle_t blas = nullptr;
   cublasComputeType_t compute = CUBLAS_COMPUTE_32F_EMULATED_16BFX9;
   void *blasWs = nullptr;
   size_t blasWsBytes = 0;
   // device buffers (FP32 unless noted)
   float *V[2] = {nullptr, nullptr}, *A[2] = {nullptr, nullptr};  // forward ping-pong [M][F]
   float *ck = nullptr;                  // checkpoints: V at the start of each segment [nseg][M][F]
   float *sV = nullptr, *sA = nullptr;   // one segment's states [K][M][F]
   float *sR = nullptr;                  // one segment's im2col'd residuals [K][M][KP]
   float *sG = nullptr;                  // one segment's adjoints dL/dV of the later state [K][M][F]
   float *sGD = nullptr;                 // one segment's -im2col(fold(gR)) [K][M][KP]
   float *WT = nullptr;                  // W transposed [KP][F]
   float *D = nullptr, *R = nullptr, *Z = nullptr, *img = nullptr;
   float *gV = nullptr, *gR = nullptr, *gD = nullptr, *gA = nullptr, *gImg = nullptr;
   double *lossPartial = nullptr;
   cudaStream_t capStream = nullptr;
   cudaGraphExec_t graph = nullptr;
   const float *gW = nullptr, *gX = nullptr;
   float *gDW = nullptr;
   double *gLoss = nullptr;
};

namespace {

// C[M][N] = alpha A[M][K] . op(B) + beta C, all row-major FP32.  transB: B is [N][K] (so op(B) =
// B^T), else [K][N].  cuBLAS is column-major: C^T = op(B)^T A^T.
pvgpu_status gemm_rm(pvgpu_lca_grad *s, cudaStream_t st, int64_t M, int64_t N, int64_t K, float alpha,
                     const float *Am, const float *B, bool transB, float beta, float *Cm) {
   (void)st;
   const cublasStatus_t r =
         g_blas.gemmEx(s->blas, transB ? CUBLAS_OP_T : CUBLAS_OP_N, CUBLAS_OP_N, (int)N, (int)M, (int)K, &alpha, B,
                       CUDA_R_32F, transB ? (int)K : (int)N, Am, CUDA_R_32F, (int)K, &beta, Cm, CUDA_R_32F, (int)N,
                       s->compute, CUBLAS_GEMM_DEFAULT);
   return r == CUBLAS_STATUS_SUCCESS ? PVGPU_OK : pvgpu::record_message(PVGPU_ERR_LAUNCH, "lca_grad: cublasGemmEx failed");
}

// C[M][N] = alpha A^T . B + beta C with A [K][M], B [K][N] row-major (the correlation over K):
// C^T = B^T A in column-major terms.
pvgpu_status gemm_tn(pvgpu_lca_grad *s, int64_t M, int64_t N, int64_t K, float alpha, const float *Am,
                     const float *B, float beta, float *Cm) {
   const cublasStatus_t r =
         g_blas.gemmEx(s->blas, CUBLAS_OP_N, CUBLAS_OP_T, (int)N, (int)M, (int)K, &alpha, B, CUDA_R_32F, (int)N, Am,
                       CUDA_R_32F, (int)M, &beta, Cm, CUDA_R_32F, (int)N, s->compute, CUBLAS_GEMM_DEFAULT);
   return r == CUBLAS_STATUS_SUCCESS ? PVGPU_OK : pvgpu::record_message(PVGPU_ERR_LAUNCH, "lca_grad: cublasGemmEx failed");
}

#define PVGPU_TRY(x)                   \
   do {                                \
      pvgpu_status st_ = (x);          \
      if (st_ != PVGPU_OK) return st_; \
   } while (0)

// One forward timestep from (v, a) to (vOut, aOut); the im2col'd residual goes to Rout.
pvgpu_status forward_step(pvgpu_lca_grad *s, cudaStream_t st, const float *W, const float *x, const float *v,
                          const float *a, float *vOut, float *aOut, float *Rout) {
   const Geo &g = s->g;
   PVGPU_TRY(gemm_rm(s, st, g.M, g.KP, g.F, 1.0f, a, s->WT, true, 0.0f, s->D));  // D = A . W
   const int64_t nImg = (int64_t)g.nb * g.iny * g.inx * g.C;
   fold_kernel<<<grid_for(nImg), kThreads, 0, st>>>(g, s->D, x, -1.0f, s->img);  // r = x - fold(D)
   im2col_kernel<<<(unsigned)g.M, kThreads, 0, st>>>(g, s->img, 1.0f, Rout);
   PVGPU_TRY(gemm_rm(s, st, g.M, g.F, g.KP, 1.0f, Rout, W, true, 0.0f, s->Z));  // Z = R . W^T
   update_kernel<<<grid_for(g.M * g.F), kThreads, 0, st>>>((int)(g.M * g.F), s->e, s->d.VThresh, v, a, s->Z, vOut,
                                                           aOut);
   PVGPU_CHECK_LAUNCH("lca_grad forward");
   return PVGPU_OK;
}

pvgpu_status enqueue(pvgpu_lca_grad *s, const float *W, const float *x, float *dW, double *loss, cudaStream_t st) {
   const Geo &g = s->g;
   const int T = s->d.steps, K = s->d.checkpointEvery;
   const int64_t nV = g.M * g.F, nRk = g.M * g.KP;
   const float vt = s->d.VThresh, e = s->e;
   transpose_kernel<<<dim3((g.KP + 31) / 32, (g.F + 31) / 32), dim3(32, 8), 0, st>>>(g.F, g.KP, W, s->WT);
   // ---- forward, V = 0, checkpoint V at the start of every segment ----
   PVGPU_CUDA(cudaMemsetAsync(s->V[0], 0, nV * sizeof(float), st), "lca_grad zero");
   PVGPU_CUDA(cudaMemsetAsync(s->A[0], 0, nV * sizeof(float), st), "lca_grad zero");
   int cur = 0;
   for (int t = 0; t < T; t++) {
      if (t % K == 0)
         PVGPU_CUDA(cudaMemcpyAsync(s->ck + (size_t)(t / K) * nV, s->V[cur], nV * sizeof(float), cudaMemcpyDeviceToDevice,
                                    st),
                    "lca_grad checkpoint");
      PVGPU_TRY(forward_step(s, st, W, x, s->V[cur], s->A[cur], s->V[1 - cur], s->A[1 - cur], s->R));
      cur = 1 - cur;
   }
   // ---- the loss at a_T, and the seed of the adjoint ----
   PVGPU_TRY(gemm_rm(s, st, g.M, g.KP, g.F, 1.0f, s->A[cur], s->WT, true, 0.0f, s->D));
   const int64_t nImg = (int64_t)g.nb * g.iny * g.inx * g.C;
   fold_kernel<<<grid_for(nImg), kThreads, 0, st>>>(g, s->D, x, -1.0f, s->img);  // r_T
   im2col_kernel<<<(unsigned)g.M, kThreads, 0, st>>>(g, s->img, 1.0f, s->R);     // R_T
   PVGPU_TRY(gemm_rm(s, st, g.M, g.F, g.KP, 1.0f, s->R, W, true, 0.0f, s->Z));  // Z_T = R_T . W^T
   loss_partial_kernel<<<kLossBlocks, kThreads, 0, st>>>(nImg, s->img, nV, s->A[cur], (double)s->d.lambda1,
                                                         s->lossPartial);
   loss_final_kernel<<<1, 32, 0, st>>>(s->lossPartial, kLossBlocks, loss);
   seed_kernel<<<grid_for(nV), kThreads, 0, st>>>(nV, vt, s->d.lambda1, s->V[cur], s->A[cur], s->Z, s->gV);
   PVGPU_TRY(gemm_tn(s, g.F, g.KP, g.M, -1.0f, s->A[cur], s->R, 0.0f, dW));  // dW = -A_T^T R_T
   PVGPU_CHECK_LAUNCH("lca_grad loss");
   // ---- segments in reverse: recompute the segment's states, then its adjoint steps ----
   for (int seg = s->nseg - 1; seg >= 0; seg--) {
      const int t0 = seg * K, t1 = t0 + K < T ? t0 + K : T, n = t1 - t0;
      PVGPU_CUDA(cudaMemcpyAsync(s->sV, s->ck + (size_t)seg * nV, nV * sizeof(float), cudaMemcpyDeviceToDevice, st),
                 "lca_grad restore");
      threshold_kernel<<<grid_for(nV), kThreads, 0, st>>>(nV, vt, s->sV, s->sA);
      for (int i = 0; i < n; i++) {
         // state i + 1 goes to slot i + 1; the segment's last output is not needed
         float *vo = i + 1 < n ? s->sV + (size_t)(i + 1) * nV : s->V[0];
         float *ao = i + 1 < n ? s->sA + (size_t)(i + 1) * nV : s->A[0];
         PVGPU_TRY(forward_step(s, st, W, x, s->sV + (size_t)i * nV, s->sA + (size_t)i * nV, vo, ao,
                                s->sR + (size_t)i * nRk));
      }
      // the adjoint steps: g of step i lives in sG[i]; step i writes dL/dV_t into sG[i - 1], or
      // into gV for the segment before
      PVGPU_CUDA(cudaMemcpyAsync(s->sG + (size_t)(n - 1) * nV, s->gV, nV * sizeof(float), cudaMemcpyDeviceToDevice, st),
                 "lca_grad adjoint carry");
      for (int i = n - 1; i >= 0; i--) {
         const float *Vt = s->sV + (size_t)i * nV, *gi = s->sG + (size_t)i * nV;
         float *gDi = s->sGD + (size_t)i * nRk;
         PVGPU_TRY(gemm_rm(s, st, g.M, g.KP, g.F, 1.0f - e, gi, s->WT, true, 0.0f, s->gR));  // gR = (1-e) g . W
         fold_kernel<<<grid_for(nImg), kThreads, 0, st>>>(g, s->gR, nullptr, 1.0f, s->gImg);  // gr = fold(gR)
         im2col_kernel<<<(unsigned)g.M, kThreads, 0, st>>>(g, s->gImg, -1.0f, gDi);         // gD = -im2col(gr)
         PVGPU_TRY(gemm_rm(s, st, g.M, g.F, g.KP, 1.0f, gDi, W, true, 0.0f, s->gA));        // gA = gD . W^T
         adjoint_update_kernel<<<grid_for(nV), kThreads, 0, st>>>((int)nV, e, vt, Vt, s->gA, gi,
                                                                  i > 0 ? s->sG + (size_t)(i - 1) * nV : s->gV);
         PVGPU_CHECK_LAUNCH("lca_grad adjoint");
      }
      // the segment's correlations, each one GEMM over all its steps' positions:
      // dW += (1 - e) sum_i g_i^T R_i + sum_i A_i^T gD_i
      PVGPU_TRY(gemm_tn(s, g.F, g.KP, (int64_t)n * g.M, 1.0f - e, s->sG, s->sR, 1.0f, dW));
      PVGPU_TRY(gemm_tn(s, g.F, g.KP, (int64_t)n * g.M, 1.0f, s->sA, s->sGD, 1.0f, dW));
   }
   return PVGPU_OK;
}

void free_all(pvgpu_lca_grad *s) {
   if (!s) return;
   if (s->graph) cudaGraphExecDestroy(s->graph);
   if (s->capStream) cudaStreamDestroy(s->capStream);
   if (s->blas) g_blas.destroy(s->blas);
   void *bufs[] = {s->V[0], s->V[1], s->A[0], s->A[1], s->ck, s->sV, s->sA, s->sR, s->sG, s->sGD, s->WT, s->D, s->R,
                   s->Z, s->img, s->gV, s->gR, s->gD, s->gA, s->gImg, s->lossPartial, s->blasWs};
   for (void *p : bufs)
      if (p) cudaFree(p);
   delete s;
}

}  // namespace

extern "C" pvgpu_status pvgpu_lca_grad_create(const pvgpu_lca_grad_desc *d, pvgpu_lca_grad **out) {
   if (!d || !out) return PVGPU_ERR_BAD_ARG;
   *out = nullptr;
   if (d->nbatch <= 0 || d->inNx <= 0 || d->inNy <= 0 || d->inNf <= 0 || d->v1Nx <= 0 || d->v1Ny <= 0 ||
       d->v1Nf <= 0 || d->nxp <= 0 || d->steps <= 0 || d->checkpointEvery <= 0 || !(d->tau > 0.0f) ||
       !(d->dt > 0.0f))
      return PVGPU_ERR_BAD_ARG;
   if (d->inNx % d->v1Nx || d->inNy % d->v1Ny || d->inNx / d->v1Nx != d->inNy / d->v1Ny)
      return pvgpu::record_message(PVGPU_ERR_UNSUPPORTED_SHAPE, "lca_grad: V1 must tile the input with one stride");
   const int S = d->inNx / d->v1Nx;
   if (d->nxp < S || (d->nxp - S) % 2)
      return pvgpu::record_message(PVGPU_ERR_ILLEGAL_GEOMETRY, "lca_grad: patch must exceed the stride by an even amount");
   std::call_once(g_blas_once, load_blas);
   if (!g_blas.ok) return pvgpu::record_message(PVGPU_ERR_UNSUPPORTED_SHAPE, "lca_grad: cuBLAS could not be loaded");
   pvgpu_lca_grad *s = new (std::nothrow) pvgpu_lca_grad();
   if (!s) return PVGPU_ERR_OOM;
   s->d = *d;
   Geo &g = s->g;
   g.nb = d->nbatch;
   g.iny = d->inNy;
   g.inx = d->inNx;
   g.C = d->inNf;
   g.vy = d->v1Ny;
   g.vx = d->v1Nx;
   g.F = d->v1Nf;
   g.P = d->nxp;
   g.S = S;
   g.E = (d->nxp - S) / 2;
   g.KP = g.P * g.P * g.C;
   g.Np = g.vy * g.vx;
   g.M = (int64_t)g.nb * g.Np;
   s->e = (float)std::exp(-(double)d->dt / (double)d->tau);
   const int K = d->checkpointEvery;
   s->nseg = (d->steps + K - 1) / K;
   const size_t nV = (size_t)g.M * g.F, nR = (size_t)g.M * g.KP, nImg = (size_t)g.nb * g.iny * g.inx * g.C;
   bool ok = true;
   auto alloc = [&](void **p, size_t bytes) {
      if (ok && cudaMalloc(p, bytes) != cudaSuccess) ok = false;
   };
   for (int i = 0; i < 2; i++) {
      alloc(reinterpret_cast<void **>(&s->V[i]), nV * 4);
      alloc(reinterpret_cast<void **>(&s->A[i]), nV * 4);
   }
   alloc(reinterpret_cast<void **>(&s->ck), (size_t)s->nseg * nV * 4);
   alloc(reinterpret_cast<void **>(&s->sV), (size_t)K * nV * 4);
   alloc(reinterpret_cast<void **>(&s->sA), (size_t)K * nV * 4);
   alloc(reinterpret_cast<void **>(&s->sR), (size_t)K * nR * 4);
   alloc(reinterpret_cast<void **>(&s->sG), (size_t)K * nV * 4);
   alloc(reinterpret_cast<void **>(&s->sGD), (size_t)K * nR * 4);
   alloc(reinterpret_cast<void **>(&s->WT), (size_t)g.F * g.KP * 4);
   alloc(reinterpret_cast<void **>(&s->D), nR * 4);
   alloc(reinterpret_cast<void **>(&s->R), nR * 4);
   alloc(reinterpret_cast<void **>(&s->Z), nV * 4);
   alloc(reinterpret_cast<void **>(&s->img), nImg * 4);
   alloc(reinterpret_cast<void **>(&s->gV), nV * 4);
   alloc(reinterpret_cast<void **>(&s->gR), nR * 4);
   alloc(reinterpret_cast<void **>(&s->gD), nR * 4);
   alloc(reinterpret_cast<void **>(&s->gA), nV * 4);
   alloc(reinterpret_cast<void **>(&s->gImg), nImg * 4);
   alloc(reinterpret_cast<void **>(&s->lossPartial), kLossBlocks * sizeof(double));
   s->blasWsBytes = 64u << 20;  // cuBLAS takes this instead of allocating (also inside a capture)
   alloc(&s->blasWs, s->blasWsBytes);
   if (!ok) {
      cudaGetLastError();
      free_all(s);
      return PVGPU_ERR_OOM;
   }
   if (g_blas.create(&s->blas) != CUBLAS_STATUS_SUCCESS ||
       g_blas.setWorkspace(s->blas, s->blasWs, s->blasWsBytes) != CUBLAS_STATUS_SUCCESS) {
      s->blas = nullptr;
      free_all(s);
      return pvgpu::record_message(PVGPU_ERR_LAUNCH, "lca_grad: cuBLAS handle");
   }
   // the operands are finite (a run with an inf or NaN in W or x has no meaningful gradient), so the
   // emulated GEMMs skip their scans for special values
   if (g_blas.setSpecialValues) g_blas.setSpecialValues(s->blas, CUDA_EMULATION_SPECIAL_VALUES_SUPPORT_NONE);
   if (cudaStreamCreateWithFlags(&s->capStream, cudaStreamNonBlocking) != cudaSuccess) {
      cudaGetLastError();
      s->capStream = nullptr;
   }
   // FP32 emulated on the BF16 tensor cores where cuBLAS takes it, else plain FP32: one probe GEMM
   {
      float *p = s->Z;
      const float one = 1.0f, zero = 0.0f;
      g_blas.setStream(s->blas, nullptr);
      if (g_blas.gemmEx(s->blas, CUBLAS_OP_N, CUBLAS_OP_N, 16, 16, 16, &one, p, CUDA_R_32F, 16, p, CUDA_R_32F, 16, &zero,
                        p + 256, CUDA_R_32F, 16, CUBLAS_COMPUTE_32F_EMULATED_16BFX9, CUBLAS_GEMM_DEFAULT) !=
          CUBLAS_STATUS_SUCCESS)
         s->compute = CUBLAS_COMPUTE_32F;
      cudaDeviceSynchronize();
      cudaGetLastError();
   }
   *out = s;
   return PVGPU_OK;
}

extern "C" pvgpu_status pvgpu_lca_grad_destroy(pvgpu_lca_grad *s) {
   if (!s) return PVGPU_ERR_BAD_ARG;
   free_all(s);
   return PVGPU_OK;
}

extern "C" pvgpu_status pvgpu_lca_grad_info(const pvgpu_lca_grad *s, int *emulatedFp32) {
   if (!s || !emulatedFp32) return PVGPU_ERR_BAD_ARG;
   *emulatedFp32 = s->compute == CUBLAS_COMPUTE_32F_EMULATED_16BFX9 ? 1 : 0;
   return PVGPU_OK;
}

extern "C" pvgpu_status pvgpu_lca_grad_run(pvgpu_lca_grad *s, const float *W, const float *x, float *dW,
                                           double *loss, void *stream) {
   if (!s || !W || !x || !dW || !loss) return PVGPU_ERR_BAD_ARG;
   cudaStream_t st = pvgpu::as_stream(stream);
   if (!s->capStream) {  // no capture stream: enqueue directly on the caller's stream
      if (g_blas.setStream(s->blas, st) != CUBLAS_STATUS_SUCCESS)
         return pvgpu::record_message(PVGPU_ERR_LAUNCH, "lca_grad: cublasSetStream");
      return enqueue(s, W, x, dW, loss, st);
   }
   if (!s->graph || s->gW != W || s->gX != x || s->gDW != dW || s->gLoss != loss) {
      if (s->graph) cudaGraphExecDestroy(s->graph);
      s->graph = nullptr;
      if (g_blas.setStream(s->blas, s->capStream) != CUBLAS_STATUS_SUCCESS)
         return pvgpu::record_message(PVGPU_ERR_LAUNCH, "lca_grad: cublasSetStream");
      PVGPU_CUDA(cudaStreamBeginCapture(s->capStream, cudaStreamCaptureModeThreadLocal), "lca_grad capture");
      pvgpu_status r = enqueue(s, W, x, dW, loss, s->capStream);
      cudaGraph_t gr = nullptr;
      cudaError_t ee = cudaStreamEndCapture(s->capStream, &gr);
      if (r != PVGPU_OK || ee != cudaSuccess) {
         if (gr) cudaGraphDestroy(gr);
         return r != PVGPU_OK ? r : pvgpu::record_cuda_error(ee, "lca_grad capture");
      }
      cudaError_t ei = cudaGraphInstantiate(&s->graph, gr, 0);
      cudaGraphDestroy(gr);
      if (ei != cudaSuccess) {
         s->graph = nullptr;
         return pvgpu::record_cuda_error(ei, "lca_grad instantiate");
      }
      s->gW = W;
      s->gX = x;
      s->gDW = dW;
      s->gLoss = loss;
   }
   PVGPU_CUDA(cudaGraphLaunch(s->graph, st), "lca_grad launch");
   return PVGPU_OK;
}
