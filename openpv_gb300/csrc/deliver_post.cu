// deliver_post.cu -- a5: postsynaptic-perspective delivery (dense gather) in FP32.
//
// The reference computes, for every restricted target neuron, the dot product of its
// receptive field (nypPost rows of nxpPost*nf contiguous source values, starting at the
// unshrunken patch start) with the post-perspective weights
// (PostsynapticPerspectiveConvolveDelivery.cpp:56-151); its GPU path hands this to
// cudnnConvolutionForward after permuting NHWC->NCHW (CudaRecvPost.cpp:357-389).
//
// FAST mode is an implicit GEMM read straight from the NHWC extended activity: M = target
// positions, N = target features, K = nypPost * nxpPost * src.nf.  Positions are grouped by
// kernel phase (x mod nkx, y mod nky) so that one CTA tile shares one weight matrix.  CTA
// tile 64 x 64, K step 16, 256 threads each holding a 4 x 4 accumulator block; the
// receptive-field gather and the weight tile are staged through shared memory with a
// register prefetch of the next K step.  REFERENCE_ORDER mode runs one thread per target
// neuron with the reference's loop order and separately rounded products and sums.
#include "pvgpu_internal.cuh"

namespace {

using pvgpu::Axis;
using pvgpu::Loc;

struct PostGeom {
   Loc src, tgt;
   Axis ax, ay;       // tgt -> src geometry (pre = target layer, post = source layer)
   int nxpP, nypP;    // post-perspective patch
   int nkx, nky;      // kernel phases of the target layer
   int nkf;           // = tgt.nf
   int K, numPerStride, sy;
   float dtf;
};

// unshrunken source start (extended index) for a restricted target position (x, y)
__device__ __forceinline__ int64_t src_start(const PostGeom &g, int x, int y) {
   int sx = g.ax.start(x + g.tgt.lt) + g.src.lt;
   int sy = g.ay.start(y + g.tgt.dn) + g.src.dn;
   return ((int64_t)sy * g.src.nxExt() + sx) * g.src.nf;
}

__device__ __forceinline__ int post_kernel(const PostGeom &g, int x, int y, int f) {
   return ((y % g.nky) * g.nkx + (x % g.nkx)) * g.nkf + f;
}

constexpr int BM = 64, BN = 64, BK = 16, kThreads = 256;

__global__ void __launch_bounds__(kThreads) post_gemm_kernel(PostGeom g, const float *__restrict__ aExt,
                                                             const float *__restrict__ W,
                                                             float *__restrict__ gsyn) {
   __shared__ float As[2][BK][BM + 4];
   __shared__ float Bs[2][BK][BN + 4];
   __shared__ int64_t rowBase[BM];

   const int phase = blockIdx.z;
   const int phx = phase % g.nkx, phy = phase / g.nkx;
   const int nxPh = g.tgt.nx / g.nkx, nyPh = g.tgt.ny / g.nky;
   const int64_t perImg = (int64_t)nxPh * nyPh;
   const int64_t M = perImg * g.tgt.nb;
   const int64_t m0 = (int64_t)blockIdx.x * BM;
   const int n0 = blockIdx.y * BN;
   const int tid = threadIdx.x;

   if (tid < BM) {
      int64_t m = m0 + tid;
      int64_t base = -1;
      if (m < M) {
         int b = (int)(m / perImg);
         int r = (int)(m % perImg);
         int x = phx + g.nkx * (r % nxPh), y = phy + g.nky * (r / nxPh);
         base = (int64_t)b * g.src.numExt() + src_start(g, x, y);
      }
      rowBase[tid] = base;
   }
   __syncthreads();

   // loader mapping: A: 64 rows x 16 k -> each thread 4 (row = tid % 64, k = tid / 64 * 4 + j)
   //                 B: 16 k x 64 cols -> each thread 4 (col = tid % 64, k = tid / 64 * 4 + j)
   const int lrow = tid & 63, lk = (tid >> 6) * 4;
   const int64_t myBase = rowBase[lrow];
   const int ncol = n0 + lrow;
   const float *wcol = ncol < g.nkf ? W + (size_t)post_kernel(g, phx, phy, ncol) * g.K : nullptr;

   float ra[4], rb[4];
   auto loadTile = [&](int k0) {
#pragma unroll
      for (int j = 0; j < 4; j++) {
         int k = k0 + lk + j;
         float av = 0.0f, bv = 0.0f;
         if (k < g.K) {
            if (myBase >= 0) {
               int ky = k / g.numPerStride, r = k - ky * g.numPerStride;
               av = __ldg(aExt + myBase + (int64_t)ky * g.sy + r);
            }
            if (wcol) bv = __ldg(wcol + k);
         }
         ra[j] = av;
         rb[j] = bv;
      }
   };
   auto storeTile = [&](int buf) {
#pragma unroll
      for (int j = 0; j < 4; j++) {
         As[buf][lk + j][lrow] = ra[j];
         Bs[buf][lk + j][lrow] = rb[j];
      }
   };

   const int tm = (tid >> 4) * 4, tn = (tid & 15) * 4;
   float acc[4][4];
#pragma unroll
   for (int i = 0; i < 4; i++)
#pragma unroll
      for (int j = 0; j < 4; j++) acc[i][j] = 0.0f;

   const int nk = (g.K + BK - 1) / BK;
   loadTile(0);
   storeTile(0);
   __syncthreads();
   for (int t = 0; t < nk; t++) {
      const int cur = t & 1;
      if (t + 1 < nk) loadTile((t + 1) * BK);
#pragma unroll
      for (int kk = 0; kk < BK; kk++) {
         float4 a4 = *reinterpret_cast<const float4 *>(&As[cur][kk][tm]);
         float4 b4 = *reinterpret_cast<const float4 *>(&Bs[cur][kk][tn]);
         float av[4] = {a4.x, a4.y, a4.z, a4.w}, bv[4] = {b4.x, b4.y, b4.z, b4.w};
#pragma unroll
         for (int i = 0; i < 4; i++)
#pragma unroll
            for (int j = 0; j < 4; j++) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
      }
      if (t + 1 < nk) storeTile(cur ^ 1);
      __syncthreads();
   }

   // epilogue: gsyn += dtf * acc
#pragma unroll
   for (int i = 0; i < 4; i++) {
      int64_t m = m0 + tm + i;
      if (m >= M) continue;
      int b = (int)(m / perImg);
      int r = (int)(m % perImg);
      int x = phx + g.nkx * (r % nxPh), y = phy + g.nky * (r / nxPh);
      float *gp = gsyn + (size_t)b * g.tgt.numRes() + ((size_t)y * g.tgt.nx + x) * g.tgt.nf;
#pragma unroll
      for (int j = 0; j < 4; j++) {
         int n = n0 + tn + j;
         if (n < g.nkf) gp[n] = fmaf(g.dtf, acc[i][j], gp[n]);
      }
   }
}

// REFERENCE_ORDER: one thread per restricted target neuron, loops as in the reference.
__global__ void post_exact_kernel(PostGeom g, const float *__restrict__ aExt, const float *__restrict__ W,
                                  float *__restrict__ gsyn) {
   int64_t idxAll = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
   int64_t nRes = g.tgt.numRes();
   if (idxAll >= nRes * g.tgt.nb) return;
   int b = (int)(idxAll / nRes);
   int64_t idx = idxAll % nRes;
   int f = (int)(idx % g.tgt.nf);
   int x = (int)((idx / g.tgt.nf) % g.tgt.nx);
   int y = (int)(idx / ((int64_t)g.tgt.nf * g.tgt.nx));
   const float *a0 = aExt + (size_t)b * g.src.numExt() + src_start(g, x, y);
   const float *w0 = W + (size_t)post_kernel(g, x, y, f) * g.K;
   float gs = gsyn[idxAll];
   for (int ky = 0; ky < g.nypP; ky++) {
      const float *a = a0 + (int64_t)ky * g.sy;
      const float *w = w0 + ky * g.numPerStride;
      float dv = 0.0f;
      for (int k = 0; k < g.numPerStride; k++) dv = __fadd_rn(dv, __fmul_rn(a[k], w[k]));
      gs = __fadd_rn(gs, __fmul_rn(g.dtf, dv));
   }
   gsyn[idxAll] = gs;
}

}  // namespace

extern "C" pvgpu_status pvgpu_deliver_post(const pvgpu_conn_desc *conn, const float *aExt, const float *postWeights,
                                           float *gsyn, int mode, void *stream) {
   if (!conn || !aExt || !postWeights || !gsyn) return PVGPU_ERR_BAD_ARG;
   const pvgpu_loc &pre = conn->pre, &post = conn->post;
   if (!pvgpu::loc_valid(pre) || !pvgpu::loc_valid(post) || pre.nbatch != post.nbatch) return PVGPU_ERR_BAD_ARG;
   if (!pvgpu::axis_legal(pre.nx, post.nx, conn->nxp) || !pvgpu::axis_legal(pre.ny, post.ny, conn->nyp))
      return PVGPU_ERR_ILLEGAL_GEOMETRY;
   PostGeom g;
   g.src = pvgpu::to_loc(pre);
   g.tgt = pvgpu::to_loc(post);
   g.nxpP = pvgpu::post_patch_size(conn->nxp, pre.nx, post.nx);
   g.nypP = pvgpu::post_patch_size(conn->nyp, pre.ny, post.ny);
   // The post-perspective read needs the whole unshrunken receptive field inside the halo.
   int mx = pvgpu::required_margin(post.nx, pre.nx, g.nxpP), my = pvgpu::required_margin(post.ny, pre.ny, g.nypP);
   if (pre.halo.lt < mx || pre.halo.rt < mx || pre.halo.dn < my || pre.halo.up < my) return PVGPU_ERR_BAD_ARG;
   // PatchGeometry::setPatchGeometry offsets x by the post halo's dn (components/PatchGeometry.cpp:194-206);
   // equal margins on both axes keep that identical to lt.
   if (pre.halo.lt != pre.halo.dn || pre.halo.lt != pre.halo.rt || pre.halo.dn != pre.halo.up)
      return PVGPU_ERR_UNSUPPORTED_SHAPE;
   g.ax = Axis{post.nx, pre.nx, g.nxpP, post.halo.lt};
   g.ay = Axis{post.ny, pre.ny, g.nypP, post.halo.dn};
   g.nkx = post.nx > pre.nx ? post.nx / pre.nx : 1;
   g.nky = post.ny > pre.ny ? post.ny / pre.ny : 1;
   g.nkf = post.nf;
   g.numPerStride = g.nxpP * pre.nf;
   g.K = g.nypP * g.numPerStride;
   g.sy = g.src.nxExt() * pre.nf;
   g.dtf = conn->dt_factor;
   cudaStream_t s = pvgpu::as_stream(stream);
   if (mode == PVGPU_DELIVER_REFERENCE_ORDER) {
      int64_t n = g.tgt.numRes() * g.tgt.nb;
      post_exact_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(g, aExt, postWeights, gsyn);
      PVGPU_CHECK_LAUNCH("deliver_post exact");
      return PVGPU_OK;
   }
   int64_t M = (int64_t)(post.nx / g.nkx) * (post.ny / g.nky) * post.nbatch;
   int64_t gx = (M + BM - 1) / BM;
   int gy = (post.nf + BN - 1) / BN;
   if (gx > 0x7fffffff || gy > 65535) return PVGPU_ERR_UNSUPPORTED_SHAPE;
   dim3 grid((unsigned)gx, gy, g.nkx * g.nky);
   post_gemm_kernel<<<grid, kThreads, 0, s>>>(g, aExt, postWeights, gsyn);
   PVGPU_CHECK_LAUNCH("deliver_post");
   return PVGPU_OK;
}
