// weights.cu -- a3 / a12: weight transpose for post-perspective delivery and the Hebbian
// weight update (the weight gradient of delivery).
#include "pvgpu_internal.cuh"

namespace {

using pvgpu::Axis;
using pvgpu::Loc;

struct TGeom {
   int nxp, nyp, nfp;           // pre patch (nfp = post.nf)
   int nkx, nky, nkf;           // pre kernels
   int xStride, yStride, xTStride, yTStride;
   int nxpPost, nypPost;
   int nkxPost, nkyPost, nkfPost;
};

// PatchGeometry::setTransposeItemIndices (components/PatchGeometry.cpp:264-332) and
// TransposeWeights::transposeShared (utils/TransposeWeights.cpp:56-115), one thread per pre weight.
__global__ void transpose_kernel(TGeom g, const float *__restrict__ wPre, float *__restrict__ wPost) {
   const int patchSize = g.nxp * g.nyp * g.nfp;
   const int64_t total = (int64_t)g.nkx * g.nky * g.nkf * patchSize;
   int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
   if (t >= total) return;
   int kp = (int)(t / patchSize), item = (int)(t % patchSize);
   int kxPre = (kp / g.nkf) % g.nkx, kyPre = kp / (g.nkf * g.nkx), kfPre = kp % g.nkf;
   int ixPre = (item / g.nfp) % g.nxp, iyPre = item / (g.nfp * g.nxp), ifPre = item % g.nfp;
   int extX = (g.nxp - 1) * g.xStride / 2;
   int ksX = (kxPre - extX) % g.xStride;
   if (ksX < 0) ksX += g.xStride;
   int ixPost = (g.xStride * (g.nxp - 1 - ixPre) + ksX) / g.xTStride;
   int extY = (g.nyp - 1) * g.yStride / 2;
   int ksY = (kyPre - extY) % g.yStride;
   if (ksY < 0) ksY += g.yStride;
   int iyPost = (g.yStride * (g.nyp - 1 - iyPre) + ksY) / g.yTStride;
   int itemPost = (iyPost * g.nxpPost + ixPost) * g.nkf + kfPre;
   int pxPost = 0, pyPost = 0;
   if (g.nkxPost > 1) {
      pxPost = (-(g.nxp - g.nkxPost) / 2 + ixPre) % g.nkxPost;
      if (pxPost < 0) pxPost += g.nkxPost;
   }
   if (g.nkyPost > 1) {
      pyPost = (-(g.nyp - g.nkyPost) / 2 + iyPre) % g.nkyPost;
      if (pyPost < 0) pyPost += g.nkyPost;
   }
   int patchPost = (pyPost * g.nkxPost + pxPost) * g.nkfPost + ifPre;
   int patchSizePost = g.nxpPost * g.nypPost * g.nkf;
   wPost[(size_t)patchPost * patchSizePost + itemPost] = wPre[t];
}

struct HGeom {
   Loc pre, post;
   Axis ax, ay;
   int nxp, nyp, nfp;
   int nkx, nky, nkf;
   float dWMax;
};

// HebbianUpdater::update_dW / updateInd_dW (weightupdaters/HebbianUpdater.cpp:476-629):
// one thread per weight (kernel, ky, kx, fp).  It visits the batch, then the kernel's unit
// cells in (y, x) order -- the order the reference accumulates into that weight -- and adds
// dWMax*pre*post wherever the weight lies inside the (shrunken) patch.
__global__ void hebbian_kernel(HGeom g, const float *__restrict__ preExt, const float *__restrict__ postExt,
                               float *__restrict__ dw) {
   const int patchSize = g.nxp * g.nyp * g.nfp;
   const int64_t total = (int64_t)g.nkx * g.nky * g.nkf * patchSize;
   int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
   if (t >= total) return;
   int kernel = (int)(t / patchSize), item = (int)(t % patchSize);
   int kxc = (kernel / g.nkf) % g.nkx, kyc = kernel / (g.nkf * g.nkx), kf = kernel % g.nkf;
   int kx = (item / g.nfp) % g.nxp, ky = item / (g.nfp * g.nxp), fp = item % g.nfp;
   const int nxExt = g.pre.nxExt(), nyExt = g.pre.nyExt();
   const int64_t nPreExt = g.pre.numExt(), nPostExt = g.post.numExt();
   const int postNxExt = g.post.nxExt();
   float acc = 0.0f;
   for (int b = 0; b < g.pre.nb; b++) {
      const float *pb = preExt + (size_t)b * nPreExt;
      const float *qb = postExt + (size_t)b * nPostExt;
      for (int ye = kyc; ye < nyExt; ye += g.nky) {
         int py = g.ay.start(ye) + ky;
         if (py < 0 || py >= g.post.ny) continue;
         for (int xe = kxc; xe < nxExt; xe += g.nkx) {
            int px = g.ax.start(xe) + kx;
            if (px < 0 || px >= g.post.nx) continue;
            float a = pb[((int64_t)ye * nxExt + xe) * g.pre.nf + kf];
            if (a == 0.0f) continue;
            // the x offset uses the post halo's dn, as PatchGeometry::setPatchGeometry's aPostOffset
            // does (components/PatchGeometry.cpp:194-206); margins are equal on both axes in practice
            float q = qb[((int64_t)(py + g.post.dn) * postNxExt + (px + g.post.dn)) * g.post.nf + fp];
            acc = __fadd_rn(acc, __fmul_rn(__fmul_rn(g.dWMax, a), q));
         }
      }
   }
   dw[t] = acc;
}

}  // namespace

extern "C" pvgpu_status pvgpu_transpose_weights(const pvgpu_conn_desc *conn, const float *preWeights,
                                                float *postWeights, void *stream) {
   if (!conn || !preWeights || !postWeights) return PVGPU_ERR_BAD_ARG;
   const pvgpu_loc &pre = conn->pre, &post = conn->post;
   if (!pvgpu::loc_valid(pre) || !pvgpu::loc_valid(post)) return PVGPU_ERR_BAD_ARG;
   if (!pvgpu::axis_legal(pre.nx, post.nx, conn->nxp) || !pvgpu::axis_legal(pre.ny, post.ny, conn->nyp))
      return PVGPU_ERR_ILLEGAL_GEOMETRY;
   TGeom g;
   g.nxp = conn->nxp;
   g.nyp = conn->nyp;
   g.nfp = post.nf;
   g.nkx = pre.nx > post.nx ? pre.nx / post.nx : 1;
   g.nky = pre.ny > post.ny ? pre.ny / post.ny : 1;
   g.nkf = pre.nf;
   g.xStride = g.nkx;
   g.yStride = g.nky;
   g.xTStride = post.nx > pre.nx ? post.nx / pre.nx : 1;
   g.yTStride = post.ny > pre.ny ? post.ny / pre.ny : 1;
   g.nxpPost = g.nxp * g.xStride / g.xTStride;
   g.nypPost = g.nyp * g.yStride / g.yTStride;
   g.nkxPost = g.xTStride;
   g.nkyPost = g.yTStride;
   g.nkfPost = post.nf;
   int64_t total = (int64_t)g.nkx * g.nky * g.nkf * g.nxp * g.nyp * g.nfp;
   transpose_kernel<<<(unsigned)((total + 255) / 256), 256, 0, pvgpu::as_stream(stream)>>>(g, preWeights, postWeights);
   PVGPU_CHECK_LAUNCH("transpose_weights");
   return PVGPU_OK;
}

extern "C" pvgpu_status pvgpu_hebbian_dw(const pvgpu_conn_desc *conn, float dWMax, const float *preExt,
                                         const float *postExt, float *dw, void *stream) {
   if (!conn || !preExt || !postExt || !dw) return PVGPU_ERR_BAD_ARG;
   const pvgpu_loc &pre = conn->pre, &post = conn->post;
   if (!pvgpu::loc_valid(pre) || !pvgpu::loc_valid(post) || pre.nbatch != post.nbatch) return PVGPU_ERR_BAD_ARG;
   if (!pvgpu::axis_legal(pre.nx, post.nx, conn->nxp) || !pvgpu::axis_legal(pre.ny, post.ny, conn->nyp))
      return PVGPU_ERR_ILLEGAL_GEOMETRY;
   HGeom g;
   g.pre = pvgpu::to_loc(pre);
   g.post = pvgpu::to_loc(post);
   g.ax = Axis{pre.nx, post.nx, conn->nxp, pre.halo.lt};
   g.ay = Axis{pre.ny, post.ny, conn->nyp, pre.halo.dn};
   g.nxp = conn->nxp;
   g.nyp = conn->nyp;
   g.nfp = post.nf;
   g.nkx = pre.nx > post.nx ? pre.nx / post.nx : 1;
   g.nky = pre.ny > post.ny ? pre.ny / post.ny : 1;
   g.nkf = pre.nf;
   g.dWMax = dWMax;
   int64_t total = (int64_t)g.nkx * g.nky * g.nkf * g.nxp * g.nyp * g.nfp;
   hebbian_kernel<<<(unsigned)((total + 127) / 128), 128, 0, pvgpu::as_stream(stream)>>>(g, preExt, postExt, dw);
   PVGPU_CHECK_LAUNCH("hebbian_dw");
   return PVGPU_OK;
}

// ---- MomentumUpdater (weightupdaters/MomentumUpdater.cpp:291-345) ----------------------------
// applyMomentum then prev_dW = dW then HebbianUpdater::updateWeights (W += dW), one thread per
// weight, every operation separately rounded as the reference's loop does.
namespace {
__global__ void momentum_weights_kernel(int64_t n, float dwFactor, float wFactor, float *__restrict__ dw,
                                        float *__restrict__ prevDw, float *__restrict__ w) {
   const float keep = __fadd_rn(1.0f, -dwFactor);
   for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
      float d = __fmul_rn(dw[k], keep);
      d = __fadd_rn(d, __fmul_rn(dwFactor, prevDw[k]));
      const float wk = w[k];
      d = __fadd_rn(d, -__fmul_rn(wFactor, wk));
      dw[k] = d;
      prevDw[k] = d;
      w[k] = __fadd_rn(wk, d);
   }
}
}  // namespace

extern "C" pvgpu_status pvgpu_momentum_factors(char method, float tau, float decay, float dWMax, float *dwFactor,
                                               float *wFactor) {
   if (!dwFactor || !wFactor) return PVGPU_ERR_BAD_ARG;
   switch (method) {
      case 'v':  // viscosity: exp(-1/tau), 0 when tau is 0 (host expf, as the reference)
         *dwFactor = tau != 0.0f ? std::exp(-1.0f / tau) : 0.0f;
         *wFactor = decay;
         return PVGPU_OK;
      case 's':
         *dwFactor = tau;
         *wFactor = decay;
         return PVGPU_OK;
      case 'a':
         *dwFactor = tau;
         *wFactor = decay * dWMax;
         return PVGPU_OK;
      default: return PVGPU_ERR_BAD_ARG;
   }
}

extern "C" pvgpu_status pvgpu_momentum_update_weights(int64_t n, float dwFactor, float wFactor, float *dw,
                                                      float *prevDw, float *w, void *stream) {
   if (n < 0 || (n > 0 && (!dw || !prevDw || !w))) return PVGPU_ERR_BAD_ARG;
   if (n == 0) return PVGPU_OK;
   const int64_t blocks = (n + 255) / 256;
   momentum_weights_kernel<<<(unsigned)(blocks < 4096 ? blocks : 4096), 256, 0, pvgpu::as_stream(stream)>>>(
         n, dwFactor, wFactor, dw, prevDw, w);
   PVGPU_CHECK_LAUNCH("momentum_update_weights");
   return PVGPU_OK;
}
