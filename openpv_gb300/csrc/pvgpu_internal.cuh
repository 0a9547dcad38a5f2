// pvgpu_internal.cuh -- shared helpers of the libpvgpu translation units.
#pragma once

#include "pvgpu.h"

#include <cuda_runtime.h>
#include <stdint.h>

namespace pvgpu {

// Records the CUDA error string for pvgpu_last_error() and maps it to a status.
pvgpu_status record_cuda_error(cudaError_t err, const char *where);
// Records a plain message for pvgpu_last_error() and returns status.
pvgpu_status record_message(pvgpu_status status, const char *message);

#define PVGPU_CHECK_LAUNCH(where)                                                  \
   do {                                                                            \
      cudaError_t e_ = cudaGetLastError();                                         \
      if (e_ != cudaSuccess) return ::pvgpu::record_cuda_error(e_, where);         \
   } while (0)

#define PVGPU_CUDA(call, where)                                                    \
   do {                                                                            \
      cudaError_t e_ = (call);                                                     \
      if (e_ != cudaSuccess) return ::pvgpu::record_cuda_error(e_, where);         \
   } while (0)

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// Geometry of one layer, restated from include/PVLayerLoc.h and utils/conversions.hpp.
struct Loc {
   int nb, nx, ny, nf, lt, rt, dn, up;
   __host__ __device__ int nxExt() const { return nx + lt + rt; }
   __host__ __device__ int nyExt() const { return ny + dn + up; }
   __host__ __device__ int64_t numExt() const { return (int64_t)nxExt() * nyExt() * nf; }
   __host__ __device__ int64_t numRes() const { return (int64_t)nx * ny * nf; }
   // kIndexExtended (utils/conversions.hpp:402-407)
   __host__ __device__ int64_t kex(int64_t k) const {
      int f = (int)(k % nf);
      int x = (int)((k / nf) % nx);
      int y = (int)(k / ((int64_t)nf * nx));
      return ((int64_t)(y + up) * nxExt() + (x + lt)) * nf + f;
   }
};

inline Loc to_loc(const pvgpu_loc &l) {
   return Loc{l.nbatch, l.nx, l.ny, l.nf, l.halo.lt, l.halo.rt, l.halo.dn, l.halo.up};
}

inline bool loc_valid(const pvgpu_loc &l) {
   return l.nbatch > 0 && l.nx > 0 && l.ny > 0 && l.nf > 0 && l.halo.lt >= 0 && l.halo.rt >= 0 &&
          l.halo.dn >= 0 && l.halo.up >= 0;
}

__host__ __device__ inline bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

// One axis of a pre->post connection: PatchGeometry::calcPatchStartInPost
// (components/PatchGeometry.cpp:334-390), in restricted coordinates.  The start is not
// clipped; clipping it to [0, nPost) is what produces the reference's shrunken patches.
struct Axis {
   int nPre, nPost, patch, preBorder;
   __host__ __device__ int start(int idxExtPre) const {
      int r = idxExtPre - preBorder;
      if (nPre == nPost) return r - (patch - 1) / 2;
      if (nPre < nPost) {
         int t = nPost / nPre;
         return r * t - (patch - t) / 2;
      }
      int s = nPre / nPost;
      int e = (s / 2) * (patch - 1);
      // floor((r - e) / s) without the float round trip (exact for these integer sizes)
      int num = r - e;
      return num >= 0 ? num / s : -((-num + s - 1) / s);
   }
};

// PatchGeometry::verifyPatchSize (components/PatchGeometry.cpp:88-150), one axis.
__host__ __device__ inline bool axis_legal(int nPre, int nPost, int patch) {
   if (nPre > nPost) {
      int s = nPre / nPost;
      return s * nPost == nPre && is_pow2(s);
   }
   if (nPre < nPost) {
      int t = nPost / nPre;
      return t * nPre == nPost && patch % t == 0 && is_pow2(t);
   }
   return patch % 2 == 1;
}

// utils/requiredConvolveMargin.hpp
__host__ __device__ inline int required_margin(int nPre, int nPost, int patch) {
   if (nPre == nPost) return (patch - 1) / 2;
   if (nPre > nPost) return (patch - 1) * (nPre / nPost) / 2;
   return (patch / (nPost / nPre)) / 2;
}

// PatchSize::calcPostPatchSize (components/PatchSize.cpp:98-130)
__host__ __device__ inline int post_patch_size(int prePatch, int nPre, int nPost) {
   if (nPre == nPost) return prePatch;
   if (nPre > nPost) return prePatch * (nPre / nPost);
   return prePatch / (nPost / nPre);
}

}  // namespace pvgpu
