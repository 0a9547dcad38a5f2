// tmap.cuh -- host helper: encode TMA tensor maps through the driver entry point
// (no link-time dependency on libcuda).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace pvgpu {

using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

inline EncodeTiledFn encode_tiled_fn() {
   static EncodeTiledFn fn = nullptr;
   if (!fn) {
      void *p = nullptr;
      cudaDriverEntryPointQueryResult q;
      if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
          q == cudaDriverEntryPointSuccess)
         fn = reinterpret_cast<EncodeTiledFn>(p);
   }
   return fn;
}

// 2-D row-major BF16 matrix [rows][cols] (cols contiguous, row pitch in elements), box
// boxRows x 64 columns, 128-byte swizzle: the K-major SW128 operand layout of tc_ptx.cuh.
inline bool make_tmap_bf16_sw128(CUtensorMap *map, const void *base, uint64_t rows, uint64_t cols, uint64_t pitch,
                                 uint32_t boxRows) {
   EncodeTiledFn enc = encode_tiled_fn();
   if (!enc) return false;
   if ((reinterpret_cast<uintptr_t>(base) & 15) || ((pitch * 2) & 15) || boxRows == 0 || boxRows > 256) return false;
   cuuint64_t dims[2] = {cols, rows};
   cuuint64_t strides[1] = {pitch * 2};
   cuuint32_t box[2] = {64, boxRows};
   cuuint32_t estr[2] = {1, 1};
   CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
   return r == CUDA_SUCCESS;
}

}  // namespace pvgpu
