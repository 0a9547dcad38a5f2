// pvp.cu -- device side of the .pvp activity files (utils/BufferUtilsPvp.hpp, io/SparseLayerFile.cpp,
// io/LayerFile.cpp): the frame payloads are built on the device so that the host copies only what
// the file holds.
//
//   sparse frame (PVP_ACT_SPARSEVALUES_FILE_TYPE): the layer's SparseList (extended indices) as the
//     file stores it -- SparseLayerBatchGatherScatter::gather followed by SparseList::crop
//     (io/SparseLayerBatchGatherScatter.cpp:24-80, structures/SparseList.hpp:76-110): halo entries
//     dropped, indices converted to restricted, order kept;
//   dense frame (PVP_NONSPIKING_ACT_FILE_TYPE): the restricted activity [ny][nx][nf];
//   reading back: a file's sparse frame scattered into a zeroed extended activity.
// Byte work, HBM-bound.
#include "pvgpu_internal.cuh"

namespace {

constexpr int kThreads = 1024;

// One CTA per batch element walks its SparseList in tiles of 1024 entries; a block scan of the
// keep flags gives each kept entry its output slot, so the order is the list's.
__global__ void __launch_bounds__(kThreads) crop_kernel(pvgpu::Loc l, const pvgpu_entry *__restrict__ in,
                                                        const int64_t *__restrict__ numActive,
                                                        pvgpu_entry *__restrict__ out, int32_t *__restrict__ counts) {
   const int b = blockIdx.x;
   const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
   const int64_t numExt = l.numExt(), numRes = l.numRes();
   const pvgpu_entry *ib = in + (size_t)b * numExt;
   pvgpu_entry *ob = out + (size_t)b * numRes;
   const int64_t n = numActive[b] < numExt ? numActive[b] : numExt;
   const int nxExt = l.nxExt();
   __shared__ int warpTot[kThreads / 32];
   __shared__ int carry;
   if (threadIdx.x == 0) carry = 0;
   __syncthreads();
   for (int64_t base = 0; base < n; base += kThreads) {
      const int64_t i = base + threadIdx.x;
      bool keep = false;
      pvgpu_entry e{0u, 0.0f};
      if (i < n) {
         e = ib[i];
         const int64_t k = e.index;
         const int f = (int)(k % l.nf);
         const int x = (int)((k / l.nf) % nxExt) - l.lt;
         const int y = (int)(k / ((int64_t)nxExt * l.nf)) - l.up;
         keep = k < numExt && x >= 0 && x < l.nx && y >= 0 && y < l.ny;
         if (keep) e.index = (uint32_t)(f + l.nf * (x + l.nx * y));
      }
      const unsigned m = __ballot_sync(0xffffffffu, keep);
      if (lane == 0) warpTot[warp] = __popc(m);
      __syncthreads();
      if (warp == 0) {
         int v = warpTot[lane];
         int x = v;
#pragma unroll
         for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
         }
         warpTot[lane] = x - v;  // exclusive
      }
      __syncthreads();
      const int c0 = carry;
      if (keep) ob[c0 + warpTot[warp] + __popc(m & ((1u << lane) - 1u))] = e;
      __syncthreads();
      if (threadIdx.x == kThreads - 1) carry = c0 + warpTot[warp] + __popc(m);
      __syncthreads();
   }
   if (threadIdx.x == 0) counts[b] = carry;
}

__global__ void restrict_kernel(pvgpu::Loc l, const float *__restrict__ aExt, float *__restrict__ out) {
   const int64_t numRes = l.numRes(), total = numRes * l.nb;
   for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
      const int64_t b = i / numRes, k = i - b * numRes;
      out[i] = aExt[b * l.numExt() + l.kex(k)];
   }
}

__global__ void scatter_kernel(pvgpu::Loc l, const pvgpu_entry *__restrict__ in, const int32_t *__restrict__ counts,
                               float *__restrict__ aExt, int32_t *__restrict__ bad) {
   const int b = blockIdx.y;
   const int64_t numRes = l.numRes();
   const pvgpu_entry *ib = in + (size_t)b * numRes;
   const int n = counts[b];
   for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n && i < numRes;
        i += (int64_t)gridDim.x * blockDim.x) {
      const pvgpu_entry e = ib[i];
      if ((int64_t)e.index >= numRes) {
         atomicExch(bad, 1);
         continue;
      }
      aExt[(size_t)b * l.numExt() + l.kex(e.index)] = e.value;
   }
}

int grid_for(int64_t n, int threads) {
   int dev = 0, sms = 148;
   cudaGetDevice(&dev);
   cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
   const int64_t blocks = (n + threads - 1) / threads;
   const int64_t cap = (int64_t)sms * 8;
   return (int)(blocks < 1 ? 1 : blocks < cap ? blocks : cap);
}

}  // namespace

extern "C" pvgpu_status pvgpu_pvp_sparse_frames(const pvgpu_loc *loc, const pvgpu_entry *entries,
                                                const int64_t *numActive, pvgpu_entry *out, int32_t *counts,
                                                void *stream) {
   if (!loc || !entries || !numActive || !out || !counts || !pvgpu::loc_valid(*loc)) return PVGPU_ERR_BAD_ARG;
   const pvgpu::Loc l = pvgpu::to_loc(*loc);
   if (l.numExt() > 0xffffffffLL) return PVGPU_ERR_UNSUPPORTED_SHAPE;
   crop_kernel<<<l.nb, kThreads, 0, pvgpu::as_stream(stream)>>>(l, entries, numActive, out, counts);
   PVGPU_CHECK_LAUNCH("pvp_sparse_frames");
   return PVGPU_OK;
}

extern "C" pvgpu_status pvgpu_pvp_dense_frames(const pvgpu_loc *loc, const float *aExt, float *out, void *stream) {
   if (!loc || !aExt || !out || !pvgpu::loc_valid(*loc)) return PVGPU_ERR_BAD_ARG;
   const pvgpu::Loc l = pvgpu::to_loc(*loc);
   restrict_kernel<<<grid_for(l.numRes() * l.nb, 256), 256, 0, pvgpu::as_stream(stream)>>>(l, aExt, out);
   PVGPU_CHECK_LAUNCH("pvp_dense_frames");
   return PVGPU_OK;
}

extern "C" pvgpu_status pvgpu_pvp_scatter_sparse(const pvgpu_loc *loc, const pvgpu_entry *fileEntries,
                                                 const int32_t *counts, float *aExt, int32_t *badIndex,
                                                 void *stream) {
   if (!loc || !fileEntries || !counts || !aExt || !badIndex || !pvgpu::loc_valid(*loc)) return PVGPU_ERR_BAD_ARG;
   const pvgpu::Loc l = pvgpu::to_loc(*loc);
   cudaStream_t s = pvgpu::as_stream(stream);
   PVGPU_CUDA(cudaMemsetAsync(aExt, 0, sizeof(float) * (size_t)(l.numExt() * l.nb), s), "pvp_scatter memset");
   dim3 grid((unsigned)grid_for(l.numRes(), 256), (unsigned)l.nb);
   scatter_kernel<<<grid, 256, 0, s>>>(l, fileEntries, counts, aExt, badIndex);
   PVGPU_CHECK_LAUNCH("pvp_scatter_sparse");
   return PVGPU_OK;
}
