// compact.cu -- a1: stable active-index compaction (DataStore::updateActiveIndices,
// columns/DataStore.cpp:46-66) on the device.
//
// Layout: each batch element's extended activity is cut into chunks of kChunk floats.
// Pass 1 counts nonzeros per chunk, pass 2 scans the chunk counts of each batch element
// (and writes numActive), pass 3 re-reads each chunk and writes {index, value} entries at
// the chunk's offset.  Inside a chunk, 256 threads take 256 consecutive elements per
// iteration (coalesced loads); a warp ballot plus a block scan of the 8 warp counts gives
// every nonzero its rank, so entries come out in ascending index exactly as the host loop
// produces them.  Integer/byte work: HBM-bound, 2 reads of the activity + 8 B per entry.
#include "pvgpu_internal.cuh"

#include <mutex>

namespace {

constexpr int kThreads = 256;
constexpr int kIters = 16;
constexpr int kChunk = kThreads * kIters;

__global__ void __launch_bounds__(kThreads) count_kernel(const float *__restrict__ a, int64_t numExt, int nchunks,
                                                         uint32_t *__restrict__ counts) {
   const int c = blockIdx.x, b = blockIdx.y;
   const float *ab = a + (size_t)b * numExt;
   int64_t base = (int64_t)c * kChunk;
   int cnt = 0;
#pragma unroll 4
   for (int i = 0; i < kIters; i++) {
      int64_t e = base + i * kThreads + threadIdx.x;
      bool nz = e < numExt && ab[e] != 0.0f;
      cnt += __popc(__ballot_sync(0xffffffffu, nz));
   }
   __shared__ int wsum[kThreads / 32];
   if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = cnt;
   __syncthreads();
   if (threadIdx.x == 0) {
      int t = 0;
      for (int w = 0; w < kThreads / 32; w++) t += wsum[w];
      counts[(size_t)b * nchunks + c] = (uint32_t)t;
   }
}

// One block per batch element: exclusive scan of the chunk counts, in place.
__global__ void __launch_bounds__(1024) scan_kernel(uint32_t *__restrict__ counts, int nchunks,
                                                    int64_t *__restrict__ numActive) {
   const int b = blockIdx.x;
   uint32_t *cb = counts + (size_t)b * nchunks;
   __shared__ uint32_t warpTot[32];
   __shared__ uint32_t carry;
   if (threadIdx.x == 0) carry = 0;
   __syncthreads();
   const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
   for (int base = 0; base < nchunks; base += 1024) {
      int i = base + threadIdx.x;
      uint32_t v = i < nchunks ? cb[i] : 0u;
      uint32_t x = v;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
         uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
         if (lane >= o) x += y;
      }
      if (lane == 31) warpTot[warp] = x;
      __syncthreads();
      if (warp == 0) {
         uint32_t w = warpTot[lane];
         uint32_t s = w;
#pragma unroll
         for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
         }
         warpTot[lane] = s - w;  // exclusive prefix of warp totals
      }
      __syncthreads();
      uint32_t excl = carry + warpTot[warp] + (x - v);
      if (i < nchunks) cb[i] = excl;
      __syncthreads();
      if (threadIdx.x == 1023) carry = excl + v;
      __syncthreads();
   }
   if (threadIdx.x == 0) numActive[b] = (int64_t)carry;
}

__global__ void __launch_bounds__(kThreads) write_kernel(const float *__restrict__ a, int64_t numExt, int nchunks,
                                                         const uint32_t *__restrict__ offsets,
                                                         pvgpu_entry *__restrict__ entries) {
   const int c = blockIdx.x, b = blockIdx.y;
   const float *ab = a + (size_t)b * numExt;
   pvgpu_entry *eb = entries + (size_t)b * numExt;
   const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
   __shared__ uint32_t wpre[kThreads / 32];
   __shared__ uint32_t wtot[kThreads / 32];
   uint32_t running = offsets[(size_t)b * nchunks + c];
   int64_t base = (int64_t)c * kChunk;
   for (int i = 0; i < kIters; i++) {
      int64_t e = base + i * kThreads + threadIdx.x;
      float v = e < numExt ? ab[e] : 0.0f;
      bool nz = v != 0.0f;
      uint32_t m = __ballot_sync(0xffffffffu, nz);
      if (lane == 0) wtot[warp] = __popc(m);
      __syncthreads();
      if (threadIdx.x == 0) {
         uint32_t s = 0;
         for (int w = 0; w < kThreads / 32; w++) {
            wpre[w] = s;
            s += wtot[w];
         }
      }
      __syncthreads();
      if (nz) {
         uint32_t r = running + wpre[warp] + __popc(m & ((1u << lane) - 1u));
         pvgpu_entry en;
         en.index = (uint32_t)e;
         en.value = v;
         eb[r] = en;
      }
      running += wpre[kThreads / 32 - 1] + wtot[kThreads / 32 - 1];
      __syncthreads();
   }
}

}  // namespace

extern "C" size_t pvgpu_compact_scratch_bytes(int nbatch, int64_t numExt) {
   if (nbatch <= 0 || numExt <= 0) return 0;
   int64_t nchunks = (numExt + kChunk - 1) / kChunk;
   return (size_t)nbatch * (size_t)nchunks * sizeof(uint32_t);
}

extern "C" pvgpu_status pvgpu_compact_active(const float *aExt, int nbatch, int64_t numExt, pvgpu_entry *entries,
                                             int64_t *numActive, void *scratch, size_t scratchBytes, void *stream) {
   if (!aExt || !entries || !numActive || nbatch <= 0 || numExt <= 0 || numExt > 0xffffffffLL) return PVGPU_ERR_BAD_ARG;
   size_t need = pvgpu_compact_scratch_bytes(nbatch, numExt);
   if (!scratch || scratchBytes < need) return PVGPU_ERR_BAD_ARG;
   int nchunks = (int)((numExt + kChunk - 1) / kChunk);
   if (nbatch > 65535) return PVGPU_ERR_UNSUPPORTED_SHAPE;
   cudaStream_t s = pvgpu::as_stream(stream);
   uint32_t *counts = static_cast<uint32_t *>(scratch);
   dim3 grid(nchunks, nbatch);
   count_kernel<<<grid, kThreads, 0, s>>>(aExt, numExt, nchunks, counts);
   PVGPU_CHECK_LAUNCH("compact count");
   scan_kernel<<<nbatch, 1024, 0, s>>>(counts, nchunks, numActive);
   PVGPU_CHECK_LAUNCH("compact scan");
   write_kernel<<<grid, kThreads, 0, s>>>(aExt, numExt, nchunks, counts, entries);
   PVGPU_CHECK_LAUNCH("compact write");
   return PVGPU_OK;
}

// ---------------------------------------------------------------------------------------------
// Compaction without any device allocation.
//
// Some callers cannot hand this library a scratch buffer and must not make it allocate one:
// code that runs inside a host function enqueued on a stream (CUDA API calls that allocate are
// not allowed there), latency-critical loops that cannot afford the implicit device
// synchronisation cudaMalloc/cudaFree may cause, and hosts whose device memory is entirely
// owned by their own pool allocator.  For them the per-chunk counts live in a fixed array in
// this library's device image, sized for kNoAllocMaxChunks chunks in total
// (nbatch * ceil(numExt / 4096) <= 262144, i.e. up to 2^30 activity values per call).
// The array is loaded with the library, once per device, and held until the process exits.
// ---------------------------------------------------------------------------------------------
namespace {

constexpr int64_t kNoAllocMaxChunks = 1 << 18;  // 262144 x 4 bytes = 1 MiB per device

static __device__ __align__(256) uint32_t g_compact_noalloc_scratch[kNoAllocMaxChunks];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
void *g_noalloc_addr[kMaxDevices] = {};

// Device address of g_compact_noalloc_scratch on the current device.  The host-side symbol is
// only a stand-in: a kernel handed its host address would read the wrong memory, so the
// address is looked up with the device current, checked, and cached per device.
pvgpu_status noalloc_scratch(uint32_t **out) {
   int dev = 0;
   cudaError_t e = cudaGetDevice(&dev);
   if (e != cudaSuccess) return pvgpu::record_cuda_error(e, "compact_active_noalloc: cudaGetDevice");
   if (dev < 0 || dev >= kMaxDevices)
      return pvgpu::record_message(PVGPU_ERR_UNSUPPORTED_SHAPE, "compact_active_noalloc: device ordinal out of range");
   std::lock_guard<std::mutex> lock(g_noalloc_mutex);
   if (!g_noalloc_addr[dev]) {
      void *p = nullptr;
      e = cudaGetSymbolAddress(&p, g_compact_noalloc_scratch);
      if (e != cudaSuccess || !p) return pvgpu::record_cuda_error(e, "compact_active_noalloc: cudaGetSymbolAddress");
      g_noalloc_addr[dev] = p;
   }
   *out = static_cast<uint32_t *>(g_noalloc_addr[dev]);
   return PVGPU_OK;
}

}  // namespace

extern "C" pvgpu_status pvgpu_compact_active_noalloc(const float *aExt, int nbatch, int64_t numExt,
                                                     pvgpu_entry *entries, int64_t *numActive, void *stream) {
   if (!aExt || !entries || !numActive || nbatch <= 0 || numExt <= 0 || numExt > 0xffffffffLL) return PVGPU_ERR_BAD_ARG;
   if (nbatch > 65535) return PVGPU_ERR_UNSUPPORTED_SHAPE;
   const int64_t nchunks = (numExt + kChunk - 1) / kChunk;
   if ((int64_t)nbatch * nchunks > kNoAllocMaxChunks)
      return pvgpu::record_message(PVGPU_ERR_BAD_ARG,
                                   "compact_active_noalloc: nbatch * ceil(numExt / 4096) exceeds the fixed scratch "
                                   "of 262144 chunk counts; use pvgpu_compact_active with caller scratch");
   uint32_t *counts = nullptr;
   pvgpu_status st = noalloc_scratch(&counts);
   if (st != PVGPU_OK) return st;
   // Every chunk count the kernels read is written earlier in the same call, so nothing has to
   // be cleared between calls.
   cudaStream_t s = pvgpu::as_stream(stream);
   dim3 grid((unsigned)nchunks, nbatch);
   count_kernel<<<grid, kThreads, 0, s>>>(aExt, numExt, (int)nchunks, counts);
   PVGPU_CHECK_LAUNCH("compact_active_noalloc count");
   scan_kernel<<<nbatch, 1024, 0, s>>>(counts, (int)nchunks, numActive);
   PVGPU_CHECK_LAUNCH("compact_active_noalloc scan");
   write_kernel<<<grid, kThreads, 0, s>>>(aExt, numExt, (int)nchunks, counts, entries);
   PVGPU_CHECK_LAUNCH("compact_active_noalloc write");
   return PVGPU_OK;
}
