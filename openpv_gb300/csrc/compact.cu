// compact.cu -- a1: stable active-index compaction (DataStore::updateActiveIndices,
// columns/DataStore.cpp:46-66) on the device, in one pass over the activity.
//
// Each batch element's extended activity is cut into chunks of kChunk = 16384 floats (64 KB).
// Entries must come out in ascending extended index.  Per chunk:
//   * every thread holds a fixed set of units of the chunk (float4s, or single floats when the
//     images are not 16-byte aligned) at unit index k * threads + t, so a warp's units of one k
//     are one contiguous run and entries are ordered by (k, warp, lane, element-of-unit);
//   * inside a warp, the rank of a thread's unit k comes from a warp scan of per-thread counts
//     (float4 units: four 8-bit fields, one per k, scanned together in one 32-bit scan; scalar
//     units: a ballot per k);
//   * across the warps, warp 0 scans the warp totals in (k, warp) order;
//   * across chunks, a decoupled look-back (Merrill & Garland, "Single-pass Parallel Prefix Scan
//     with Decoupled Look-back", 2016): the chunk's total is published as soon as it is known,
//     then warp 0 reads the status words of up to 128 predecessors per round trip, summing
//     totals back to the nearest chunk that has published its inclusive prefix.
// Chunks are handed out by an atomic ticket in the scratch, chunk-major (ticket t = chunk
// t / nbatch of image t % nbatch), so the chunks in flight spread over every image's chain and
// each look-back finds a published prefix close by.  A chunk only waits for chunks with smaller
// tickets, whose owners are running and take their tickets in increasing order: the look-back
// always ends.  Its spin is bounded in time all the same; a chunk that gives up publishes an
// error status that propagates down the image's chain and makes the image's count -1.
//
// One CTA per chunk of 512 threads, float4 units (images 16-byte aligned) or scalar units;
// every load of the chunk is issued before any is used.  (Tried and not
// kept: a persistent kernel streaming chunks through a shared-memory ring -- its consumers
// take their chunks in order, so a chunk's total is published late and look-backs convoy
// across CTAs, 0.21 ms against 0.10 ms on 16 x 134x134x256 values; a dedicated look-back warp
// started with the loads -- its early polling cost more than it hid, 0.14 ms.)
//
// Integer/byte work, HBM-bound: one read of the activity + 8 B per entry written.
// Scratch: one 8-byte ticket word, then one 8-byte status word per chunk, zeroed before each call.
#include "pvgpu_internal.cuh"
#include "tc_ptx.cuh"

#include <algorithm>
#include <mutex>

namespace {

using pvgpu::tc::global_ns;
using pvgpu::tc::kWaitNs;

constexpr int kChunk = 16384;
constexpr uint64_t kFlagAgg = 1ull << 62, kFlagPre = 2ull << 62, kFlagErr = 3ull << 62;

__device__ __forceinline__ void st_release(uint64_t *p, uint64_t v) {
   asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint64_t ld_acquire(const uint64_t *p) {
   uint64_t v;
   asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
   return v;
}

__device__ __forceinline__ uint32_t lanemask_lt() {
   uint32_t m;
   asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
   return m;
}

// Warp 0 of a chunk's consumers: exclusive scan (in place) of the NT warp totals in tot, in
// index order (NT a multiple of 32); returns the chunk's total.
template <int NT>
__device__ __forceinline__ uint32_t scan_totals(uint32_t *tot, int lane) {
   constexpr int PER = NT / 32;
   uint32_t loc[PER], sum = 0;
#pragma unroll
   for (int i = 0; i < PER; i++) {
      loc[i] = tot[lane * PER + i];
      sum += loc[i];
   }
   uint32_t incl = sum;
#pragma unroll
   for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
   }
   uint32_t run = incl - sum;
#pragma unroll
   for (int i = 0; i < PER; i++) {
      tot[lane * PER + i] = run;
      run += loc[i];
   }
   return __shfl_sync(0xffffffffu, incl, 31);
}

// Warp 0: publishes chunk c's total, looks back over the image's statuses st[0 .. c-1] for the
// exclusive prefix, publishes the inclusive prefix; *err on a timeout or an upstream error.
__device__ __forceinline__ uint32_t look_back(uint64_t *st, int c, uint32_t total, int lane, bool *err) {
   *err = false;
   if (c == 0) {
      if (lane == 0) st_release(&st[0], kFlagPre | total);
      return 0;
   }
   if (lane == 0) st_release(&st[c], kFlagAgg | total);
   // lane l reads the statuses of chunks j - 4l .. j - 4l - 3 (128 predecessors per round trip);
   // chunks before 0 read as a published prefix of 0
   uint32_t excl = 0;
   int j = c - 1;
   uint64_t t0 = 0;
   bool timing = false;
   for (;;) {
      uint64_t sv[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
         const int idx = j - 4 * lane - q;
         sv[q] = idx >= 0 ? ld_acquire(&st[idx]) : kFlagPre;
      }
      // this lane's nearest stop (inclusive prefix or error), and whether a status up to it is
      // not ready yet
      int stopQ = 4;
#pragma unroll
      for (int q = 3; q >= 0; q--)
         if ((sv[q] >> 62) >= 2) stopQ = q;
      bool laneNotReady = false;
#pragma unroll
      for (int q = 0; q < 4; q++)
         if (q <= stopQ && (sv[q] >> 62) == 0) laneNotReady = true;
      const uint32_t stopMask = __ballot_sync(0xffffffffu, stopQ < 4);
      const int firstStop = stopMask ? __ffs(stopMask) - 1 : 31;
      const uint32_t notReady = __ballot_sync(0xffffffffu, laneNotReady);
      const uint32_t need = firstStop == 31 ? 0xffffffffu : ((2u << firstStop) - 1u);
      if (notReady & need) {
         if (!timing) {
            t0 = global_ns();
            timing = true;
         } else if (global_ns() - t0 > kWaitNs) {
            *err = true;
            break;
         }
         continue;
      }
      uint32_t part = 0;
      if (lane <= firstStop) {
#pragma unroll
         for (int q = 0; q < 4; q++)
            if (lane < firstStop || q <= stopQ) part += (uint32_t)sv[q];
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
      excl += part;
      if (stopMask) {
         const int fq = __shfl_sync(0xffffffffu, stopQ, firstStop);
         uint64_t fs = sv[0];
#pragma unroll
         for (int q = 1; q < 4; q++)
            if (q == fq) fs = sv[q];
         *err = (uint32_t)(__shfl_sync(0xffffffffu, fs, firstStop) >> 62) == 3u;
         break;
      }
      j -= 128;
   }
   if (lane == 0) st_release(&st[c], (*err ? kFlagErr : kFlagPre) | (uint32_t)(excl + total));
   return excl;
}

// ---- one CTA per chunk -------------------------------------------------------------------------
// 512 threads, two CTAs per SM: 64 KB of a chunk's float4 loads in flight per CTA (8 per
// thread), the look-back once per 64 KB.  Measured on 16 x 131x131x256 values at p = 0.01 / 0.2:
// 8192-value chunks on 128-thread CTAs (five per SM) 0.103 / 0.124 ms, on 256-thread CTAs
// 0.110 / 0.129, 4096-value chunks 0.137 / 0.157, 16384-value chunks on 256 threads 0.095 /
// 0.118 (register spills) or 0.100 / 0.119 (two per SM), 32768 on 512 threads 0.100 / 0.118,
// this shape 0.095 / 0.113.  VEC = 1: scalar units, 512 threads x 32 units, one CTA per SM.
template <int VEC>
struct Shape {
   static constexpr int kThreads = 512;
   static constexpr int kWarps = kThreads / 32;
   static constexpr int KU = kChunk / (kThreads * VEC);  // units per thread (8 float4 or 32 floats)
};

template <int VEC>
__global__ void __launch_bounds__(Shape<VEC>::kThreads, VEC == 4 ? 2 : 1)
      compact_kernel(const float *__restrict__ a, int64_t numExt, int nbatch, int nchunks,
                     uint64_t *__restrict__ scratch, pvgpu_entry *__restrict__ entries,
                     int64_t *__restrict__ numActive) {
   constexpr int kThreads = Shape<VEC>::kThreads, kWarps = Shape<VEC>::kWarps, KU = Shape<VEC>::KU;
   __shared__ uint32_t ticketSh, prefixSh;
   __shared__ uint32_t wtot[KU * kWarps];  // warp totals, then their exclusive scan
   const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
   if (tid == 0) ticketSh = (uint32_t)atomicAdd(reinterpret_cast<unsigned long long *>(scratch), 1ull);
   __syncthreads();
   const uint32_t t = ticketSh;
   const int c = (int)(t / (uint32_t)nbatch), b = (int)(t % (uint32_t)nbatch);
   const int64_t base = (int64_t)c * kChunk;
   const float *ab = a + (size_t)b * numExt;
   float v[KU * VEC];
   if constexpr (VEC == 4) {
      const float4 *a4 = reinterpret_cast<const float4 *>(ab);
#pragma unroll
      for (int k = 0; k < KU; k++) {
         const int64_t e = base + (int64_t)(k * kThreads + tid) * 4;
         float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
         if (e < numExt) q = __ldcs(a4 + e / 4);  // numExt is a multiple of 4 here
         v[4 * k] = q.x;
         v[4 * k + 1] = q.y;
         v[4 * k + 2] = q.z;
         v[4 * k + 3] = q.w;
      }
   } else {
#pragma unroll
      for (int k = 0; k < KU; k++) {
         const int64_t e = base + k * kThreads + tid;
         v[k] = e < numExt ? __ldcs(ab + e) : 0.0f;
      }
   }
   // rank of this thread's unit k among the warp's units k.  float4 units: four 8-bit fields
   // per word (a warp's field sum is <= 128, so fields never carry), one warp scan per word;
   // scalar units: a ballot per k.
   constexpr int NW = VEC == 4 ? KU / 4 : 1;
   uint32_t packed[NW], incl[NW];
   uint32_t wexs[VEC == 4 ? 1 : KU];
   if constexpr (VEC == 4) {
#pragma unroll
      for (int w = 0; w < NW; w++) packed[w] = 0u;
#pragma unroll
      for (int k = 0; k < KU; k++) {
         const uint32_t n = (v[4 * k] != 0.f) + (v[4 * k + 1] != 0.f) + (v[4 * k + 2] != 0.f) + (v[4 * k + 3] != 0.f);
         packed[k >> 2] |= n << (8 * (k & 3));
      }
#pragma unroll
      for (int w = 0; w < NW; w++) incl[w] = packed[w];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
         for (int w = 0; w < NW; w++) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl[w], o);
            if (lane >= o) incl[w] += y;
         }
      }
      if (lane == 31) {
#pragma unroll
         for (int k = 0; k < KU; k++) wtot[k * kWarps + warp] = (incl[k >> 2] >> (8 * (k & 3))) & 0xffu;
      }
   } else {
      const uint32_t lt = lanemask_lt();
#pragma unroll
      for (int k = 0; k < KU; k++) {
         const uint32_t m = __ballot_sync(0xffffffffu, v[k] != 0.f);
         wexs[k] = __popc(m & lt);
         if (lane == 0) wtot[k * kWarps + warp] = __popc(m);
      }
   }
   __syncthreads();
   if (warp == 0) {
      const uint32_t total = scan_totals<KU * kWarps>(wtot, lane);
      bool err;
      const uint32_t excl = look_back(scratch + 1 + (size_t)b * nchunks, c, total, lane, &err);
      if (lane == 0) {
         prefixSh = excl;
         if (c == nchunks - 1) numActive[b] = err ? (int64_t)-1 : (int64_t)(excl + total);
      }
   }
   __syncthreads();
   const uint32_t prefix = prefixSh;
   const uint32_t cap = (uint32_t)numExt;  // ranks stay below it; the test only guards the store
   uint2 *eb = reinterpret_cast<uint2 *>(entries + (size_t)b * numExt);
#pragma unroll
   for (int k = 0; k < KU; k++) {
      if constexpr (VEC == 4) {
         uint32_t r = prefix + wtot[k * kWarps + warp] + (((incl[k >> 2] - packed[k >> 2]) >> (8 * (k & 3))) & 0xffu);
         const uint32_t e = (uint32_t)base + 4u * (uint32_t)(k * kThreads + tid);
#pragma unroll
         for (int q = 0; q < 4; q++) {
            if (v[4 * k + q] != 0.f) {
               if (r < cap) eb[r] = make_uint2(e + q, __float_as_uint(v[4 * k + q]));
               r++;
            }
         }
      } else {
         const uint32_t r = prefix + wtot[k * kWarps + warp] + wexs[k];
         const int64_t e = base + k * kThreads + tid;
         if (v[k] != 0.f && r < cap) eb[r] = make_uint2((uint32_t)e, __float_as_uint(v[k]));
      }
   }
}

int64_t chunks_of(int64_t numExt) { return (numExt + kChunk - 1) / kChunk; }

pvgpu_status check_args(const float *aExt, int nbatch, int64_t numExt, const pvgpu_entry *entries,
                        const int64_t *numActive) {
   if (!aExt || !entries || !numActive || nbatch <= 0 || numExt <= 0 || numExt > 0xffffffffLL) return PVGPU_ERR_BAD_ARG;
   if (reinterpret_cast<uintptr_t>(entries) % 8 != 0 || reinterpret_cast<uintptr_t>(aExt) % 4 != 0)
      return pvgpu::record_message(PVGPU_ERR_BAD_ARG, "compact_active: entries must be 8-byte aligned, activity 4-byte");
   if ((int64_t)nbatch * chunks_of(numExt) > 0x7fffffffLL) return PVGPU_ERR_UNSUPPORTED_SHAPE;
   return PVGPU_OK;
}

// Zeroes the ticket and the chunk statuses, then runs the one-pass kernel.
pvgpu_status launch(const float *aExt, int nbatch, int64_t numExt, pvgpu_entry *entries, int64_t *numActive,
                    uint64_t *scratch, cudaStream_t s, const char *where) {
   const int64_t nchunks = chunks_of(numExt);
   const int64_t total = (int64_t)nbatch * nchunks;
   const size_t words = 1 + (size_t)total;
   cudaError_t e = cudaMemsetAsync(scratch, 0, words * sizeof(uint64_t), s);
   if (e != cudaSuccess) return pvgpu::record_cuda_error(e, where);
   const bool vec = reinterpret_cast<uintptr_t>(aExt) % 16 == 0 && numExt % 4 == 0;
   if (vec)
      compact_kernel<4><<<(unsigned)total, Shape<4>::kThreads, 0, s>>>(aExt, numExt, nbatch, (int)nchunks, scratch,
                                                                       entries, numActive);
   else
      compact_kernel<1><<<(unsigned)total, Shape<1>::kThreads, 0, s>>>(aExt, numExt, nbatch, (int)nchunks, scratch,
                                                                       entries, numActive);
   PVGPU_CHECK_LAUNCH(where);
   return PVGPU_OK;
}

}  // namespace

extern "C" size_t pvgpu_compact_scratch_bytes(int nbatch, int64_t numExt) {
   if (nbatch <= 0 || numExt <= 0) return 0;
   return (1 + (size_t)nbatch * (size_t)chunks_of(numExt)) * sizeof(uint64_t);
}

extern "C" pvgpu_status pvgpu_compact_active(const float *aExt, int nbatch, int64_t numExt, pvgpu_entry *entries,
                                             int64_t *numActive, void *scratch, size_t scratchBytes, void *stream) {
   pvgpu_status st = check_args(aExt, nbatch, numExt, entries, numActive);
   if (st != PVGPU_OK) return st;
   if (!scratch || scratchBytes < pvgpu_compact_scratch_bytes(nbatch, numExt) ||
       reinterpret_cast<uintptr_t>(scratch) % 8 != 0)
      return PVGPU_ERR_BAD_ARG;
   return launch(aExt, nbatch, numExt, entries, numActive, static_cast<uint64_t *>(scratch), pvgpu::as_stream(stream),
                 "compact_active");
}

// ---------------------------------------------------------------------------------------------
// Compaction without any device allocation.
//
// Some callers cannot hand this library a scratch buffer and must not make it allocate one:
// latency-critical loops that cannot afford the implicit device synchronisation that
// cudaMalloc / cudaFree may cause, and hosts whose device memory is entirely owned by their own
// pool allocator.  For them the ticket and the chunk statuses live in a fixed array in this
// library's device image: kNoAllocWords 8-byte words, i.e. nbatch * ceil(numExt / 16384) <=
// 131071 chunks (up to about 2^30 activity values per call).  The array is loaded with the
// library, once per device, and held until the process exits.
// ---------------------------------------------------------------------------------------------
namespace {

constexpr int64_t kNoAllocWords = 1 << 17;  // 131072 x 8 bytes = 1 MiB per device
constexpr int64_t kNoAllocMaxChunks = kNoAllocWords - 1;

static __device__ __align__(256) uint64_t g_compact_noalloc_scratch[kNoAllocWords];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
void *g_noalloc_addr[kMaxDevices] = {};

// Device address of g_compact_noalloc_scratch on the current device.  The host-side symbol is
// only a stand-in: a kernel handed its host address would read the wrong memory, so the
// address is looked up with the device current, checked, and cached per device ordinal.  The
// cache assumes the device's context lives as long as the process: after cudaDeviceReset the
// cached address is stale.
pvgpu_status noalloc_scratch(uint64_t **out) {
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
   *out = static_cast<uint64_t *>(g_noalloc_addr[dev]);
   return PVGPU_OK;
}

}  // namespace

extern "C" pvgpu_status pvgpu_compact_active_noalloc(const float *aExt, int nbatch, int64_t numExt,
                                                     pvgpu_entry *entries, int64_t *numActive, void *stream) {
   pvgpu_status st = check_args(aExt, nbatch, numExt, entries, numActive);
   if (st != PVGPU_OK) return st;
   if ((int64_t)nbatch * chunks_of(numExt) > kNoAllocMaxChunks)
      return pvgpu::record_message(PVGPU_ERR_BAD_ARG,
                                   "compact_active_noalloc: nbatch * ceil(numExt / 16384) exceeds the fixed scratch "
                                   "of 131071 chunk statuses; use pvgpu_compact_active with caller scratch");
   uint64_t *scratch = nullptr;
   st = noalloc_scratch(&scratch);
   if (st != PVGPU_OK) return st;
   // The ticket and the statuses left by the previous call are cleared (cudaMemsetAsync on the
   // stream, no allocation) before the kernel reads them.
   return launch(aExt, nbatch, numExt, entries, numActive, scratch, pvgpu::as_stream(stream),
                 "compact_active_noalloc");
}
