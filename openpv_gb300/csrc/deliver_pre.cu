// deliver_pre.cu -- a4: presynaptic-perspective delivery without atomics.
//
// The reference scatters a*w into GSyn from every active presynaptic neuron
// (PresynapticPerspectiveConvolveDelivery.cpp:61-192 on the CPU; one thread per
// (neuron, weight) doing a global atomicAdd in CudaRecvPre.cu:10-88 on the GPU).  Here the
// output owns the work instead: a CTA owns a tile of GSyn (8 post rows x TX columns x FT
// features), each warp one post row, each lane a fixed set of (column, feature) elements
// held in registers.  For every patch row ky the warp finds the presynaptic rows whose
// patch row ky lands on its post row, and, inside those rows, the contiguous index range
// of presynaptic neurons whose patch overlaps the tile: a binary search in the ascending
// SparseList (or a direct walk of the dense activity).  Every GSyn element therefore gets
// its contributions in the reference's order -- row of the shrunken patch ascending, then
// presynaptic index ascending -- with no atomics and no second pass.  In REFERENCE_ORDER mode products
// and sums are rounded separately (no FMA), which makes the result bit-identical to the
// reference CPU loop run on one thread.
//
// Geometry is arithmetic (PatchGeometry::calcPatchStartInPost restated in Axis::start);
// shrunken border patches fall out of the tile bounds, as in PatchGeometry::calcPatchData.
#include "pvgpu_internal.cuh"

namespace {

using pvgpu::Axis;
using pvgpu::Loc;

constexpr int kWarps = 8;
constexpr int kMaxElemsPerRow = 512;

struct PreGeom {
   Loc pre, post;
   Axis ax, ay;
   int nxp, nyp, nfp;
   int nkx, nky, nkf;
   int patchSize;
   int TX, FT;  // tile columns, tile features
   float dtf;
};

// Weights::calcDataIndexFromPatchIndex (components/Weights.cpp:208-232)
__device__ __forceinline__ int kernel_index(const PreGeom &g, int xe, int ye, int f) {
   int x = (xe - g.pre.lt) % g.nkx;
   if (x < 0) x += g.nkx;
   int y = (ye - g.pre.up) % g.nky;
   if (y < 0) y += g.nky;
   return (y * g.nkx + x) * g.nkf + f;
}

// first i in [0, n) with ax.start(i) >= v (start is nondecreasing in i)
__device__ __forceinline__ int first_start_ge(const Axis &ax, int n, int v) {
   int lo = 0, hi = n;
   while (lo < hi) {
      int mid = (lo + hi) >> 1;
      if (ax.start(mid) >= v) hi = mid;
      else lo = mid + 1;
   }
   return lo;
}

__device__ __forceinline__ int64_t lower_bound_entries(const pvgpu_entry *e, int64_t n, uint32_t key) {
   int64_t lo = 0, hi = n;
   while (lo < hi) {
      int64_t mid = (lo + hi) >> 1;
      if (e[mid].index < key) lo = mid + 1;
      else hi = mid;
   }
   return lo;
}

template <bool EXACT>
__device__ __forceinline__ float madd(float acc, float a, float w) {
   if (EXACT) return __fadd_rn(acc, __fmul_rn(a, w));
   return fmaf(a, w, acc);
}

template <bool SPARSE, bool EXACT, int EPL>
__global__ void __launch_bounds__(kWarps * 32) deliver_pre_kernel(PreGeom g, const pvgpu_entry *__restrict__ entries,
                                                                  const int64_t *__restrict__ numActive,
                                                                  const float *__restrict__ aExt,
                                                                  const float *__restrict__ W,
                                                                  float *__restrict__ gsyn) {
   const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
   const int nFT = (g.nfp + g.FT - 1) / g.FT;
   const int X0 = (blockIdx.x / nFT) * g.TX;
   const int F0 = (blockIdx.x % nFT) * g.FT;
   const int py = blockIdx.y * kWarps + warp;
   const int b = blockIdx.z;
   if (py >= g.post.ny) return;

   const int ftile = min(g.FT, g.nfp - F0);
   const int tx = min(g.TX, g.post.nx - X0);
   const int elems = tx * ftile;
   float *grow = gsyn + (size_t)b * g.post.numRes() + ((size_t)py * g.post.nx) * g.nfp;

   float acc[EPL];
   int pxo[EPL], fpo[EPL];
#pragma unroll
   for (int i = 0; i < EPL; i++) {
      int e = lane + 32 * i;
      pxo[i] = e < elems ? e / ftile : -1000000;  // tile-relative column; sentinel fails every range check
      fpo[i] = e < elems ? F0 + e % ftile : 0;
      acc[i] = e < elems ? grow[(size_t)(X0 + pxo[i]) * g.nfp + fpo[i]] : 0.0f;
   }

   const int nxExt = g.pre.nxExt(), nyExt = g.pre.nyExt(), nf = g.pre.nf;
   const pvgpu_entry *eb = SPARSE ? entries + (size_t)b * g.pre.numExt() : nullptr;
   const int64_t nAct = SPARSE ? numActive[b] : 0;
   const float *ab = SPARSE ? nullptr : aExt + (size_t)b * g.pre.numExt();
   const int rowStride = g.nxp * g.nfp;

   // presynaptic columns whose patch overlaps [X0, X0 + tx)
   const int xlo = first_start_ge(g.ax, nxExt, X0 - g.nxp + 1);
   const int xhi = first_start_ge(g.ax, nxExt, X0 + tx) - 1;
   if (xlo <= xhi) {
   // The reference loops over rows y of the *shrunken* patch.  For post row py, patch row
   // ky lands at shrunken row min(ky, py): rows ky < py come one by one in ascending order,
   // and all rows ky >= py (patches clipped at the top border) share shrunken row py, where
   // they are ordered by presynaptic index, i.e. by descending ky.
   const int nAsc = min(py, g.nyp);
   for (int it = 0; it < g.nyp; it++) {
      const int ky = it < nAsc ? it : g.nyp - 1 - (it - nAsc);
      const int want = py - ky;
      for (int ye = first_start_ge(g.ay, nyExt, want); ye < nyExt && g.ay.start(ye) == want; ye++) {
         const uint32_t kLo = (uint32_t)(((int64_t)ye * nxExt + xlo) * nf);
         const uint32_t kHi = (uint32_t)(((int64_t)ye * nxExt + xhi) * nf + nf - 1);
         const float *wky = W + (size_t)ky * rowStride;
         int64_t i0, i1;
         if (SPARSE) {
            i0 = lower_bound_entries(eb, nAct, kLo);
            i1 = lower_bound_entries(eb, nAct, kHi + 1);
         } else {
            i0 = kLo;
            i1 = (int64_t)kHi + 1;
         }
         for (int64_t base = i0; base < i1; base += 32) {
            // one candidate per lane, then broadcast in order
            uint32_t myIdx = 0;
            float myVal = 0.0f;
            if (base + lane < i1) {
               if (SPARSE) {
                  pvgpu_entry en = eb[base + lane];
                  myIdx = en.index;
                  myVal = en.value;
               } else {
                  myIdx = (uint32_t)(base + lane);
                  myVal = ab[base + lane];
               }
            }
            const int cnt = (int)min((int64_t)32, i1 - base);
            for (int j = 0; j < cnt; j++) {
               const float a = __shfl_sync(0xffffffffu, myVal, j);
               if (a == 0.0f) continue;  // reference skips zeros (dense and sparse branches)
               const uint32_t k = __shfl_sync(0xffffffffu, myIdx, j);
               const int f = (int)(k % nf);
               const int xe = (int)((k / nf) % nxExt);
               const int sx = g.ax.start(xe) - X0;
               const float av = EXACT ? __fmul_rn(a, g.dtf) : a * g.dtf;
               const float *wr = wky + (size_t)kernel_index(g, xe, ye, f) * g.patchSize;
#pragma unroll
               for (int i = 0; i < EPL; i++) {
                  const int kx = pxo[i] - sx;
                  if (kx >= 0 && kx < g.nxp) acc[i] = madd<EXACT>(acc[i], av, __ldg(wr + kx * g.nfp + fpo[i]));
               }
            }
         }
      }
   }
   }  // xlo <= xhi
#pragma unroll
   for (int i = 0; i < EPL; i++) {
      int e = lane + 32 * i;
      if (e < elems) grow[(size_t)(X0 + pxo[i]) * g.nfp + fpo[i]] = acc[i];
   }
}

template <bool SPARSE, bool EXACT>
pvgpu_status launch(const PreGeom &g, int epl, dim3 grid, cudaStream_t s, const pvgpu_entry *entries,
                    const int64_t *numActive, const float *aExt, const float *W, float *gsyn) {
   switch (epl) {
#define PVGPU_CASE(N) \
   case N: deliver_pre_kernel<SPARSE, EXACT, N><<<grid, kWarps * 32, 0, s>>>(g, entries, numActive, aExt, W, gsyn); break;
      PVGPU_CASE(1)
      PVGPU_CASE(2)
      PVGPU_CASE(4)
      PVGPU_CASE(8)
      PVGPU_CASE(16)
#undef PVGPU_CASE
      default: return PVGPU_ERR_UNSUPPORTED_SHAPE;
   }
   PVGPU_CHECK_LAUNCH("deliver_pre");
   return PVGPU_OK;
}

}  // namespace

extern "C" pvgpu_status pvgpu_deliver_pre(const pvgpu_conn_desc *conn, const pvgpu_entry *entries,
                                          const int64_t *numActive, const float *aExt, const float *weights,
                                          float *gsyn, int mode, void *stream) {
   if (!conn || !weights || !gsyn) return PVGPU_ERR_BAD_ARG;
   if (!pvgpu::loc_valid(conn->pre) || !pvgpu::loc_valid(conn->post)) return PVGPU_ERR_BAD_ARG;
   if (conn->pre.nbatch != conn->post.nbatch || conn->nxp <= 0 || conn->nyp <= 0) return PVGPU_ERR_BAD_ARG;
   if (entries ? !numActive : !aExt) return PVGPU_ERR_BAD_ARG;
   const pvgpu_loc &pre = conn->pre, &post = conn->post;
   if (!pvgpu::axis_legal(pre.nx, post.nx, conn->nxp) || !pvgpu::axis_legal(pre.ny, post.ny, conn->nyp))
      return PVGPU_ERR_ILLEGAL_GEOMETRY;
   if (pre.halo.lt != pre.halo.rt || pre.halo.dn != pre.halo.up) return PVGPU_ERR_UNSUPPORTED_SHAPE;
   PreGeom g;
   g.pre = pvgpu::to_loc(pre);
   g.post = pvgpu::to_loc(post);
   if (g.pre.numExt() > 0xffffffffLL) return PVGPU_ERR_UNSUPPORTED_SHAPE;
   g.ax = Axis{pre.nx, post.nx, conn->nxp, pre.halo.lt};
   g.ay = Axis{pre.ny, post.ny, conn->nyp, pre.halo.dn};
   g.nxp = conn->nxp;
   g.nyp = conn->nyp;
   g.nfp = post.nf;
   g.nkx = pre.nx > post.nx ? pre.nx / post.nx : 1;
   g.nky = pre.ny > post.ny ? pre.ny / post.ny : 1;
   g.nkf = pre.nf;
   g.patchSize = g.nxp * g.nyp * g.nfp;
   g.dtf = conn->dt_factor;
   g.FT = g.nfp < kMaxElemsPerRow ? g.nfp : kMaxElemsPerRow;
   g.TX = kMaxElemsPerRow / g.FT;
   if (g.TX > post.nx) g.TX = post.nx;
   int elems = g.TX * g.FT;
   int epl = (elems + 31) / 32;
   int p2 = 1;
   while (p2 < epl) p2 <<= 1;
   int nFT = (g.nfp + g.FT - 1) / g.FT;
   int64_t gx = (int64_t)((post.nx + g.TX - 1) / g.TX) * nFT;
   int gy = (post.ny + kWarps - 1) / kWarps;
   if (gx > 0x7fffffff || gy > 65535 || pre.nbatch > 65535) return PVGPU_ERR_UNSUPPORTED_SHAPE;
   dim3 grid((unsigned)gx, gy, pre.nbatch);
   cudaStream_t s = pvgpu::as_stream(stream);
   bool exact = mode == PVGPU_DELIVER_REFERENCE_ORDER;
   if (entries)
      return exact ? launch<true, true>(g, p2, grid, s, entries, numActive, nullptr, weights, gsyn)
                   : launch<true, false>(g, p2, grid, s, entries, numActive, nullptr, weights, gsyn);
   return exact ? launch<false, true>(g, p2, grid, s, nullptr, nullptr, aExt, weights, gsyn)
                : launch<false, false>(g, p2, grid, s, nullptr, nullptr, aExt, weights, gsyn);
}
