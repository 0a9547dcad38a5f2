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

// -------------------------------------------------------------------------------------------
// FAST mode, one-to-one connections (pre and post of the same size): row-sliding kernel.
//
// A CTA owns 8 post columns (one per warp) x RS post rows x all nfp features (lane = FPL
// consecutive features).  It walks the presynaptic extended rows that reach its rows in
// ascending order -- the SparseList order -- and each warp keeps one register accumulator per
// patch row in a sliding window: presynaptic row ye adds its patch row ky to post row
// ye - Hy + ky, held in acc[ky]; once row ye is done post row ye - Hy (acc[0]) has all its
// contributions and is added into GSyn (one read-modify-write per output, no atomics), and the
// window shifts by one row (NYP x FPL register moves, so every index stays a compile-time
// constant without unrolling the row loop -- an unrolled loop outgrows the instruction cache at
// 11 and 13 patch rows).  Each active entry is read and
// decoded once per warp and feeds NYP x FPL FMAs per lane; its weights W[f][ky][kx][*] come
// through the read-only path (one coalesced 32*FPL-float row per ky).  The entry range of a
// row inside the CTA's column window comes from a binary search per row, done in parallel by
// the CTA's threads up front.  Order per output: presynaptic rows ascending, entries ascending
// -- deterministic, not the reference's (that is what REFERENCE_ORDER mode is for).
// -------------------------------------------------------------------------------------------
constexpr int kRowsRS = 32;      // post rows per CTA
constexpr int kRowsMax = 64;     // presynaptic rows a CTA may visit (RS + NYP - 1)

template <int FPL>
struct VecF;
template <>
struct VecF<1> {
   using T = float;
   __device__ static void ld(const float *p, float *v) { v[0] = __ldg(p); }
   __device__ static void rmw(float *p, const float *v) { p[0] += v[0]; }
};
template <>
struct VecF<2> {
   __device__ static void ld(const float *p, float *v) {
      const float2 t = __ldg(reinterpret_cast<const float2 *>(p));
      v[0] = t.x;
      v[1] = t.y;
   }
   __device__ static void rmw(float *p, const float *v) {
      float2 t = *reinterpret_cast<float2 *>(p);
      t.x += v[0];
      t.y += v[1];
      *reinterpret_cast<float2 *>(p) = t;
   }
};
template <>
struct VecF<4> {
   __device__ static void ld(const float *p, float *v) {
      const float4 t = __ldg(reinterpret_cast<const float4 *>(p));
      v[0] = t.x;
      v[1] = t.y;
      v[2] = t.z;
      v[3] = t.w;
   }
   __device__ static void rmw(float *p, const float *v) {
      float4 t = *reinterpret_cast<float4 *>(p);
      t.x += v[0];
      t.y += v[1];
      t.z += v[2];
      t.w += v[3];
      *reinterpret_cast<float4 *>(p) = t;
   }
};

// acc[q] += a * w[q] for the lane's FPL features: pairs of features by the packed FP32 FMA (one
// instruction, each element rounded once, as fmaf), a single feature by fmaf
template <int FPL>
__device__ __forceinline__ void fma_row(float *acc, float a, const float *w) {
   if constexpr (FPL % 2 == 0) {
      const float2 a2 = make_float2(a, a);
#pragma unroll
      for (int q = 0; q < FPL; q += 2) {
         const float2 r = __ffma2_rn(a2, make_float2(w[q], w[q + 1]), make_float2(acc[q], acc[q + 1]));
         acc[q] = r.x;
         acc[q + 1] = r.y;
      }
   } else {
#pragma unroll
      for (int q = 0; q < FPL; q++) acc[q] = fmaf(a, w[q], acc[q]);
   }
}

// More than 16 accumulators per lane (NYP x FPL) do not fit the 64 registers of four CTAs per SM
// next to the entry pipeline; those instantiations take two CTAs per SM (128 registers) instead.
template <int FPL, int NYP, bool SPARSE>
__global__ void __launch_bounds__(kWarps * 32, (FPL * NYP > 16) ? 2 : 4) deliver_pre_rows_kernel(PreGeom g, const pvgpu_entry *__restrict__ entries,
                                                                       const int64_t *__restrict__ numActive,
                                                                       const float *__restrict__ aExt,
                                                                       const float *__restrict__ W,
                                                                       float *__restrict__ gsyn) {
   __shared__ int64_t rowLo[kRowsMax], rowHi[kRowsMax];
   const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
   const int X0 = blockIdx.x * kWarps, X = X0 + warp;
   const int P0 = blockIdx.y * kRowsRS, P1 = min(P0 + kRowsRS, g.post.ny);
   const int b = blockIdx.z;
   const int nxExt = g.pre.nxExt(), nyExt = g.pre.nyExt(), nf = g.pre.nf;
   // one-to-one: patch start = index - H on both axes
   const int Hy = -g.ay.start(0), Hx = -g.ax.start(0);
   // presynaptic rows reaching post rows [P0, P1) and the columns reaching [X0, X0 + 8)
   const int yeLo = max(0, P0 + Hy - NYP + 1), yeHi = min(nyExt - 1, P1 - 1 + Hy);
   const int xlo = max(0, X0 + Hx - g.nxp + 1), xhi = min(nxExt - 1, X0 + kWarps - 1 + Hx);
   const int nRows = yeHi - yeLo + 1;
   auto key_lo = [&](int ye) { return ((int64_t)ye * nxExt + xlo) * nf; };
   auto key_hi = [&](int ye) { return ((int64_t)ye * nxExt + xhi) * nf + nf; };  // one past
   if (SPARSE) {
      const pvgpu_entry *eb = entries + (size_t)b * g.pre.numExt();
      const int64_t nAct = numActive[b];
      for (int t = threadIdx.x; t < 2 * nRows && xlo <= xhi; t += blockDim.x) {
         const int r = t >> 1;
         const int64_t key = (t & 1) ? key_hi(yeLo + r) : key_lo(yeLo + r);
         const int64_t v = lower_bound_entries(eb, nAct, (uint32_t)min(key, (int64_t)0xffffffffLL));
         if (t & 1) rowHi[r] = key > 0xffffffffLL ? nAct : v;
         else rowLo[r] = v;
      }
   }
   __syncthreads();
   if (X >= g.post.nx || xlo > xhi || nRows <= 0) return;  // no barrier below

   const pvgpu_entry *eb = SPARSE ? entries + (size_t)b * g.pre.numExt() : nullptr;
   const float *ab = SPARSE ? nullptr : aExt + (size_t)b * g.pre.numExt();
   const int fo0 = lane * FPL;
   const int rowStrideW = g.nxp * g.nfp;
   float *gcol = gsyn + (size_t)b * g.post.numRes() + (size_t)X * g.nfp + fo0;
   const size_t gRow = (size_t)g.post.nx * g.nfp;

   float acc[NYP][FPL];
#pragma unroll
   for (int s = 0; s < NYP; s++)
#pragma unroll
      for (int q = 0; q < FPL; q++) acc[s][q] = 0.0f;

   // Window of NYP post rows: while presynaptic row ye is processed, acc[j] holds post row
   // ye - Hy + j, so patch row ky of an entry of row ye always adds into acc[ky] (a static index).
   // After row ye, post row ye - Hy (acc[0]) has all its contributions: it is added into GSyn and
   // the window shifts by one row.  The first row visited puts post row P0 in acc[NYP - 1].
   const int yeFirst = P0 + Hy - (NYP - 1);
   const int yeEnd = P1 - 1 + Hy;  // the row that completes post row P1 - 1
   for (int ye = yeFirst; ye <= yeEnd; ye++) {
      if (ye >= yeLo && ye <= yeHi) {
         const int64_t lo = SPARSE ? rowLo[ye - yeLo] : key_lo(ye);
         const int64_t hi = SPARSE ? rowHi[ye - yeLo] : key_hi(ye);
         const int64_t kRow = (int64_t)ye * nxExt * nf;
         // patch rows of this presynaptic row that land inside [P0, P1)
         const int kyMin = max(0, P0 - (ye - Hy)), kyMax = min(NYP - 1, P1 - 1 - (ye - Hy));
         for (int64_t base = lo; base < hi; base += 32) {
            int64_t k = 0;
            float a = 0.0f;
            const bool have = base + lane < hi;
            if (have) {
               if (SPARSE) {
                  const pvgpu_entry en = eb[base + lane];
                  k = en.index;
                  a = en.value;
               } else {
                  k = base + lane;
                  a = ab[base + lane];
               }
            }
            const int kr = (int)(k - kRow);
            const int xe = kr / nf, f = kr - xe * nf;
            const int kx = X - (xe - Hx);
            const bool rel = have && a != 0.0f && kx >= 0 && kx < g.nxp;
            unsigned m = __ballot_sync(0xffffffffu, rel);
            const int woffMine = f * g.patchSize + kx * g.nfp;  // kernel index = f (one-to-one)
            // two entries per round: their weight loads are all in flight before the FMAs
            while (m) {
               const int j1 = __ffs(m) - 1;
               m &= m - 1;
               const bool two = m != 0;  // warp-uniform
               const int j2 = two ? __ffs(m) - 1 : j1;
               if (two) m &= m - 1;
               const float a1 = __shfl_sync(0xffffffffu, a, j1) * g.dtf;
               const float a2 = two ? __shfl_sync(0xffffffffu, a, j2) * g.dtf : 0.0f;
               const float *wp1 = W + __shfl_sync(0xffffffffu, woffMine, j1) + fo0;
               const float *wp2 = W + __shfl_sync(0xffffffffu, woffMine, j2) + fo0;
               float w1[NYP][FPL], w2[NYP][FPL];
#pragma unroll
               for (int ky = 0; ky < NYP; ky++) {
                  if (ky >= kyMin && ky <= kyMax) {
                     VecF<FPL>::ld(wp1 + ky * rowStrideW, w1[ky]);
                     if (two) VecF<FPL>::ld(wp2 + ky * rowStrideW, w2[ky]);
                  }
               }
#pragma unroll
               for (int ky = 0; ky < NYP; ky++) {
                  if (ky >= kyMin && ky <= kyMax) {
                     fma_row<FPL>(acc[ky], a1, w1[ky]);
                     if (two) fma_row<FPL>(acc[ky], a2, w2[ky]);
                  }
               }
            }
         }
      }
      // post row ye - Hy has all its contributions
      const int py = ye - Hy;
      if (py >= P0 && py < P1) VecF<FPL>::rmw(gcol + (size_t)py * gRow, acc[0]);
#pragma unroll
      for (int j = 0; j + 1 < NYP; j++)
#pragma unroll
         for (int q = 0; q < FPL; q++) acc[j][q] = acc[j + 1][q];
#pragma unroll
      for (int q = 0; q < FPL; q++) acc[NYP - 1][q] = 0.0f;
   }
}

template <int FPL, int NYP>
pvgpu_status launch_rows(const PreGeom &g, cudaStream_t s, const pvgpu_entry *entries, const int64_t *numActive,
                         const float *aExt, const float *W, float *gsyn) {
   dim3 grid((g.post.nx + kWarps - 1) / kWarps, (g.post.ny + kRowsRS - 1) / kRowsRS, g.post.nb);
   if (entries)
      deliver_pre_rows_kernel<FPL, NYP, true><<<grid, kWarps * 32, 0, s>>>(g, entries, numActive, nullptr, W, gsyn);
   else
      deliver_pre_rows_kernel<FPL, NYP, false><<<grid, kWarps * 32, 0, s>>>(g, nullptr, nullptr, aExt, W, gsyn);
   PVGPU_CHECK_LAUNCH("deliver_pre rows");
   return PVGPU_OK;
}

template <int FPL>
pvgpu_status launch_rows_nyp(const PreGeom &g, cudaStream_t s, const pvgpu_entry *entries, const int64_t *numActive,
                             const float *aExt, const float *W, float *gsyn) {
   switch (g.nyp) {
      case 1: return launch_rows<FPL, 1>(g, s, entries, numActive, aExt, W, gsyn);
      case 3: return launch_rows<FPL, 3>(g, s, entries, numActive, aExt, W, gsyn);
      case 5: return launch_rows<FPL, 5>(g, s, entries, numActive, aExt, W, gsyn);
      case 7: return launch_rows<FPL, 7>(g, s, entries, numActive, aExt, W, gsyn);
      case 9: return launch_rows<FPL, 9>(g, s, entries, numActive, aExt, W, gsyn);
      // taller patches keep NYP x FPL accumulators per lane: 32 and 64 post features only
      case 11: return FPL <= 2 ? launch_rows<FPL <= 2 ? FPL : 1, 11>(g, s, entries, numActive, aExt, W, gsyn)
                               : PVGPU_ERR_UNSUPPORTED_SHAPE;
      case 13: return FPL <= 2 ? launch_rows<FPL <= 2 ? FPL : 1, 13>(g, s, entries, numActive, aExt, W, gsyn)
                               : PVGPU_ERR_UNSUPPORTED_SHAPE;
      default: return PVGPU_ERR_UNSUPPORTED_SHAPE;
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

// post columns one presynaptic patch covers (the patch is counted in post neurons)
int post_patch_cols(const pvgpu_conn_desc *conn) { return conn->nxp; }

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
   // Every entry is broadcast to the whole warp and tested against each of its tile elements,
   // but covers only nxp post columns: a tile about twice the patch width keeps most of that
   // work useful (the per-element summation order does not depend on the tile).
   {
      const int want = 2 * post_patch_cols(conn) > 8 ? 2 * post_patch_cols(conn) : 8;
      if (g.TX > want) g.TX = want;
   }
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
   // FAST mode, one-to-one, nfp a multiple of 32 up to 128, odd patch height up to 9 (up to 13
   // for 32 or 64 post features): the row-sliding kernel
   const int rowRange = kRowsRS + conn->nyp - 1;
   if (!exact && pre.nx == post.nx && pre.ny == post.ny && post.nf % 32 == 0 && post.nf <= 128 &&
       conn->nyp <= 13 && rowRange <= kRowsMax && (post.nf / 32) != 3) {
      const int fpl = post.nf / 32;
      pvgpu_status r = fpl == 1   ? launch_rows_nyp<1>(g, s, entries, numActive, aExt, weights, gsyn)
                       : fpl == 2 ? launch_rows_nyp<2>(g, s, entries, numActive, aExt, weights, gsyn)
                                  : launch_rows_nyp<4>(g, s, entries, numActive, aExt, weights, gsyn);
      if (r != PVGPU_ERR_UNSUPPORTED_SHAPE) return r;
   }
   if (entries)
      return exact ? launch<true, true>(g, p2, grid, s, entries, numActive, nullptr, weights, gsyn)
                   : launch<true, false>(g, p2, grid, s, entries, numActive, nullptr, weights, gsyn);
   return exact ? launch<false, true>(g, p2, grid, s, nullptr, nullptr, aExt, weights, gsyn)
                : launch<false, false>(g, p2, grid, s, nullptr, nullptr, aExt, weights, gsyn);
}
