// deliver_tc.cu -- a4 / a5 on the tensor cores: FP32 one-to-one delivery as an implicit GEMM
// whose FP32 operands are each split into two TF32 parts (hi = tf32(x), lo = tf32(x - hi)),
// three TF32 products per term (hi*hi + hi*lo + lo*hi) accumulated in FP32 in TMEM.  The dropped
// lo*lo term and the split's rounding leave a relative error of about 2^-21 per product, the size
// of FP32 rounding in a long sum, so the result stands in for the FP32 deliveries:
//
//   GSyn[b][y][x][n] += dt_factor * sum_{ky, kx, f} A_ext[b][y + ky + sy0][x + kx + sx0][f]
//                                                  * Wpost[n][ky][kx][f]
//
// which is PostsynapticPerspectiveConvolveDelivery::deliver
// (delivery/PostsynapticPerspectiveConvolveDelivery.cpp:56-151) for a one-to-one connection, and,
// with Wpost = TransposeWeights::transposeShared of the presynaptic weights
// (utils/TransposeWeights.cpp:56-115), the same sums that the presynaptic scatter
// (delivery/PresynapticPerspectiveConvolveDelivery.cpp:61-192) forms in another order.
//
// GEMM view: M = 128 target positions of one row (x0 .. x0+127), N = a tile of NT <= 128 of
// the post features, K = (ky, kx, f).  Work unit = R target rows x 128 positions x NT features.
// Per 32-feature chunk the unit needs R + KY - 1 source rows; each is loaded once by TMA as a
// 136-position x 32-feature box (128-byte swizzle, 17 KB) into a small raw ring, then split
// into hi / lo tiles laid out as K-major without swizzle: eight 16-byte K-chunk columns of 136
// rows, rows 16 B apart.  In that layout an operand may start at any row, so one split row
// serves all KX shifts kx (the descriptor starts kx rows down) and all (ky, r) with r + ky = its
// row.  (A 128-byte-swizzled tile cannot be read from a row that is not a multiple of 8: the
// MMA applies the swizzle phase from the first row it reads.)  The weight tiles (hi rows then
// lo rows, NT x 32 TF32 each, pre-split in the workspace, 128-byte swizzle) stream through a
// ring, each used by the R rows of a unit.
//
// MMA shape.  One tcgen05.mma costs about 117 cycles for N <= 128 and 171 for N = 256 (TF32,
// M = 128, same accumulator), against 32 for N = 64 at the tensor pipe's peak, and switching
// accumulators between consecutive MMAs costs more still.  So the hi and lo weight tiles are
// one N = 2*NT operand: per K step, MMA 1 = A_hi x [W_hi; W_lo] (N = 2*NT) and MMA 2 =
// A_lo x W_hi (N = NT) into the same accumulator (columns n: W_hi parts, NT + n: A_hi x W_lo),
// two MMAs where three N = NT products would take three; the dropped A_lo x W_lo is below 2^-22
// of each product.
//
// Accumulation order.  The tensor core adds each MMA's products into the FP32 accumulator
// rounding toward zero, so a long chain of MMAs into one accumulator drifts toward zero in
// proportion to its length (measured: 1e-4 of max|GSyn| at K = 12,544).  The MMAs therefore
// accumulate short chains -- a run of patch rows of one 32-feature chunk, at least 7 weight
// tiles (28 K steps) long -- into one of two TMEM chain buffers, and the epilogue warps add each
// chain's two column halves and then the chain into FP32 registers with round-to-nearest, and
// add dt_factor * sum into GSyn once per unit.  Each chain's drift is small and its sign follows the chain's own partial sum, so the
// drifts of the chains cancel like rounding errors.
//
#include "pvgpu_internal.cuh"
#include "tc_ptx.cuh"
#include "tmap.cuh"

#include <algorithm>
#include <cstdint>

namespace {

using namespace pvgpu::tc;

constexpr int kThreads = 320;
constexpr int kRowsA = 136;                  // 128 positions + up to 8 kx shifts
constexpr uint32_t kHalfA = kRowsA * 128;    // one TF32 tile of a source row (17,408 B)
constexpr uint32_t kSlotA = 2 * kHalfA;      // hi + lo
constexpr uint32_t kColA = kRowsA * 16;      // one 16-byte K-chunk column of a split tile
constexpr int kMaxNS = 8, kMaxNB = 8, kMaxNR = 2;
constexpr int kSmemLimit = 227 * 1024;

struct TcGeom {
   int nb, nx, ny, N, C, KX, KY;
   int nyExt;        // source rows per image (TMA row coordinate = b * nyExt + row)
   int sx0, sy0;     // source extended column / row read by target (0, 0) at kx = ky = 0
   int R, NS, NB, NR;  // target rows per unit, split-row slots, weight-tile slots, raw-row slots
   int NT, nNT;        // post features per unit, feature tiles
   int nXT, nYG, units, nFC;
   int groupsPerChain, chainsPerUnit;  // (fc, ky) groups per MMA chain, chains per unit
   float dtf;
   uint32_t offRaw, offB, tmemCols;
};

__device__ __forceinline__ uint8_t *align1024(uint8_t *p) {
   return reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(p) + 1023) & ~static_cast<uintptr_t>(1023));
}

// R = target rows per unit (g.R); NCH = R * NT / 32: 32-column chunks of the result, summed in
// registers by the epilogue (a chain buffer holds 2 * NCH chunks: hi-weight and lo-weight
// columns).  R is a template parameter so that the 8R MMAs of one weight tile issue as one
// branch-free sequence: a branch between consecutive tcgen05.mma instructions costs the issuing
// thread tens of cycles, as much as an N = 64 MMA itself.
template <int R, int NCH>
__global__ void __launch_bounds__(kThreads, 1) conv_tf32x3_kernel(const __grid_constant__ CUtensorMap tmA,
                                                                  const __grid_constant__ CUtensorMap tmB, TcGeom g,
                                                                  float *__restrict__ gsyn, int *__restrict__ err) {
   extern __shared__ uint8_t smem_raw[];
   uint8_t *smem = align1024(smem_raw);
   __shared__ __align__(8) uint64_t rawFull[kMaxNR], rawEmpty[kMaxNR], aReady[kMaxNS], aEmpty[kMaxNS],
         bFull[kMaxNB], bEmpty[kMaxNB], chainFull[2], chainEmpty[2], mmaDone;
   __shared__ uint32_t tmemBase;
   __shared__ volatile int abortFlag;

   const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
   const uint32_t bBytes = (uint32_t)g.NT * 128;  // one TF32 weight tile (NT rows x 32)
   const int groupsPerUnit = g.nFC * g.KY;
   const int rowsPerFC = g.R + g.KY - 1;

   if (tid == 0) {
      for (int i = 0; i < kMaxNR; i++) {
         mbar_init(&rawFull[i], 1);
         mbar_init(&rawEmpty[i], 4);  // one arrival per split warp
      }
      for (int i = 0; i < kMaxNS; i++) {
         mbar_init(&aReady[i], 4);  // one arrival per split warp
         mbar_init(&aEmpty[i], 1);
      }
      for (int i = 0; i < kMaxNB; i++) {
         mbar_init(&bFull[i], 1);
         mbar_init(&bEmpty[i], 1);
      }
      for (int i = 0; i < 2; i++) {
         mbar_init(&chainFull[i], 1);
         mbar_init(&chainEmpty[i], 4);  // one arrival per epilogue warp
      }
      mbar_init(&mmaDone, 1);
      abortFlag = 0;
      fence_mbar_init();
   }
   if (warp == 1) tmem_alloc(&tmemBase, g.tmemCols);
   tc_fence_before();
   __syncthreads();
   tc_fence_after();
   const uint32_t tmem = tmemBase;

   auto wait_or_abort = [&](uint64_t *bar, uint32_t parity) {
      if (abortFlag) return false;
      if (mbar_wait(bar, parity)) return true;
      abortFlag = 1;
      return false;
   };
   // warp-uniform wait: every lane observes the phase; the warp goes on only if all of them did
   auto warp_wait = [&](uint64_t *bar, uint32_t parity) {
      const bool mine = !abortFlag && mbar_wait(bar, parity);
      const bool all = __all_sync(0xffffffffu, mine) != 0;
      if (!all && lane == 0) abortFlag = 1;
      return all;
   };
   auto fresh0 = [](bool fresh) { return fresh ? 0u : 1u; };
   auto unit_of = [&](int u, int &b, int &y0, int &x0, int &n0) {
      n0 = (u % g.nNT) * g.NT;
      const int t0 = u / g.nNT;
      const int xt = t0 % g.nXT;
      const int t = t0 / g.nXT;
      y0 = (t % g.nYG) * g.R;
      b = t / g.nYG;
      x0 = xt * 128;
   };

   if (warp == 0) {
      // ================================ TMA producer ================================
      if (lane == 0) {
         prefetch_tmap(&tmA);
         prefetch_tmap(&tmB);
         uint32_t ca = 0, cb = 0;
         bool ok = true;
         for (int u = blockIdx.x; u < g.units && ok; u += gridDim.x) {
            int b, y0, x0, n0;
            unit_of(u, b, y0, x0, n0);
            for (int fc = 0; fc < g.nFC && ok; fc++) {
               const int f0 = fc * 32;
               auto loadA = [&](int j) {
                  const int rr = (int)(ca % g.NR);
                  if (ca >= (uint32_t)g.NR && !wait_or_abort(&rawEmpty[rr], ((ca / g.NR) - 1) & 1)) return false;
                  mbar_arrive_expect_tx(&rawFull[rr], kHalfA);
                  tma_load_3d(smem + g.offRaw + rr * kHalfA, &tmA, &rawFull[rr], f0, x0 + g.sx0,
                              b * g.nyExt + y0 + j + g.sy0);
                  ca++;
                  return true;
               };
               auto loadB = [&](int ky, int kx) {
                  const int d = (int)(cb % g.NB);
                  if (cb >= (uint32_t)g.NB && !wait_or_abort(&bEmpty[d], ((cb / g.NB) - 1) & 1)) return false;
                  uint8_t *dst = smem + g.offB + d * 2 * bBytes;
                  const int k0 = (ky * g.KX + kx) * g.C + f0;
                  mbar_arrive_expect_tx(&bFull[d], 2 * bBytes);
                  tma_load_2d(dst, &tmB, &bFull[d], k0, n0);                 // hi rows n0 ..
                  tma_load_2d(dst + bBytes, &tmB, &bFull[d], k0, g.N + n0);  // lo rows N + n0 ..
                  cb++;
                  return true;
               };
               for (int j = 0; j + 1 < g.R && ok; j++) ok = loadA(j);
               for (int ky = 0; ky < g.KY && ok; ky++) {
                  ok = loadA(ky + g.R - 1);
                  for (int kx = 0; kx < g.KX && ok; kx++) ok = loadB(ky, kx);
               }
            }
         }
         // copies still in flight must land before the CTA may exit
         if (!ok) {
            for (uint32_t c = ca > (uint32_t)g.NR ? ca - g.NR : 0; c < ca; c++) mbar_wait(&rawFull[c % g.NR], (c / g.NR) & 1);
            for (uint32_t c = cb > (uint32_t)g.NB ? cb - g.NB : 0; c < cb; c++) mbar_wait(&bFull[c % g.NB], (c / g.NB) & 1);
         }
      }
   } else if (warp == 1) {
      // ================================ MMA issuer ================================
      if (lane == 0) {
         const uint32_t idesc = idesc_tf32(128, 2 * g.NT), idescHi = idesc_tf32(128, g.NT);
         // Descriptors are built once; an operand at byte offset o from its base is the base
         // descriptor plus o >> 4 (the start-address field, which cannot carry: shared-memory
         // addresses are below 2^18).
         const uint64_t aD0 = sdesc_noswizzle(smem_u32(smem), kColA, 128);
         const uint64_t bD0 = sdesc_sw128(smem_u32(smem + g.offB));
         constexpr uint64_t kLoA = kHalfA >> 4, kStepA = (2 * kColA) >> 4;
         uint32_t cbase = 0, cb = 0, cc = 0;  // split rows, weight tiles, chains so far
         int slotBase = 0;                    // cbase % NS
         int d = 0;                           // cb % NB
         uint32_t bPar = 0;                   // (cb / NB) & 1
         bool ok = true;
         for (int u = blockIdx.x; u < g.units && ok; u += gridDim.x) {
            int grp = 0;
            uint32_t tacc = 0;
            for (int fc = 0; fc < g.nFC && ok; fc++) {
               for (int ky = 0; ky < g.KY && ok; ky++, grp++) {
                  const bool chainStart = grp % g.groupsPerChain == 0;
                  if (chainStart) {
                     const int buf = cc & 1;
                     if (cc >= 2 && !(ok = wait_or_abort(&chainEmpty[buf], ((cc >> 1) - 1) & 1))) break;
                     tc_fence_after();  // the epilogue's TMEM reads of this buffer precede the MMAs
                     tacc = tmem + (uint32_t)(buf * 2 * NCH * 32);
                  }
                  // source rows ky .. ky+R-1 of this chunk must be split
                  for (int j = ky == 0 ? 0 : ky + g.R - 1; j < ky + g.R && ok; j++) {
                     const uint32_t c = cbase + j;
                     ok = wait_or_abort(&aReady[c % g.NS], (c / g.NS) & 1);
                  }
                  if (!ok) break;
                  // operands written by TMA or by proxy-fenced stores need no tcgen05 fence
                  const int slotKy = (slotBase + ky) % g.NS;
                  for (int kx = 0; kx < g.KX && ok; kx++) {
                     if (!(ok = wait_or_abort(&bFull[d], bPar))) break;
                     const uint64_t bd = bD0 + (uint64_t)((d * 2 * bBytes) >> 4);
                     const uint32_t acc0 = fresh0(chainStart && kx == 0);
                     uint64_t adr[R];
#pragma unroll
                     for (int r = 0; r < R; r++) {
                        const int slot = slotKy + r >= g.NS ? slotKy + r - g.NS : slotKy + r;
                        adr[r] = aD0 + (uint64_t)((slot * kSlotA + kx * 16) >> 4);
                     }
#pragma unroll
                     for (int r = 0; r < R; r++) {
                        const uint32_t dt = tacc + (uint32_t)(r * 2 * g.NT);
#pragma unroll
                        for (int k = 0; k < 4; k++) {  // K step of 8 TF32 = two chunk columns
                           const uint64_t ah = adr[r] + k * kStepA, bhl = bd + 2 * k;
                           mma_tf32(dt, ah, bhl, idesc, k == 0 ? acc0 : 1u);  // A_hi x [W_hi; W_lo]
                           mma_tf32(dt, ah + kLoA, bhl, idescHi, 1);           // A_lo x W_hi
                        }
                     }
                     mma_commit(&bEmpty[d]);
                     cb++;
                     if (++d == g.NB) {
                        d = 0;
                        bPar ^= 1u;
                     }
                  }
                  if (!ok) break;
                  mma_commit(&aEmpty[slotKy]);  // row ky has no later use
                  if ((grp + 1) % g.groupsPerChain == 0 || grp + 1 == groupsPerUnit) {
                     mma_commit(&chainFull[cc & 1]);
                     cc++;
                  }
               }
               if (!ok) break;
               for (int j = g.KY; j < rowsPerFC; j++) mma_commit(&aEmpty[(slotBase + j) % g.NS]);
               cbase += rowsPerFC;
               slotBase = (slotBase + rowsPerFC) % g.NS;
            }
         }
         // every MMA issued has completed before TMEM is released
         mma_commit(&mmaDone);
         mbar_wait(&mmaDone, 0);
      }
   } else if (warp < 6) {
      // ================================ hi / lo split ================================
      // raw row (128-byte swizzle: chunk j of row r at r*128 + ((j ^ (r & 7)) << 4)) -> hi and lo
      // chunk columns (chunk j of row r at j*kColA + r*16); consecutive threads take consecutive
      // rows of one chunk, so both the reads and the writes are free of bank conflicts
      const int st = tid - 64;  // 0 .. 127
      uint32_t c = 0;
      bool ok = true;
      for (int u = blockIdx.x; u < g.units && ok; u += gridDim.x) {
         for (int fc = 0; fc < g.nFC && ok; fc++) {
            for (int j = 0; j < rowsPerFC && ok; j++, c++) {
               const int rr = (int)(c % g.NR), s = (int)(c % g.NS);
               if (!(ok = warp_wait(&rawFull[rr], (c / g.NR) & 1))) break;
               if (c >= (uint32_t)g.NS && !(ok = warp_wait(&aEmpty[s], ((c / g.NS) - 1) & 1))) break;
               const uint8_t *raw = smem + g.offRaw + rr * kHalfA;
               uint8_t *hi = smem + s * kSlotA;
               uint8_t *lo = hi + kHalfA;
               for (int i = st; i < kRowsA * 8; i += 128) {
                  const int ch = i / kRowsA, row = i - ch * kRowsA;
                  const float4 v = *reinterpret_cast<const float4 *>(raw + row * 128 + ((ch ^ (row & 7)) << 4));
                  float4 h, l;
                  h.x = to_tf32(v.x);
                  h.y = to_tf32(v.y);
                  h.z = to_tf32(v.z);
                  h.w = to_tf32(v.w);
                  l.x = to_tf32(v.x - h.x);
                  l.y = to_tf32(v.y - h.y);
                  l.z = to_tf32(v.z - h.z);
                  l.w = to_tf32(v.w - h.w);
                  *reinterpret_cast<float4 *>(hi + ch * kColA + row * 16) = h;
                  *reinterpret_cast<float4 *>(lo + ch * kColA + row * 16) = l;
               }
               fence_proxy_async_smem();
               __syncwarp();
               if (lane == 0) {
                  mbar_arrive(&aReady[s]);
                  mbar_arrive(&rawEmpty[rr]);
               }
            }
         }
      }
   } else {
      // ================================ epilogue ================================
      const int q = warp & 3;  // TMEM lane quadrant this warp may read
      const int chunksPerRow = g.NT / 32;
      uint32_t cc = 0;
      bool ok = true;
      for (int u = blockIdx.x; u < g.units && ok; u += gridDim.x) {
         float acc[NCH * 32];
#pragma unroll
         for (int i = 0; i < NCH * 32; i++) acc[i] = 0.0f;
         for (int ch = 0; ch < g.chainsPerUnit; ch++, cc++) {
            const int buf = cc & 1;
            if (!(ok = warp_wait(&chainFull[buf], (cc >> 1) & 1))) break;
            tc_fence_after();
#pragma unroll
            for (int c = 0; c < NCH; c++) {
               // chunk c = (row r, feature columns h*32 ..): hi-weight part at r*2NT + h*32,
               // lo-weight part NT columns further
               const int r = c / chunksPerRow, h = c - r * chunksPerRow;
               const uint32_t col = (uint32_t)(buf * 2 * NCH * 32 + r * 2 * g.NT + h * 32);
#pragma unroll
               for (int half = 0; half < 2; half++) {
                  float vh[16], vl[16];
                  tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + col + 16 * half, vh);
                  tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + col + 16 * half + g.NT, vl);
#pragma unroll
                  for (int i = 0; i < 16; i++)
                     acc[c * 32 + 16 * half + i] = __fadd_rn(acc[c * 32 + 16 * half + i], __fadd_rn(vh[i], vl[i]));
               }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&chainEmpty[buf]);
         }
         if (!ok) break;
         int b, y0, x0, n0;
         unit_of(u, b, y0, x0, n0);
         const int x = x0 + 32 * q + lane;
#pragma unroll
         for (int c = 0; c < NCH; c++) {
            const int r = c / chunksPerRow, nc = n0 + (c - r * chunksPerRow) * 32;
            const int y = y0 + r;
            if (y < g.ny && x < g.nx) {
               float4 *p4 = reinterpret_cast<float4 *>(gsyn + (((size_t)b * g.ny + y) * g.nx + x) * g.N + nc);
#pragma unroll
               for (int i = 0; i < 8; i++) {
                  float4 o = p4[i];
                  o.x = fmaf(g.dtf, acc[c * 32 + 4 * i], o.x);
                  o.y = fmaf(g.dtf, acc[c * 32 + 4 * i + 1], o.y);
                  o.z = fmaf(g.dtf, acc[c * 32 + 4 * i + 2], o.z);
                  o.w = fmaf(g.dtf, acc[c * 32 + 4 * i + 3], o.w);
                  p4[i] = o;
               }
            }
         }
      }
   }
   __syncthreads();
   if (tid == 0 && abortFlag) atomicExch(err, 1);
   tc_fence_before();
   __syncthreads();
   if (warp == 1) tmem_dealloc(tmem, g.tmemCols);
}

// hi / lo TF32 split of the post-perspective weights: out = [hi: n][lo: n]
__global__ void split_tf32_kernel(const float *__restrict__ w, float *__restrict__ out, int64_t n) {
   for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
      const float x = w[i];
      const float h = to_tf32(x);
      out[i] = h;
      out[n + i] = to_tf32(x - h);
   }
}

int *error_flag() {
   static int *flag = nullptr;
   if (!flag && cudaMalloc(&flag, sizeof(int)) == cudaSuccess) cudaMemset(flag, 0, sizeof(int));
   return flag;
}

// Shape checks and the tile plan; UNSUPPORTED_SHAPE for geometry this path does not take.
pvgpu_status plan(const pvgpu_conn_desc *conn, TcGeom &g, int numSms) {
   const pvgpu_loc &pre = conn->pre, &post = conn->post;
   if (!pvgpu::loc_valid(pre) || !pvgpu::loc_valid(post) || pre.nbatch != post.nbatch) return PVGPU_ERR_BAD_ARG;
   if (!pvgpu::axis_legal(pre.nx, post.nx, conn->nxp) || !pvgpu::axis_legal(pre.ny, post.ny, conn->nyp))
      return PVGPU_ERR_ILLEGAL_GEOMETRY;
   if (pre.nx != post.nx || pre.ny != post.ny) return PVGPU_ERR_UNSUPPORTED_SHAPE;  // one-to-one only
   const int mx = pvgpu::required_margin(pre.nx, post.nx, conn->nxp);
   const int my = pvgpu::required_margin(pre.ny, post.ny, conn->nyp);
   if (pre.halo.lt < mx || pre.halo.rt < mx || pre.halo.dn < my || pre.halo.up < my) return PVGPU_ERR_BAD_ARG;
   if (pre.halo.lt != pre.halo.dn || pre.halo.lt != pre.halo.rt || pre.halo.dn != pre.halo.up)
      return PVGPU_ERR_UNSUPPORTED_SHAPE;
   if (pre.nf % 32 != 0 || post.nf % 32 != 0 || conn->nxp > kRowsA - 127) return PVGPU_ERR_UNSUPPORTED_SHAPE;
   g.nb = post.nbatch;
   g.nx = post.nx;
   g.ny = post.ny;
   g.N = post.nf;
   g.C = pre.nf;
   g.KX = conn->nxp;
   g.KY = conn->nyp;
   g.nyExt = pre.ny + pre.halo.dn + pre.halo.up;
   g.sx0 = pre.halo.lt - (conn->nxp - 1) / 2;
   g.sy0 = pre.halo.dn - (conn->nyp - 1) / 2;
   g.nFC = g.C / 32;
   g.nXT = (g.nx + 127) / 128;
   g.dtf = conn->dt_factor;
   // feature tile: the largest of 128, 96, 64, 32 dividing post.nf
   g.NT = 32;
   for (int nt : {128, 96, 64})
      if (g.N % nt == 0) {
         g.NT = nt;
         break;
      }
   g.nNT = g.N / g.NT;
   // R: the epilogue holds R x NT sums per thread (R * NT <= 128); fewest (waves x rows per
   // unit), ties to the larger R (fewer weight-tile loads per MMA)
   int bestR = 1;
   int64_t bestCost = -1;
   for (int R = 1; R * g.NT <= 128; R++) {
      const int64_t units = (int64_t)g.nb * ((g.ny + R - 1) / R) * g.nXT * g.nNT;
      const int64_t waves = (units + numSms - 1) / numSms;
      const int64_t cost = waves * R * 4 + (R == 1 ? 1 : 0);
      if (bestCost < 0 || cost <= bestCost) {
         bestCost = cost;
         bestR = R;
      }
   }
   g.R = bestR;
   g.nYG = (g.ny + g.R - 1) / g.R;
   const int64_t units = (int64_t)g.nb * g.nYG * g.nXT * g.nNT;
   if (units > 0x7fffffff) return PVGPU_ERR_UNSUPPORTED_SHAPE;
   g.units = (int)units;
   // a chain spans whole patch rows of one 32-feature chunk, at least 7 weight tiles
   g.groupsPerChain = std::max(1, std::min(g.KY, (7 + g.KX - 1) / g.KX));
   {
      // chains close after group grp when (grp + 1) % groupsPerChain == 0 or at the unit's end
      const int groups = g.nFC * g.KY;
      g.chainsPerUnit = (groups + g.groupsPerChain - 1) / g.groupsPerChain;
   }
   // shared memory: weight tiles first (6 preferred: a slot frees only when its MMAs retire, and
   // a tile's MMAs are short next to an L2 round trip), then split rows (R+2 preferred, R+1 at
   // least), then raw rows (2 preferred; one suffices, a source row is needed once per patch row)
   const int64_t bTile = 2 * (int64_t)g.NT * 128;
   const int64_t budget = kSmemLimit - 1024 - 512;
   g.NS = 0;
   for (int want = 6; want >= 2 && g.NS == 0; want--)
      for (int nr = kMaxNR; nr >= 1 && g.NS == 0; nr--)
         for (int ns = std::min(kMaxNS, g.R + 2); ns >= g.R + 1 && g.NS == 0; ns--) {
            const int64_t nbFit = (budget - (int64_t)ns * kSlotA - (int64_t)nr * kHalfA) / bTile;
            if (nbFit >= want) {
               g.NS = ns;
               g.NR = nr;
               g.NB = (int)std::min<int64_t>(kMaxNB, nbFit);
            }
         }
   if (g.NS == 0) return PVGPU_ERR_UNSUPPORTED_SHAPE;
   g.offRaw = (uint32_t)g.NS * kSlotA;
   g.offB = g.offRaw + (uint32_t)g.NR * kHalfA;
   uint32_t cols = 32;
   while (cols < (uint32_t)(4 * g.R * g.NT)) cols <<= 1;  // two chain buffers of R x 2NT
   g.tmemCols = cols;
   return PVGPU_OK;
}

size_t weights_floats(const pvgpu_conn_desc *conn) {
   return (size_t)conn->post.nf * conn->nxp * conn->nyp * conn->pre.nf;
}

pvgpu_status run(const pvgpu_conn_desc *conn, const float *aExt, const float *postWeights, float *gsyn,
                 void *workspace, size_t wsBytes, bool split, cudaStream_t s) {
   int dev = 0, numSms = 0;
   PVGPU_CUDA(cudaGetDevice(&dev), "deliver_tc device");
   PVGPU_CUDA(cudaDeviceGetAttribute(&numSms, cudaDevAttrMultiProcessorCount, dev), "deliver_tc SMs");
   TcGeom g;
   pvgpu_status st = plan(conn, g, numSms);
   if (st != PVGPU_OK) return st;
   const size_t nW = weights_floats(conn);
   float *wsplit = reinterpret_cast<float *>(workspace);
   if (!workspace || wsBytes < 2 * nW * sizeof(float) || (reinterpret_cast<uintptr_t>(workspace) & 15) ||
       (reinterpret_cast<uintptr_t>(aExt) & 15) || (reinterpret_cast<uintptr_t>(gsyn) & 15))
      return PVGPU_ERR_BAD_ARG;
   if (split) {
      split_tf32_kernel<<<std::max(1, std::min(numSms * 4, (int)((nW + 255) / 256))), 256, 0, s>>>(postWeights, wsplit,
                                                                                                 (int64_t)nW);
      PVGPU_CHECK_LAUNCH("deliver_tc split");
   }
   pvgpu::EncodeTiledFn enc = pvgpu::encode_tiled_fn();
   if (!enc) return pvgpu::record_message(PVGPU_ERR_LAUNCH, "deliver_tc: cuTensorMapEncodeTiled unavailable");
   const pvgpu_loc &pre = conn->pre;
   const uint64_t nxExt = (uint64_t)pre.nx + pre.halo.lt + pre.halo.rt;
   CUtensorMap tmA, tmB;
   {
      cuuint64_t dims[3] = {(cuuint64_t)g.C, nxExt, (cuuint64_t)g.nyExt * g.nb};
      cuuint64_t strides[2] = {(cuuint64_t)g.C * 4, nxExt * g.C * 4};
      cuuint32_t box[3] = {32, (cuuint32_t)kRowsA, 1};
      cuuint32_t estr[3] = {1, 1, 1};
      if (enc(&tmA, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(aExt), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
         return pvgpu::record_message(PVGPU_ERR_UNSUPPORTED_SHAPE, "deliver_tc: activity tensor map rejected");
   }
   {
      const uint64_t K = (uint64_t)g.KY * g.KX * g.C;
      cuuint64_t dims[2] = {K, (cuuint64_t)2 * g.N};
      cuuint64_t strides[1] = {K * 4};
      cuuint32_t box[2] = {32, (cuuint32_t)g.NT};
      cuuint32_t estr[2] = {1, 1};
      if (enc(&tmB, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, wsplit, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
         return pvgpu::record_message(PVGPU_ERR_UNSUPPORTED_SHAPE, "deliver_tc: weight tensor map rejected");
   }
   const size_t smemBytes = 1024 + (size_t)g.offB + (size_t)g.NB * 2 * g.NT * 128;
   // a misread descriptor would still stay inside the allocation: the weight ring (or padding)
   // follows the last split row by more than a full split tile
   if (smemBytes - 1024 - (size_t)(g.NS - 1) * kSlotA < 2 * kSlotA) return PVGPU_ERR_UNSUPPORTED_SHAPE;
   int *err = error_flag();
   if (!err) return PVGPU_ERR_OOM;
   const int grid = std::min(g.units, numSms);
   const int nch = g.R * g.NT / 32;
   using Kern = void (*)(CUtensorMap, CUtensorMap, TcGeom, float *, int *);
   auto launch = [&](Kern kern, int idx) -> pvgpu_status {
      static bool attrSet[8] = {false, false, false, false, false, false, false, false};  // per instantiation
      if (!attrSet[idx]) {
         PVGPU_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemLimit - 512),
                    "deliver_tc smem attribute");
         attrSet[idx] = true;
      }
      kern<<<grid, kThreads, smemBytes, s>>>(tmA, tmB, g, gsyn, err);
      return PVGPU_OK;
   };
   pvgpu_status ls = PVGPU_ERR_UNSUPPORTED_SHAPE;
   switch (g.R * 8 + nch) {
      case 1 * 8 + 1: ls = launch(conv_tf32x3_kernel<1, 1>, 0); break;
      case 1 * 8 + 2: ls = launch(conv_tf32x3_kernel<1, 2>, 1); break;
      case 1 * 8 + 3: ls = launch(conv_tf32x3_kernel<1, 3>, 2); break;
      case 1 * 8 + 4: ls = launch(conv_tf32x3_kernel<1, 4>, 3); break;
      case 2 * 8 + 2: ls = launch(conv_tf32x3_kernel<2, 2>, 4); break;
      case 2 * 8 + 4: ls = launch(conv_tf32x3_kernel<2, 4>, 5); break;
      case 3 * 8 + 3: ls = launch(conv_tf32x3_kernel<3, 3>, 6); break;
      case 4 * 8 + 4: ls = launch(conv_tf32x3_kernel<4, 4>, 7); break;
      default: break;
   }
   if (ls != PVGPU_OK) return ls;
   PVGPU_CHECK_LAUNCH("deliver_tc");
   return PVGPU_OK;
}

}  // namespace

extern "C" size_t pvgpu_deliver_tc_workspace_bytes(const pvgpu_conn_desc *conn) {
   if (!conn) return 0;
   int dev = 0, numSms = 0;
   if (cudaGetDevice(&dev) != cudaSuccess ||
       cudaDeviceGetAttribute(&numSms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
      cudaGetLastError();
      numSms = 152;
   }
   TcGeom g;
   if (plan(conn, g, numSms) != PVGPU_OK) return 0;  // a shape these entries do not take
   // transposed weights (presynaptic entry) + their hi / lo split
   return 3 * weights_floats(conn) * sizeof(float);
}

extern "C" pvgpu_status pvgpu_deliver_post_tc(const pvgpu_conn_desc *conn, const float *aExt,
                                              const float *postWeights, float *gsyn, void *workspace,
                                              size_t workspaceBytes, void *stream) {
   if (!conn || !aExt || !postWeights || !gsyn) return PVGPU_ERR_BAD_ARG;
   return run(conn, aExt, postWeights, gsyn, workspace, workspaceBytes, true, pvgpu::as_stream(stream));
}

extern "C" pvgpu_status pvgpu_deliver_pre_tc(const pvgpu_conn_desc *conn, const float *aExt, const float *weights,
                                             float *gsyn, void *workspace, size_t workspaceBytes, void *stream) {
   if (!conn || !aExt || !weights || !gsyn || !workspace) return PVGPU_ERR_BAD_ARG;
   const size_t nW = weights_floats(conn);
   if (workspaceBytes < 3 * nW * sizeof(float)) return PVGPU_ERR_BAD_ARG;
   TcGeom g;
   int dev = 0, numSms = 1;
   PVGPU_CUDA(cudaGetDevice(&dev), "deliver_tc device");
   PVGPU_CUDA(cudaDeviceGetAttribute(&numSms, cudaDevAttrMultiProcessorCount, dev), "deliver_tc SMs");
   pvgpu_status st = plan(conn, g, numSms);  // refuse before writing the workspace
   if (st != PVGPU_OK) return st;
   float *wpost = reinterpret_cast<float *>(workspace) + 2 * nW;
   cudaStream_t s = pvgpu::as_stream(stream);
   st = pvgpu_transpose_weights(conn, weights, wpost, stream);
   if (st != PVGPU_OK) return st;
   return run(conn, aExt, wpost, gsyn, workspace, 2 * nW * sizeof(float), true, s);
}

extern "C" int pvgpu_deliver_tc_check_error(void) {
   int *err = error_flag();
   int h = 0;
   if (err && cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess && h) cudaMemset(err, 0, sizeof(int));
   return h;
}
