// lca_solver.cu -- the batched LCA module (input -> error <-> V1) on the tcgen05 tensor cores
// (BF16 operands, FP32 accumulation): one fused kernel per BF16 timestep (kernel F, below), or
// two kernels per timestep (kernels R and P: the first and last BF16 steps of a run, BF16x3
// steps, and every step when fusion is off); the plain FP32 form runs the two-kernel structure
// on the FP32 pipes.
//
// Reference path (per timestep, HyPerCol::advanceTime, columns/HyPerCol.cpp:659-790):
//   error layer (phase 1): G = input - W^T a(t-1)   IdentConn ch0 + HyPerConn V1->Error ch1
//                                                      (PresynapticPerspectiveConvolveDelivery)
//   V1 (phase 2):         G = W . err               TransposeConn, PostsynapticPerspectiveConvolveDelivery
//                          V = e V + (1-e)(G + A)    HyPerLCAInternalStateBuffer.kpp:18-63
//                          A = T(V)                  ANNActivityBuffer.cpp:490-558
//
// Kernel R ("recon"): one CTA per (image, block of 128 V1 positions).  GEMM
//   D[pos][k] = sum_f A[pos][f] * W[f][k],  k = (ky*P + kx)*C + c  (M = 128, N = P*P*C, K = F)
// A and W^T stream by TMA into 128B-swizzled shared tiles, tcgen05.mma accumulates in TMEM.
// The fold of D into the error image (patch (ky,kx) of position (y,x) lands on pixel
// (S*y - E + ky, S*x - E + kx)) runs in 16 tap groups; one group holds one tap of each
// pixel-parity class, so no two threads touch a pixel inside a group and every pixel sums
// its contributions in the same fixed group order -- deterministic, no atomics.  The
// block's partial reconstruction goes to HBM.
//
// Kernel P ("post"): persistent; tiles of (image, block of 128 positions, block of FT features).
//   residual r = x - sum of the image's partial reconstructions (FP32, fixed order),
//   staged for the block's receptive-field window in shared memory;
//   im2col of r into a 128B-swizzled BF16 operand by the CTA's threads;
//   D[pos][f] = sum_k r[pos][k] * W[f][k] on tcgen05 (TMEM accumulator);
//   epilogue per (position, feature): A_old = T(V_old); V = e V_old + (1-e)(D + A_old);
//   A = T(V) -> BF16 for the next step's kernel R.  A load warp, an MMA warp and 8 epilogue
//   warps hand tiles to one another through mbarriers (see the kernel's own header).
// BF16x3 mode adds the hi*lo and lo*hi products (operands split as x = hi + lo).
#include "lca_common.cuh"
#include "tc_ptx.cuh"
#include "tmap.cuh"

#include <cuda_bf16.h>

#include <algorithm>
#include <cfloat>
#include <cstdio>
#include <cstring>
#include <new>
#include <array>
#include <map>
#include <mutex>
#include <vector>

namespace {

using namespace pvgpu::tc;
using bf16 = __nv_bfloat16;

using pvgpu::LcaGeom;
using pvgpu::rwin_cols;
using pvgpu::rwin_rows;
using pvgpu::v_index;

// Rounds a pointer into the dynamic shared array up to 1024 bytes by adding an offset to it
// (not through an integer), so that accesses through the result stay shared-memory accesses.
__device__ __forceinline__ uint8_t *align1024(uint8_t *p) {
   const uint32_t a = smem_u32(p);
   return p + ((1024u - (a & 1023u)) & 1023u);
}

__device__ __forceinline__ float thresh(float v, const LcaGeom &g) { return pvgpu::lca_thresh(v, g); }

// Issue nchunks x8 TMEM loads (8 columns each) then wait once.
template <int N>
__device__ __forceinline__ void tmem_ld_cols(uint32_t taddr, float *v) {
   static_assert(N % 8 == 0, "columns in multiples of 8");
   uint32_t r[N];
#pragma unroll
   for (int c = 0; c < N; c += 8) {
      asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                   : "=r"(r[c + 0]), "=r"(r[c + 1]), "=r"(r[c + 2]), "=r"(r[c + 3]), "=r"(r[c + 4]),
                     "=r"(r[c + 5]), "=r"(r[c + 6]), "=r"(r[c + 7])
                   : "r"(taddr + c));
   }
   asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
   for (int i = 0; i < N; i++) v[i] = __uint_as_float(r[i]);
}

// -------------------------------------------------------------------------------------------
// Kernel R: reconstruction W^T a and the residual x - W^T a (persistent, warp-specialised)
//
// CTA i of the persistent grid walks images i, i + G, ...  Per image and 128-position block mb:
//   D[pos][k] = sum_f A[pos][f] * W[f][k],  k = (ky*P + kx)*C + c  (M = 128, N = P*P*C, K = F)
// Roles:
//   warp 8, lane 0 (loads): per block and chunk of 64 features, into one stage of an nStage
//                           ring: the A tile [128 x 64] and the W^T tile [P*P*C x 64] (two TMA
//                           boxes of P*P*C/2 rows), plus each image's x (bulk copy, two buffers);
//   warp 9, lane 0 (MMA):   per block the tcgen05.mma chain over F into one of two TMEM
//                           accumulators (256 columns apart); each stage is released by a
//                           tcgen05.commit once its MMAs are done;
//   warps 0-7 (fold):       thread = position (TMEM lane) and half of the patch rows.  The fold
//                           of D into the image (patch (ky,kx) of position (y,x) lands on pixel
//                           (S*y - E + ky, S*x - E + kx)) runs in (P/S)^2 tap groups; one group
//                           holds one tap of each pixel-parity class, so no two threads touch a
//                           pixel inside a group, and every pixel sums its contributions in the
//                           same fixed order (blocks in order, groups in order) -- deterministic,
//                           no atomics.  After the image's last block: the residual
//                           r = x - recon with a zero border of E pixels and rows padded to RP
//                           floats (the layout kernel P bulk-copies its windows from); the image
//                           buffer is then cleared.
// Hand-offs (mbarriers): full (armed with the stage's bytes) / empty (the MMA commit) per stage,
// accFull / accEmpty per accumulator, xFull / xEmpty per x buffer.  Waits are bounded; a timeout
// raises the abort flag, the roles drain their copies and MMAs in flight, and the kernel reports
// through *err.
// -------------------------------------------------------------------------------------------
constexpr int kMaxRStages = 4;

struct ReconPlan {
   int G;              // persistent CTAs
   int nStage;         // A + W^T ring stages
   int RP, rowsPad;    // padded residual rows
   uint32_t stageBytes, offRec, offX[2];
   uint32_t xStride;   // offX[1] - offX[0] (kernels index slots arithmetically, not through the array)
   uint32_t total;
};

template <int S, int P, int C, bool X3>
__global__ void __launch_bounds__(320, 1)
      recon_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmAlo,
                      const __grid_constant__ CUtensorMap tmWtH, const __grid_constant__ CUtensorMap tmWtloH,
                      LcaGeom g, ReconPlan rp, const float *__restrict__ x, float *__restrict__ rpad,
                      int *__restrict__ err) {
   constexpr int KP = P * P * C;
   constexpr int E = (P - S) / 2;
   constexpr uint32_t BA = 128 * 64 * 2, BW = KP * 64 * 2;  // one A tile, one W^T tile
   constexpr uint32_t AB = (X3 ? 2 : 1) * BA;                 // A part of a stage (hi, lo)
   constexpr int FOLD = 256;                                  // fold threads (warps 0-7)
   static_assert(KP <= 256 && KP % 16 == 0, "one MMA N = P*P*C <= 256, halves of whole 8-row atoms");
   static_assert(S % 2 == 0, "the fold splits the patch rows of a stride in two halves");
   extern __shared__ uint8_t smem_raw[];
   uint8_t *smem = align1024(smem_raw);
   __shared__ __align__(8) uint64_t full[kMaxRStages], empty[kMaxRStages], accFull[2], accEmpty[2], xFull[2],
         xEmpty[2];
   __shared__ uint32_t tmemBase;
   __shared__ volatile int abortFlag;

   const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
   const int G = gridDim.x;
   const int myUnits = (int)blockIdx.x < g.nb ? (g.nb - 1 - (int)blockIdx.x) / G + 1 : 0;
   const int nkc = g.F / 64;
   const int nStage = rp.nStage;
   const int nPix = g.inNx * g.inNy * C;
   auto image_of = [&](int ui) { return (int)blockIdx.x + ui * G; };

   if (tid == 0) {
      for (int i = 0; i < kMaxRStages; i++) {
         mbar_init(&full[i], 1);
         mbar_init(&empty[i], 1);  // the MMA commit
      }
      for (int i = 0; i < 2; i++) {
         mbar_init(&accFull[i], 1);
         mbar_init(&accEmpty[i], 8);  // one arrival per fold warp
         mbar_init(&xFull[i], 1);
         mbar_init(&xEmpty[i], 1);
      }
      abortFlag = 0;
      fence_mbar_init();
   }
   if (warp == 0) tmem_alloc(&tmemBase, 512);
   tc_fence_before();
   __syncthreads();
   tc_fence_after();
   const uint32_t tmem = tmemBase;
   // Set-up above overlaps the previous kernel's tail; everything below reads A (written by the
   // previous kernel P) or writes the residual (read by it).
   griddep_launch_dependents();
   griddep_wait();

   auto wait_or_abort = [&](uint64_t *bar, uint32_t parity) {
      if (abortFlag) return false;
      if (mbar_wait(bar, parity)) return true;
      abortFlag = 1;
      return false;
   };
   auto last_use = [](int n, int sl, int slots) { return sl < n ? n - 1 - ((n - 1 - sl) % slots) : -1; };

   if (warp == 8) {
      // ============================== loads ==============================
      if (lane == 0 && myUnits > 0) {
         prefetch_tmap(&tmA);
         prefetch_tmap(&tmWtH);
         if (X3) {
            prefetch_tmap(&tmAlo);
            prefetch_tmap(&tmWtloH);
         }
         int issued = 0, xIssued = 0;
         bool ok = true;
         for (int ui = 0; ok && ui < myUnits; ui++) {
            const int b = image_of(ui);
            for (int mb = 0; ok && mb < g.MB; mb++) {
               const int rowA = b * g.Npos + mb * 128;
               for (int kc = 0; kc < nkc; kc++) {
                  const int j = issued, st = j % nStage, u = j / nStage;
                  if (u > 0 && !(ok = wait_or_abort(&empty[st], (uint32_t)((u - 1) & 1)))) break;
                  uint8_t *base = smem + st * rp.stageBytes;
                  mbar_arrive_expect_tx(&full[st], AB + (X3 ? 2u : 1u) * BW);
                  tma_load_2d(base, &tmA, &full[st], kc * 64, rowA);
                  if (X3) tma_load_2d(base + BA, &tmAlo, &full[st], kc * 64, rowA);
                  // the W^T tile as two boxes of KP/2 rows
#pragma unroll
                  for (int h = 0; h < 2; h++) {
                     tma_load_2d(base + AB + h * (BW / 2), &tmWtH, &full[st], kc * 64, h * (KP / 2));
                     if (X3) tma_load_2d(base + AB + BW + h * (BW / 2), &tmWtloH, &full[st], kc * 64, h * (KP / 2));
                  }
                  issued++;
               }
               if (ok && mb == 0) {
                  // the image's x, into buffer ui % 2 once the residual of unit ui-2 has read it
                  const int xb = ui & 1;
                  if (ui >= 2 && !(ok = wait_or_abort(&xEmpty[xb], (uint32_t)(((ui >> 1) - 1) & 1)))) break;
                  mbar_arrive_expect_tx(&xFull[xb], (uint32_t)nPix * 4);
                  bulk_load(smem + rp.offX[0] + xb * rp.xStride, x + (size_t)b * nPix, (uint32_t)nPix * 4,
                            &xFull[xb]);
                  xIssued = ui + 1;
               }
            }
         }
         if (!ok) {
            for (int sl = 0; sl < nStage; sl++) {
               const int u = last_use(issued, sl, nStage);
               if (u >= 0) mbar_wait(&full[sl], (uint32_t)((u / nStage) & 1));
            }
            for (int sl = 0; sl < 2; sl++) {
               const int u = last_use(xIssued, sl, 2);
               if (u >= 0) mbar_wait(&xFull[sl], (uint32_t)((u / 2) & 1));
            }
         }
      }
   } else if (warp == 9) {
      // ============================== MMA ==============================
      if (lane == 0 && myUnits > 0) {
         const uint32_t idesc = idesc_bf16(128, KP);
         int j = 0, blk = 0, mmaBlocks = 0;
         bool ok = true;
         for (int ui = 0; ok && ui < myUnits; ui++) {
            for (int mb = 0; ok && mb < g.MB; mb++) {
               const int a = blk & 1;
               if (blk >= 2 && !(ok = wait_or_abort(&accEmpty[a], (uint32_t)(((blk >> 1) - 1) & 1)))) break;
               const uint32_t d = tmem + a * 256;
               for (int kc = 0; kc < nkc; kc++, j++) {
                  const int st = j % nStage;
                  if (!(ok = wait_or_abort(&full[st], (uint32_t)((j / nStage) & 1)))) break;
                  tc_fence_after();
                  const uint32_t base = smem_u32(smem + st * rp.stageBytes);
                  const int npass = X3 ? 3 : 1;
                  for (int pass = 0; pass < npass; pass++) {
                     // hi x hi, then hi x lo(W), then lo(A) x hi
                     const uint32_t a0 = base + ((X3 && pass == 2) ? BA : 0);
                     const uint32_t w0 = base + AB + ((X3 && pass == 1) ? BW : 0);
#pragma unroll
                     for (int k = 0; k < 4; k++)
                        mma_bf16(d, sdesc_sw128(a0 + k * 32), sdesc_sw128(w0 + k * 32), idesc, (kc | pass | k) != 0);
                  }
                  mma_commit(&empty[st]);  // the stage is free once these MMAs are done
               }
               if (!ok) break;
               mma_commit(&accFull[a]);
               blk++;
               mmaBlocks = blk;
            }
         }
         if (!ok && mmaBlocks > 0) mbar_wait(&accFull[(mmaBlocks - 1) & 1], (uint32_t)(((mmaBlocks - 1) >> 1) & 1));
      }
   } else if (warp < 8) {
      // ============================== fold and residual (warps 0-7) ==============================
      // thread = (position p = tid % 128, row half hh = tid / 128): inside a tap group the
      // thread adds the taps of its position whose patch row parity dy lies in its half, so the
      // two halves touch different pixel rows and the pixels of a group stay disjoint.
      constexpr int DH = S / 2;  // patch rows per half
      float *recon = reinterpret_cast<float *>(smem + rp.offRec);
      for (int i = tid; i < nPix; i += FOLD) recon[i] = 0.0f;
      named_bar_sync(1, FOLD);
      const int p = tid & 127, hh = tid >> 7;
      int blk = 0;
      for (int ui = 0; ui < myUnits; ui++) {
         const int b = image_of(ui);
         bool stop = false;
         for (int mb = 0; mb < g.MB; mb++, blk++) {
            const int a = blk & 1;
            if (tid == 0) wait_or_abort(&accFull[a], (uint32_t)((blk >> 1) & 1));
            if ((stop = named_bar_or(1, FOLD, abortFlag != 0))) break;
            tc_fence_after();
            const uint32_t lanes = tmem + a * 256 + ((uint32_t)((warp & 3) * 32) << 16);
            const int pos = mb * 128 + p;
            const int y1 = pos / g.v1Nx, x1 = pos % g.v1Nx;
            const int py0 = S * y1 - E, px0 = S * x1 - E;
#pragma unroll 1
            for (int ty = 0; ty < P / S; ty++) {
               float rowv[DH][P * C];
#pragma unroll
               for (int dd = 0; dd < DH; dd++)
                  tmem_ld_cols<P * C>(lanes + (uint32_t)((S * ty + hh * DH + dd) * P * C), rowv[dd]);
               if (ty == P / S - 1) {
                  tc_fence_before();
                  if (lane == 0) mbar_arrive(&accEmpty[a]);  // this warp has read the accumulator
               }
#pragma unroll
               for (int tx = 0; tx < P / S; tx++) {
                  // the group's pixels of this thread: all loads, then all stores (they are
                  // distinct, so the adds need not wait on one another)
                  float old[DH][S][C];
                  bool in[DH][S];
#pragma unroll
                  for (int dd = 0; dd < DH; dd++) {
                     const int py = py0 + S * ty + hh * DH + dd;
#pragma unroll
                     for (int dx = 0; dx < S; dx++) {
                        const int px = px0 + S * tx + dx;
                        in[dd][dx] = py >= 0 && py < g.inNy && px >= 0 && px < g.inNx;
#pragma unroll
                        for (int c = 0; c < C; c++) old[dd][dx][c] = in[dd][dx] ? recon[(py * g.inNx + px) * C + c] : 0.0f;
                     }
                  }
#pragma unroll
                  for (int dd = 0; dd < DH; dd++) {
                     const int py = py0 + S * ty + hh * DH + dd;
#pragma unroll
                     for (int dx = 0; dx < S; dx++) {
                        const int px = px0 + S * tx + dx;
                        if (in[dd][dx]) {
#pragma unroll
                           for (int c = 0; c < C; c++)
                              recon[(py * g.inNx + px) * C + c] = old[dd][dx][c] + rowv[dd][(S * tx + dx) * C + c];
                        }
                     }
                  }
                  named_bar_sync(1, FOLD);
               }
            }
         }
         if (stop) break;
         // ---- residual of image b into the padded layout ----
         const int xb = ui & 1;
         if (tid == 0) wait_or_abort(&xFull[xb], (uint32_t)((ui >> 1) & 1));
         if (named_bar_or(1, FOLD, abortFlag != 0)) break;
         const float *xs = reinterpret_cast<const float *>(smem + rp.offX[0] + xb * rp.xStride);
         float *out = rpad + (size_t)b * rp.rowsPad * rp.RP;
         const int rowElems = g.inNx * C;
         // trip counts uniform across each warp (a divergent inner loop costs far more than
         // the predicated body)
         const int RPl = rp.RP, rowsPadl = rp.rowsPad, inNyl = g.inNy;
         for (int c0 = 0; c0 < RPl; c0 += 128) {
            const int col = c0 + p, j = col - E * C;
            const bool colIn = col < RPl, colX = j >= 0 && j < rowElems;
#pragma unroll 4
            for (int yp = hh; yp < rowsPadl; yp += 2) {
               const int ye = yp - E;
               float v = 0.0f;
               if (colX && ye >= 0 && ye < inNyl) v = __fadd_rn(xs[ye * rowElems + j], -recon[ye * rowElems + j]);
               if (colIn) out[(size_t)yp * RPl + col] = v;
            }
         }
         named_bar_sync(1, FOLD);
         if (tid == 0) mbar_arrive(&xEmpty[xb]);  // x buffer free for unit ui+2
         for (int i = tid; i < nPix; i += FOLD) recon[i] = 0.0f;
         named_bar_sync(1, FOLD);
      }
   }
   __syncthreads();
   if (tid == 0 && abortFlag) atomicExch(err, 1);
   tc_fence_before();
   __syncthreads();
   if (warp == 0) tmem_dealloc(tmem, 512);
}

// -------------------------------------------------------------------------------------------
// Kernel P: post-perspective delivery and the LCA update (persistent, warp-specialised)
//
// Tile: one image, 128 V1 positions, FT (<= 256) features, i.e. FT/64 blocks of 64 features.
// Grid: one CTA per SM walking tiles blockIdx.x, +G, ...  Three roles:
//   warp 8, lane 0 (loads):   the next tile's residual window (one bulk copy of RWR padded
//                             rows), each block's weight tile by TMA and its V chunk (32 KB,
//                             contiguous in the device layout of V) by one bulk copy, into
//                             rings of nW / nV slots;
//   warp 9, lane 0 (MMA):     per block one tcgen05.mma chain (M = 128, N = 64, K = P*P*C) into
//                             one of four TMEM accumulators;
//   warps 0-7 (epilogue):     the BF16 im2col operand of each tile's window (all 8 warps, placed
//                             inside the previous tile's blocks); per block, each warp on its
//                             own: TMEM lanes 32*(w%4).., features 32*(w/4).., the LCA update of
//                             V in place in its 32 x 32 part of the shared V chunk (a contiguous
//                             4 KB, bulk-stored back by the warp), A staged in shared memory
//                             and TMA-stored by the warp.
// Loads run up to nV blocks ahead of the epilogue, so several V chunks are in flight per SM.
// Hand-offs are full/empty mbarriers:
//   stFull / stEmpty   window landed / read by the im2col
//   imFull / imEmpty   im2col built / all MMAs of the tile done (tcgen05.commit)
//   wFull / wEmpty     weight slot landed / its MMAs done (tcgen05.commit)
//   vFull / vEmpty     V slot landed / updated and read out by the 8 warps' stores
//   accFull / accEmpty accumulator written (tcgen05.commit) / read by the 8 epilogue warps
// A warp releases a V slot when its store of the next block has been issued and the slot's
// own store has read shared memory (one store in flight per warp); with a single slot it
// waits for the read at once.
// Every wait is bounded; a timeout raises a shared abort flag that every role checks, the
// roles drain their own copies and MMAs in flight, and the kernel reports through *err.
// -------------------------------------------------------------------------------------------
constexpr int kPostNT = 64;
constexpr int kMaxVSlots = 3, kMaxWSlots = 2;
constexpr int kAcc = 4;  // TMEM accumulators (64 columns each): the MMAs run up to 4 blocks ahead

struct PostPlan {
   int G;                             // persistent CTAs
   int FT;                            // features per tile (multiple of 64, <= 256)
   int nV, nW;                        // ring slots for the per-block V tiles and weight tiles
   int RP, rowsPad;                   // padded residual: floats per row, rows per image
   uint32_t offIM, offIMlo;
   uint32_t offW[kMaxWSlots], offWlo[kMaxWSlots];
   uint32_t offVT[kMaxVSlots];
   uint32_t wStride;                  // offW[s+1] - offW[s]; V slots are 32 KB apart
   uint32_t offWin;                   // residual window, RWR rows x RP floats
   uint32_t offA;                     // A staging, 2 KB per epilogue warp (when stageA)
   int stageA;                        // A leaves through shared memory and TMA stores
   uint32_t total;                    // dynamic shared memory incl. alignment slack
};

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
   __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
   return *reinterpret_cast<uint32_t *>(&h);
}

// SIMPLE: the threshold is the plain shift (g.simple), compile-time so that the instance holds
// only the update code it runs
template <int S, int P, int C, bool X3, bool SIMPLE>
__global__ void __launch_bounds__(320, 1) post_tc_kernel(const __grid_constant__ CUtensorMap tmW,
                                                         const __grid_constant__ CUtensorMap tmWlo,
                                                         const __grid_constant__ CUtensorMap tmAst, LcaGeom g,
                                                         PostPlan pl, const float *__restrict__ rpad,
                                                         float *__restrict__ V,
                                                         bf16 *__restrict__ A, bf16 *__restrict__ Alo,
                                                         int *__restrict__ err) {
   constexpr int KP = P * P * C, NKC = KP / 64;
   constexpr uint32_t WBYTES = NKC * kPostNT * 128;
   constexpr int EPI = 256;  // epilogue threads (warps 0-7)
   static_assert((S * C) % 2 == 0, "window reads are 8-byte pairs");
   extern __shared__ uint8_t smem_raw[];
   uint8_t *smem = align1024(smem_raw);
   __shared__ __align__(8) uint64_t stFull, stEmpty, imFull, imEmpty, wFull[kMaxWSlots], wEmpty[kMaxWSlots],
         vFull[kMaxVSlots], vEmpty[kMaxVSlots], accFull[kAcc], accEmpty[kAcc];
   __shared__ uint32_t tmemBase;
   __shared__ volatile int abortFlag;

   const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
   const int nFH = g.F / pl.FT, nBlk = pl.FT / kPostNT;
   const int nTiles = g.nb * g.MB * nFH;
   const int myTiles = blockIdx.x < nTiles ? (nTiles - 1 - blockIdx.x) / pl.G + 1 : 0;
   const int Q = myTiles * nBlk;
   const int nV = pl.nV, nW = pl.nW;
   const int lagV = nV >= 2 ? nV - 1 : nV;  // blocks between a V slot's use and its release
   const int RWR = rwin_rows(S, P, g.rowsPerBlock);
   const int RP = pl.RP;

   if (tid == 0) {
      mbar_init(&stFull, 1);
      mbar_init(&stEmpty, 1);
      mbar_init(&imFull, 1);
      mbar_init(&imEmpty, 1);
      for (int i = 0; i < kMaxWSlots; i++) {
         mbar_init(&wFull[i], 1);
         mbar_init(&wEmpty[i], 1);
      }
      for (int i = 0; i < kMaxVSlots; i++) {
         mbar_init(&vFull[i], 1);
         mbar_init(&vEmpty[i], 8);  // one arrival per epilogue warp
      }
      for (int i = 0; i < kAcc; i++) {
         mbar_init(&accFull[i], 1);
         mbar_init(&accEmpty[i], 8);
      }
      abortFlag = 0;
      fence_mbar_init();
   }
   if (warp == 0) tmem_alloc(&tmemBase, kAcc * kPostNT);
   tc_fence_before();
   __syncthreads();
   tc_fence_after();
   const uint32_t tmem = tmemBase;
   // Set-up above overlaps the previous kernel's tail; everything below reads the residual
   // (written by the previous kernel R) or V and A (which kernel R and the previous kernel P use).
   griddep_launch_dependents();
   griddep_wait();

   auto tile_of = [&](int ti, int &b, int &mb, int &fh) {
      const int j = blockIdx.x + ti * pl.G;
      fh = j % nFH;
      const int r = j / nFH;
      mb = r % g.MB;
      b = r / g.MB;
   };
   auto wait_or_abort = [&](uint64_t *bar, uint32_t parity) {
      if (abortFlag) return false;
      if (mbar_wait(bar, parity)) return true;
      abortFlag = 1;
      return false;
   };
   // last block (< n issued) that used ring slot sl of a ring of `slots`, or -1
   auto last_use = [](int n, int sl, int slots) { return sl < n ? n - 1 - ((n - 1 - sl) % slots) : -1; };

   if (warp == 8) {
      // ============================== loads ==============================
      if (lane == 0 && Q > 0) {
         int rowsIssued = 0, wIssued = 0, vIssued = 0;
         const uint32_t winBytes = (uint32_t)(RWR * RP * 4);
         auto issue_rows = [&](int ti) {
            int b, mb, fh;
            tile_of(ti, b, mb, fh);
            // padded rows S*mb*rowsPerBlock .. +RWR hold error rows S*y0 - E .. +RWR
            const float *src = rpad + ((size_t)b * pl.rowsPad + (size_t)S * mb * g.rowsPerBlock) * RP;
            mbar_arrive_expect_tx(&stFull, winBytes);
            bulk_load(smem + pl.offWin, src, winBytes, &stFull);
            rowsIssued = ti + 1;
         };
         prefetch_tmap(&tmW);
         if (X3) prefetch_tmap(&tmWlo);
         if (pl.stageA) prefetch_tmap(&tmAst);
         bool ok = true;
         issue_rows(0);
         // block q = (tile ti, block nb), weight slot sw in its use uw, V slot sv in its use uv:
         // stepped, not divided
         int ti = 0, nb = 0, sw = 0, uw = 0, sv = 0, uv = 0, b = 0, mb = 0, fh = 0;
         tile_of(0, b, mb, fh);
         for (int q = 0; ok && q < Q; q++) {
            // tile t+1's window goes out once tile t's has been read, before the first load that
            // waits for tile t's epilogue (V slot) or MMAs (weight slot): that load could not
            // start earlier anyway, and a later issue would leave the epilogue without a window
            while (ok && rowsIssued < myTiles && (rowsIssued - 1) * nBlk + (lagV < nW ? lagV : nW) <= q) {
               ok = wait_or_abort(&stEmpty, (uint32_t)((rowsIssued - 1) & 1));
               if (ok) issue_rows(rowsIssued);
            }
            if (!ok) break;
            const int f0 = fh * pl.FT + nb * kPostNT;
            if (uw > 0 && !(ok = wait_or_abort(&wEmpty[sw], (uint32_t)((uw - 1) & 1)))) break;
            mbar_arrive_expect_tx(&wFull[sw], (X3 ? 2 : 1) * WBYTES);
            for (int kc = 0; kc < NKC; kc++) {
               const uint32_t wo = sw * pl.wStride + kc * kPostNT * 128;
               tma_load_2d(smem + pl.offW[0] + wo, &tmW, &wFull[sw], kc * 64, f0);
               if (X3) tma_load_2d(smem + pl.offWlo[0] + wo, &tmWlo, &wFull[sw], kc * 64, f0);
            }
            wIssued = q + 1;
            if (uv > 0 && !(ok = wait_or_abort(&vEmpty[sv], (uint32_t)((uv - 1) & 1)))) break;
            mbar_arrive_expect_tx(&vFull[sv], 32768);
            bulk_load(smem + pl.offVT[0] + sv * 32768u, V + v_index(g, b, mb * 128, f0), 32768, &vFull[sv]);
            vIssued = q + 1;
            if (++sw == nW) {
               sw = 0;
               uw++;
            }
            if (++sv == nV) {
               sv = 0;
               uv++;
            }
            if (++nb == nBlk) {
               nb = 0;
               if (++ti < myTiles) tile_of(ti, b, mb, fh);
            }
         }
         while (ok && rowsIssued < myTiles) {
            ok = wait_or_abort(&stEmpty, (uint32_t)((rowsIssued - 1) & 1));
            if (ok) issue_rows(rowsIssued);
         }
         if (!ok) {
            // the copies still in flight land before shared memory goes away
            mbar_wait(&stFull, (uint32_t)((rowsIssued - 1) & 1));
            for (int sl = 0; sl < nW; sl++) {
               const int u = last_use(wIssued, sl, nW);
               if (u >= 0) mbar_wait(&wFull[sl], (uint32_t)((u / nW) & 1));
            }
            for (int sl = 0; sl < nV; sl++) {
               const int u = last_use(vIssued, sl, nV);
               if (u >= 0) mbar_wait(&vFull[sl], (uint32_t)((u / nV) & 1));
            }
         }
      }
   } else if (warp == 9) {
      // ============================== MMA ==============================
      if (lane == 0 && Q > 0) {
         int mmaDone = 0;
         bool ok = true;
         int ti = 0, nb = 0, sw = 0, uw = 0;
         for (int q = 0; ok && q < Q; q++) {
            const int a = q & (kAcc - 1);
            if (nb == 0 && !(ok = wait_or_abort(&imFull, (uint32_t)(ti & 1)))) break;
            if (!(ok = wait_or_abort(&wFull[sw], (uint32_t)(uw & 1)))) break;
            if (q >= kAcc && !(ok = wait_or_abort(&accEmpty[a], (uint32_t)((q / kAcc - 1) & 1)))) break;
            tc_fence_after();
            const uint32_t idesc = idesc_bf16(128, kPostNT);
            const uint32_t d = tmem + a * kPostNT;
            const int npass = X3 ? 3 : 1;
            for (int pass = 0; pass < npass; pass++) {
               const uint32_t a0 = smem_u32(smem + ((X3 && pass == 2) ? pl.offIMlo : pl.offIM));
               const uint32_t w0 = smem_u32(smem + ((X3 && pass == 1) ? pl.offWlo[0] : pl.offW[0]) + sw * pl.wStride);
               for (int kc = 0; kc < NKC; kc++)
#pragma unroll
                  for (int k = 0; k < 4; k++)
                     mma_bf16(d, sdesc_sw128(a0 + kc * 16384 + k * 32), sdesc_sw128(w0 + kc * kPostNT * 128 + k * 32),
                              idesc, (pass | kc | k) != 0);
            }
            mma_commit(&accFull[a]);
            mma_commit(&wEmpty[sw]);
            if (nb == nBlk - 1) mma_commit(&imEmpty);
            mmaDone = q + 1;
            if (++sw == nW) {
               sw = 0;
               uw++;
            }
            if (++nb == nBlk) {
               nb = 0;
               ti++;
            }
         }
         // MMAs still in flight finish before shared memory and TMEM go away
         if (!ok && mmaDone > 0) mbar_wait(&accFull[(mmaDone - 1) % kAcc], (uint32_t)(((mmaDone - 1) / kAcc) & 1));
      }
   } else {
      // ============================== epilogue (warps 0-7) ==============================
      const float *win = reinterpret_cast<const float *>(smem + pl.offWin);
      const int qd = warp & 3, h = warp >> 2;
      const int pw = 32 * qd + lane;  // this thread's position (TMEM lane) in the epilogue
      int pendingV = -1;              // V slot whose store this warp has in flight
      // im2col of tile t: all 8 warps, between two named barriers.  A warp whose own wait failed
      // skips its block work until the next im2col, whose first barrier sees the abort flag in
      // that warp, so that every warp leaves together (no warp skips a barrier).
      auto im2col = [&](int t) {
         if (tid == 0 && wait_or_abort(&stFull, (uint32_t)(t & 1)) && t > 0)
            wait_or_abort(&imEmpty, (uint32_t)((t - 1) & 1));  // the previous tile's MMAs are done
         if (named_bar_or(1, EPI, abortFlag != 0)) return false;
            // ---- BF16 im2col of the window (row runs of P*C elements, read in pairs) ----
            {
               constexpr int RUN = P * C;
               constexpr int CPR = RUN / 8;
               static_assert(RUN % 8 == 0, "patch rows must fill whole 16-byte chunks");
               const int p = tid & 127, half = tid >> 7;
               const int yl = p / g.v1Nx, x1 = p % g.v1Nx;
               const float *src0 = win + (S * yl) * RP + S * x1 * C;
   #pragma unroll 1
               for (int ky = half * (P / 2); ky < (half + 1) * (P / 2); ky++) {
                  const float2 *src = reinterpret_cast<const float2 *>(src0 + ky * RP);
   #pragma unroll
                  for (int cc = 0; cc < CPR; cc++) {
                     float vals[8];
   #pragma unroll
                     for (int jj = 0; jj < 4; jj++) {
                        const float2 t = src[cc * 4 + jj];
                        vals[2 * jj] = t.x;
                        vals[2 * jj + 1] = t.y;
                     }
                     uint4 hi;
                     hi.x = pack2(vals[0], vals[1]);
                     hi.y = pack2(vals[2], vals[3]);
                     hi.z = pack2(vals[4], vals[5]);
                     hi.w = pack2(vals[6], vals[7]);
                     const int c8 = ky * CPR + cc;
                     const uint32_t off = (c8 >> 3) * 16384 + sw128_offset(p, (c8 & 7) * 8);
                     *reinterpret_cast<uint4 *>(smem + pl.offIM + off) = hi;
                     if (X3) {
                        const __nv_bfloat162 *h2 = reinterpret_cast<const __nv_bfloat162 *>(&hi);
                        float2 f01 = __bfloat1622float2(h2[0]), f23 = __bfloat1622float2(h2[1]);
                        float2 f45 = __bfloat1622float2(h2[2]), f67 = __bfloat1622float2(h2[3]);
                        uint4 lo;
                        lo.x = pack2(vals[0] - f01.x, vals[1] - f01.y);
                        lo.y = pack2(vals[2] - f23.x, vals[3] - f23.y);
                        lo.z = pack2(vals[4] - f45.x, vals[5] - f45.y);
                        lo.w = pack2(vals[6] - f67.x, vals[7] - f67.y);
                        *reinterpret_cast<uint4 *>(smem + pl.offIMlo + off) = lo;
                     }
                  }
               }
            }
         fence_proxy_async_smem();
         named_bar_sync(1, EPI);
         if (tid == 0) {
            mbar_arrive(&imFull);
            mbar_arrive(&stEmpty);  // the window is read: the next tile's may land
         }
         return true;
      };
      // The next tile's im2col goes in after block kIm of the current one: late enough that the
      // loads of the current tile's remaining blocks are out and its MMAs (up to 4 blocks ahead)
      // have released the operand, early enough that the next tile's MMAs run before its blocks.
      int kIm = nBlk - 1 - lagV;
      if (kIm < 1) kIm = 1;
      if (kIm > nBlk - 1) kIm = nBlk - 1;
      bool go = myTiles > 0 && im2col(0), dead = false;
      int ti = 0, nb = 0, sv = 0, uv = 0, b = 0, mb = 0, fh = 0;  // stepped, not divided
      if (myTiles > 0) tile_of(0, b, mb, fh);
      for (int q = 0; go && q < Q; q++) {
         // ---- block q, each warp on its own ----
         const int a = q & (kAcc - 1);
         const int f0 = fh * pl.FT + nb * kPostNT, rowV = b * g.Npos + mb * 128;
         int okw = !dead;
         if (lane == 0 && okw)
            okw = wait_or_abort(&accFull[a], (uint32_t)((q / kAcc) & 1)) &&
                  wait_or_abort(&vFull[sv], (uint32_t)(uv & 1));
         okw = __shfl_sync(0xffffffffu, okw, 0);
         dead = !okw;
         if (okw) {
            tc_fence_after();
            float d[32], vo[32];
            tmem_ld32(tmem + a * kPostNT + ((uint32_t)(32 * qd) << 16) + 32 * h, d);
            tc_fence_before();
            if (lane == 0) mbar_arrive(&accEmpty[a]);  // this warp is done with the accumulator
            uint8_t *vsub = smem + pl.offVT[0] + sv * 32768u + h * 16384 + 32 * qd * 128;  // this warp's 32 x 32 part
            uint8_t *vt = vsub + lane * 128;
#pragma unroll
            for (int qq = 0; qq < 8; qq++) {
               const float4 t = *reinterpret_cast<const float4 *>(vt + ((qq ^ (pw & 7)) << 4));
               vo[4 * qq] = t.x;
               vo[4 * qq + 1] = t.y;
               vo[4 * qq + 2] = t.z;
               vo[4 * qq + 3] = t.w;
            }
            float vn[32], an[32];
            const float om = 1.0f - g.e;
            if constexpr (SIMPLE) {  // AMax = +inf, VWidth = 0: A = V < VThresh ? AMin : V - AShift
               // element pairs on the packed FP32 pipe: t = d + si*ao, t = om*t, v = e*v + t
               const float2 si2 = make_float2(g.si, g.si), om2 = make_float2(om, om), e2 = make_float2(g.e, g.e);
#pragma unroll
               for (int jj = 0; jj < 32; jj += 2) {
                  const float ao0 = vo[jj] < g.VThresh ? g.AMin : vo[jj] - g.AShift;
                  const float ao1 = vo[jj + 1] < g.VThresh ? g.AMin : vo[jj + 1] - g.AShift;
                  float2 t = __ffma2_rn(si2, make_float2(ao0, ao1), make_float2(d[jj], d[jj + 1]));
                  t = __fmul2_rn(om2, t);
                  const float2 v2 = __ffma2_rn(e2, make_float2(vo[jj], vo[jj + 1]), t);
                  vn[jj] = v2.x;
                  vn[jj + 1] = v2.y;
                  an[jj] = vn[jj] < g.VThresh ? g.AMin : vn[jj] - g.AShift;
                  an[jj + 1] = vn[jj + 1] < g.VThresh ? g.AMin : vn[jj + 1] - g.AShift;
               }
            } else {
#pragma unroll
               for (int jj = 0; jj < 32; jj++) {
                  vn[jj] = fmaf(g.e, vo[jj], om * (d[jj] + g.si * thresh(vo[jj], g)));
                  an[jj] = thresh(vn[jj], g);
               }
            }
            // this warp's previous stores have read shared memory: their V slot goes back to the
            // loads warp, and the A staging buffer may be rewritten
            if (lane == 0 && pendingV >= 0) {
               bulk_wait_read_all();
               mbar_arrive(&vEmpty[pendingV]);
            }
            __syncwarp();
#pragma unroll
            for (int qq = 0; qq < 8; qq++)
               *reinterpret_cast<float4 *>(vt + ((qq ^ (pw & 7)) << 4)) =
                     make_float4(vn[4 * qq], vn[4 * qq + 1], vn[4 * qq + 2], vn[4 * qq + 3]);
            uint8_t *abuf = smem + pl.offA + warp * 2048;  // 32 rows x 64 B, 64-byte swizzle
            if (pl.stageA) {
#pragma unroll
               for (int c = 0; c < 4; c++)
                  *reinterpret_cast<uint4 *>(abuf + lane * 64 + ((c ^ ((lane >> 1) & 3)) << 4)) =
                        make_uint4(pack2(an[8 * c], an[8 * c + 1]), pack2(an[8 * c + 2], an[8 * c + 3]),
                                   pack2(an[8 * c + 4], an[8 * c + 5]), pack2(an[8 * c + 6], an[8 * c + 7]));
            } else {
               bf16 *ag = A + (size_t)(rowV + pw) * g.F + f0 + 32 * h;
#pragma unroll
               for (int t = 0; t < 2; t++)
                  st_global_32B(ag + 16 * t,
                                make_uint4(pack2(an[16 * t], an[16 * t + 1]), pack2(an[16 * t + 2], an[16 * t + 3]),
                                           pack2(an[16 * t + 4], an[16 * t + 5]), pack2(an[16 * t + 6], an[16 * t + 7])),
                                make_uint4(pack2(an[16 * t + 8], an[16 * t + 9]), pack2(an[16 * t + 10], an[16 * t + 11]),
                                           pack2(an[16 * t + 12], an[16 * t + 13]),
                                           pack2(an[16 * t + 14], an[16 * t + 15])));
            }
            if (X3) {
               uint4 *lg = reinterpret_cast<uint4 *>(Alo + (size_t)(rowV + pw) * g.F + f0 + 32 * h);
#pragma unroll
               for (int t = 0; t < 4; t++) {
                  float l[8];
#pragma unroll
                  for (int u = 0; u < 8; u++) l[u] = an[8 * t + u] - __bfloat162float(__float2bfloat16_rn(an[8 * t + u]));
                  lg[t] = make_uint4(pack2(l[0], l[1]), pack2(l[2], l[3]), pack2(l[4], l[5]), pack2(l[6], l[7]));
               }
            }
            fence_proxy_async_smem();
            __syncwarp();
            if (lane == 0) {
               bulk_store(V + v_index(g, b, mb * 128 + 32 * qd, f0 + 32 * h), vsub, 4096);
               if (pl.stageA) tma_store_2d(&tmAst, abuf, f0 + 32 * h, rowV + 32 * qd);
               bulk_commit();
               if (nV == 1) {  // the only slot: release it as soon as the store has read it
                  bulk_wait_read_all();
                  mbar_arrive(&vEmpty[sv]);
               }
            }
            pendingV = nV == 1 ? -1 : sv;
         }
         if (nb == kIm && ti + 1 < myTiles) go = im2col(ti + 1);
         if (++sv == nV) {
            sv = 0;
            uv++;
         }
         if (++nb == nBlk) {
            nb = 0;
            if (++ti < myTiles) tile_of(ti, b, mb, fh);
         }
      }
      if (lane == 0) bulk_wait_all();
   }
   __syncthreads();
   if (tid == 0 && abortFlag) atomicExch(err, 1);
   tc_fence_before();
   __syncthreads();
   if (warp == 0) tmem_dealloc(tmem, kAcc * kPostNT);
}

// -------------------------------------------------------------------------------------------
// Kernel F: a whole BF16 LCA timestep in one launch -- kernel P's post delivery and update,
// then the reconstruction of the new activity, without the activity leaving the SM.
//
// Tile (image b, block mb of 128 positions, feature tile fh of FT features) as in kernel P.
// Per 64-feature block q of the tile: GEMM1 D1 = im2col(r) . W_q^T (the im2col operand in TMEM
// where it fits, else in shared memory), the update, then the block's new activity A_q (BF16,
// 128 positions x 64 features) goes into one of two TMEM A tiles and GEMM2 accumulates
// D2[pos][k] += sum_f A_q[pos][f] W_q[f][k] (N = P*P*C) in TMEM, reading the block's weight
// tile again as an MN-major operand.  After the tile's last GEMM2 the tile warps fold D2 into a
// band: padded rows S*mb*rpb .. +RWR (every row the block's patches reach), starting from x on
// the rows the block owns when fh == 0 and from 0 otherwise, each tap subtracted (kernel R's
// fold: tap groups in which no two threads touch one pixel, every pixel's taps in one fixed
// order).  The band goes to HBM.  Block mb owns padded rows S*mb*rpb .. S*(mb+1)*rpb - 1, the
// last block also the rows below; bands of blocks mb and mb + 1 overlap in P - S rows
// (P - S <= S*rpb).
// The next timestep's tile (b, mb) sums its residual window r = x - W^T a from the bands of
// (b, mb) and the overlapping rows of (b, mb - 1) and (b, mb + 1), all feature tiles: per
// pixel (sum over fh of the lower block's band) + (sum over fh of the upper block's band),
// so that both windows holding a pixel compute it in the same order.  The first timestep of
// a run reads kernel R's padded residual window instead (mode 0).
// Roles (736 threads):
//   warps 0-15 (epilogue): two groups of eight on alternating 64-feature blocks (group 0 the
//             even blocks of the CTA's sequence, group 1 the odd ones), so that the hand-off
//             chains of two blocks (accumulator, TMEM load, update, A into TMEM, V store) are
//             in flight at once.  Group g owns GEMM1 accumulator g, TMEM A tile g and V slots
//             g, g + 2 (the V ring has 2 or 4 slots, so each slot's phases are waited on by one
//             group only and an mbarrier's parity never stands for two phases).  Warp = (lane
//             quarter qd, 32-feature half hh): the update of its 32 positions x 32 features from
//             D1 and its 4 KB of the V chunk, V back in place and to HBM by its own bulk store,
//             A into the group's A tile once GEMM2 of the group's previous block has read it.
//             No named barrier: every hand-off is an mbarrier;
//   warps 16-19 (tile): named barrier 1.  Per tile t: the window of tile t + 1 summed from the
//             bands and its im2col (one position per thread, all P*P*C taps) once tile t's
//             last GEMM1 has read the operand; then tile t's fold: x of the owned rows (or 0)
//             into the stage, which tile t + 1's im2col has read, D2 folded in once tile t's
//             last GEMM2 is done, d2Empty as soon as D2 is read, the band stored;
//   warp 20 (weights): each block's weight tile by TMA into a 2- to 4-slot ring;
//   warp 21 (MMA):     an event loop issuing GEMM1 of the next block as soon as its weight
//             tile, accumulator and im2col operand are ready, and GEMM2 of the oldest block
//             whose A tile is written (the first GEMM2 of a tile also once the fold of the tile
//             before has read D2); a weight slot is freed by GEMM2's commit;
//   warp 22 (V, stage): an event loop: V chunks by bulk copy into the ring as slots free, and
//             tile t's bands (or residual window) as one stage once tile t - 1's im2col has
//             read the stage and tile t - 2's fold (which runs in the stage) is stored.
// Every wait is bounded (a wait that gives up sets the abort flag; the tile warps decide at
// barriers that OR the flag, so all four leave together; the other roles skip their work).
// -------------------------------------------------------------------------------------------
struct FusePlan {
   int G;                         // persistent CTAs
   int FT;                        // features per tile (multiple of 64)
   int nV, nW;                    // V (2 or 4) and weight (2..4) ring slots
   int RP, rowsPad, RWR;          // padded rows: floats per row, rows per image, rows per band
   uint32_t bandFloats, sliceFloats;
   uint32_t offIM, offW[4], offVT[4], offStage, offTop, offBot, offFold;
   uint32_t wStride;              // offW[s+1] - offW[s]; V slots are 32 KB apart
   uint32_t total;
};

constexpr int kFuseThreads = 736;

// SIMPLE: the threshold is the plain shift (g.simple); WRITEA: the launch also writes A and its
// low half for the kernels of a later unfused step.  Compile-time, so that each instance holds
// only the epilogue code it runs (the roles' code competes for the instruction cache).
template <int S, int P, int C, bool SIMPLE, bool WRITEA>
__global__ void __launch_bounds__(kFuseThreads, 1)
      step_tc_kernel(const __grid_constant__ CUtensorMap tmW, LcaGeom g, FusePlan fp, int mode,
                     const float *__restrict__ rin, float *__restrict__ bandsOut, const float *__restrict__ xpad,
                     float *__restrict__ V, bf16 *__restrict__ A, bf16 *__restrict__ Alo, int *__restrict__ err) {
   constexpr int KP = P * P * C, NKC = KP / 64;
   constexpr uint32_t WBYTES = NKC * kPostNT * 128;
   constexpr int EW = 16;                    // epilogue warps: two groups of eight
   constexpr int GW = EW / 2;                // warps per group
   constexpr int TW = 16, TT = 128;          // tile warps 16-19 (named barrier 1, 128 threads)
   constexpr int WW = 20, MW = 21, LW = 22;  // weights, MMA, V / stage loads
   static_assert(kFuseThreads == 32 * (LW + 1), "one thread per role slot");
   constexpr int kMaxW = 4, kMaxVF = 4;
   // TMEM columns: two GEMM1 accumulators, D2 (KP), two A tiles of GEMM2 (64 BF16 = 32 columns
   // each) and, where it fits, the im2col operand of GEMM1 (KP BF16 = KP / 2 columns) -- the
   // MMAs then read both A operands from TMEM, not shared memory
   constexpr int kAccF = 2;
   constexpr uint32_t colD2 = kAccF * kPostNT, colA = colD2 + KP, colIM = colA + 64;
   constexpr bool IMT = colIM + KP / 2 <= 512;
   static_assert(P % S == 0, "the fold's tap groups tile the patch");
   static_assert((S * C) % 2 == 0, "window reads are 8-byte pairs");
   static_assert(KP % 16 == 0 && KP <= 256, "GEMM2 is one MMA of N = P*P*C");
   // the fold holds FD patch rows of D2 in registers per round (all S of a tap group, or half)
   constexpr int FH = S * P * C <= 48 ? 1 : 2, FD = S / FH;
   static_assert(S % FH == 0, "fold halves");
   extern __shared__ uint8_t smem_raw[];
   uint8_t *smem = align1024(smem_raw);
   __shared__ __align__(8) uint64_t stFull, stEmpty, imFull, imEmpty, wFull[kMaxW], wEmpty[kMaxW], vFull[kMaxVF],
         vEmpty[kMaxVF], accFull[kAccF], accEmpty[kAccF], aFull[2], aEmpty[2], d2Full, d2Empty, foldFree, xFull,
         drain;
   __shared__ uint32_t tmemBase;
   __shared__ volatile int abortFlag;

   const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
   const int nFH = g.F / fp.FT, nBlk = fp.FT / kPostNT;
   const int nTiles = g.nb * g.MB * nFH;
   const int myTiles = blockIdx.x < nTiles ? (nTiles - 1 - blockIdx.x) / fp.G + 1 : 0;
   const int Q = myTiles * nBlk;
   const int nV = fp.nV, nW = fp.nW;
   const int RWR = fp.RWR, RP = fp.RP, rpb = g.rowsPerBlock;
   const uint32_t bandBytes = fp.bandFloats * 4u, sliceBytes = fp.sliceFloats * 4u;
   auto owned_rows = [&](int mb) { return mb == g.MB - 1 ? RWR : S * rpb; };

   if (tid == 0) {
      mbar_init(&stFull, 1);
      mbar_init(&stEmpty, 1);
      mbar_init(&imFull, 1);
      mbar_init(&imEmpty, 1);
      for (int i = 0; i < kMaxW; i++) {
         mbar_init(&wFull[i], 1);
         mbar_init(&wEmpty[i], 1);
      }
      for (int i = 0; i < kMaxVF; i++) {
         mbar_init(&vFull[i], 1);
         mbar_init(&vEmpty[i], GW);  // one arrival per warp of the slot's group (its store has read it)
      }
      for (int i = 0; i < kAccF; i++) {
         mbar_init(&accFull[i], 1);
         mbar_init(&accEmpty[i], GW);
      }
      // one full / empty pair per TMEM A tile (= per group)
      for (int i = 0; i < 2; i++) {
         mbar_init(&aFull[i], GW);
         mbar_init(&aEmpty[i], 1);
      }
      mbar_init(&d2Full, 1);
      mbar_init(&d2Empty, TT / 32);  // one arrival per tile warp (its D2 reads are done)
      mbar_init(&foldFree, 1);
      mbar_init(&xFull, 1);
      mbar_init(&drain, 1);
      abortFlag = 0;
      fence_mbar_init();
   }
   if (warp == 0) tmem_alloc(&tmemBase, 512);
   tc_fence_before();
   __syncthreads();
   tc_fence_after();
   const uint32_t tmem = tmemBase;
   const uint32_t tmemD2 = tmem + colD2;
   // Set-up above overlaps the previous kernel's tail; everything below reads the bands or the
   // residual (written by the previous launch) or V (which the previous launch writes).
   griddep_launch_dependents();
   griddep_wait();

   auto tile_of = [&](int ti, int &b, int &mb, int &fh) {
      const int j = blockIdx.x + ti * fp.G;
      fh = j % nFH;
      const int r = j / nFH;
      mb = r % g.MB;
      b = r / g.MB;
   };
   auto wait_or_abort = [&](uint64_t *bar, uint32_t parity) {
      if (abortFlag) return false;
      if (mbar_wait(bar, parity)) return true;
      abortFlag = 1;
      return false;
   };
   // an event loop's idle policy: after the wait limit with nothing ready, give up (abort flag)
   auto idle_step = [&](uint32_t &idle, uint64_t &idleSince) {
      if (abortFlag) return false;
      if (idle == 0) idleSince = global_ns();
      if ((++idle & 255) == 0 && global_ns() - idleSince > kWaitNs) {
         abortFlag = 1;
         return false;
      }
      if (idle > 16) __nanosleep(32);  // leave the issue slots to the epilogue warps on this sub-partition
      return true;
   };
   auto last_use = [](int n, int sl, int slots) { return sl < n ? n - 1 - ((n - 1 - sl) % slots) : -1; };
   auto band_in = [&](int b, int mb, int fh) {
      return rin + (((size_t)b * g.MB + mb) * nFH + fh) * fp.bandFloats;
   };

   if (warp == WW) {
      // ============================== weight loads ==============================
      if (lane == 0 && Q > 0) {
         prefetch_tmap(&tmW);
         int wIssued = 0;
         bool ok = true;
         int ti = 0, nb = 0, sw = 0, uw = 0, b = 0, mb = 0, fh = 0;
         tile_of(0, b, mb, fh);
         for (int q = 0; ok && q < Q; q++) {
            const int f0 = fh * fp.FT + nb * kPostNT;
            if (uw > 0 && !(ok = wait_or_abort(&wEmpty[sw], (uint32_t)((uw - 1) & 1)))) break;
            mbar_arrive_expect_tx(&wFull[sw], WBYTES);
            for (int kc = 0; kc < NKC; kc++)
               tma_load_2d(smem + fp.offW[0] + sw * fp.wStride + kc * kPostNT * 128, &tmW, &wFull[sw], kc * 64, f0);
            wIssued = q + 1;
            if (++sw == nW) {
               sw = 0;
               uw++;
            }
            if (++nb == nBlk) {
               nb = 0;
               if (++ti < myTiles) tile_of(ti, b, mb, fh);
            }
         }
         if (!ok) {  // the copies still in flight land before shared memory goes away
            for (int sl = 0; sl < nW; sl++) {
               const int u = last_use(wIssued, sl, nW);
               if (u >= 0) mbar_wait(&wFull[sl], (uint32_t)((u / nW) & 1));
            }
         }
      }
   } else if (warp == LW) {
      // ============================== V and stage loads ==============================
      if (lane == 0 && Q > 0) {
         auto issue_stage = [&](int ti) {
            int b, mb, fh;
            tile_of(ti, b, mb, fh);
            uint8_t *st = smem + fp.offStage;
            if (mode == 0) {
               // kernel R's padded residual: rows S*mb*rpb .. +RWR of image b
               const float *src = rin + ((size_t)b * fp.rowsPad + (size_t)S * mb * rpb) * RP;
               mbar_arrive_expect_tx(&stFull, bandBytes);
               bulk_load(st, src, bandBytes, &stFull);
            } else {
               const uint32_t bytes = nFH * bandBytes + (mb > 0 ? nFH * sliceBytes : 0u) +
                                      (mb < g.MB - 1 ? nFH * sliceBytes : 0u);
               mbar_arrive_expect_tx(&stFull, bytes);
               for (int f = 0; f < nFH; f++) bulk_load(st + f * bandBytes, band_in(b, mb, f), bandBytes, &stFull);
               if (mb > 0)  // the upper neighbour's last P - S rows
                  for (int f = 0; f < nFH; f++)
                     bulk_load(smem + fp.offTop + f * sliceBytes, band_in(b, mb - 1, f) + (size_t)S * rpb * RP,
                               sliceBytes, &stFull);
               if (mb < g.MB - 1)  // the lower neighbour's first P - S rows
                  for (int f = 0; f < nFH; f++)
                     bulk_load(smem + fp.offBot + f * sliceBytes, band_in(b, mb + 1, f), sliceBytes, &stFull);
            }
         };
         bool ok = true;
         int stNext = 0, vq = 0;
         int ti = 0, nb = 0, sv = 0, uv = 0, b = 0, mb = 0, fh = 0;
         tile_of(0, b, mb, fh);
         uint32_t idle = 0;
         uint64_t idleSince = 0;
         while (ok && (stNext < myTiles || vq < Q)) {
            bool did = false;
            // stage t once tile t - 1's im2col has read the stage and tile t - 2's fold (which
            // runs in the stage after that im2col) has been stored
            if (stNext < myTiles && (stNext == 0 || mbar_test(&stEmpty, (uint32_t)((stNext - 1) & 1))) &&
                (stNext < 2 || mbar_test(&foldFree, (uint32_t)((stNext - 2) & 1)))) {
               issue_stage(stNext++);
               did = true;
            }
            // V chunk vq once its slot's previous chunk has been stored by its group
            if (vq < Q && (uv == 0 || mbar_test(&vEmpty[sv], (uint32_t)((uv - 1) & 1)))) {
               const int f0 = fh * fp.FT + nb * kPostNT;
               mbar_arrive_expect_tx(&vFull[sv], 32768);
               bulk_load(smem + fp.offVT[0] + sv * 32768u, V + v_index(g, b, mb * 128, f0), 32768, &vFull[sv]);
               vq++;
               if (++sv == nV) {
                  sv = 0;
                  uv++;
               }
               if (++nb == nBlk) {
                  nb = 0;
                  if (++ti < myTiles) tile_of(ti, b, mb, fh);
               }
               did = true;
            }
            if (did)
               idle = 0;
            else
               ok = idle_step(idle, idleSince);
         }
         if (!ok) {
            // the copies still in flight land before shared memory goes away (a stage is issued
            // only after the one before it has landed and been read)
            if (stNext > 0) mbar_wait(&stFull, (uint32_t)((stNext - 1) & 1));
            for (int sl = 0; sl < nV; sl++) {
               const int u = last_use(vq, sl, nV);
               if (u >= 0) mbar_wait(&vFull[sl], (uint32_t)((u / nV) & 1));
            }
         }
      }
   } else if (warp == MW) {
      // ============================== MMA ==============================
      // An event loop over two in-order streams: GEMM1 of block g1 as soon as its weight tile,
      // its accumulator and (first block of a tile) the im2col operand are ready; GEMM2 of
      // block g2 < g1 as soon as the epilogue has written its A tile (and, first block of a
      // tile, the fold of the tile before has read D2).  GEMM1 of the next block therefore
      // never waits behind GEMM2 of an earlier one.  Polls never suspend; the loop ends when
      // nothing has been ready for the wait limit's time (or on the abort flag).
      if (lane == 0 && Q > 0) {
         const uint32_t idesc1 = idesc_bf16(128, kPostNT), idesc2 = idesc_bf16_bmn(128, KP);
         bool ok = true;
         int issued = 0;
         int g1 = 0, ti1 = 0, nb1 = 0, sw1 = 0, uw1 = 0;
         int g2 = 0, ti2 = 0, nb2 = 0, sw2 = 0;
         uint32_t idle = 0;
         uint64_t idleSince = 0;
         while (ok && g2 < Q) {
            bool did = false;
            if (g1 < Q) {
               const int a = g1 & (kAccF - 1);
               if ((nb1 != 0 || mbar_test(&imFull, (uint32_t)(ti1 & 1))) && mbar_test(&wFull[sw1], (uint32_t)(uw1 & 1)) &&
                   (g1 < kAccF || mbar_test(&accEmpty[a], (uint32_t)((g1 / kAccF - 1) & 1)))) {
                  tc_fence_after();
                  const uint32_t d = tmem + a * kPostNT;
                  const uint32_t w0 = smem_u32(smem + fp.offW[0] + sw1 * fp.wStride);
                  for (int kc = 0; kc < NKC; kc++)
#pragma unroll
                     for (int k = 0; k < 4; k++) {
                        const uint64_t bd = sdesc_sw128(w0 + kc * kPostNT * 128 + k * 32);
                        if constexpr (IMT)
                           mma_bf16_ta(d, tmem + colIM + 32 * kc + 8 * k, bd, idesc1, (kc | k) != 0);
                        else
                           mma_bf16(d, sdesc_sw128(smem_u32(smem + fp.offIM) + kc * 16384 + k * 32), bd, idesc1,
                                    (kc | k) != 0);
                     }
                  mma_commit(&accFull[a]);
                  if (nb1 == nBlk - 1) mma_commit(&imEmpty);
                  issued++;
                  g1++;
                  if (++sw1 == nW) {
                     sw1 = 0;
                     uw1++;
                  }
                  if (++nb1 == nBlk) {
                     nb1 = 0;
                     ti1++;
                  }
                  did = true;
               }
            }
            if (g2 < g1 && mbar_test(&aFull[g2 & 1], (uint32_t)((g2 >> 1) & 1)) &&
                (nb2 != 0 || ti2 == 0 || mbar_test(&d2Empty, (uint32_t)((ti2 - 1) & 1)))) {
               // GEMM2 of block g2: its A tile (TMEM) times its weight tile read MN-major
               tc_fence_after();
               const uint32_t w0 = smem_u32(smem + fp.offW[0] + sw2 * fp.wStride);
               const uint32_t at = tmem + colA + 32 * (g2 & 1);
#pragma unroll
               for (int k = 0; k < 4; k++)
                  mma_bf16_ta(tmemD2, at + 8 * k, sdesc_sw128_mn(w0 + k * 2048, kPostNT * 128), idesc2,
                              (nb2 | k) != 0);
               mma_commit(&aEmpty[g2 & 1]);
               mma_commit(&wEmpty[sw2]);
               if (nb2 == nBlk - 1) mma_commit(&d2Full);
               g2++;
               if (++sw2 == nW) sw2 = 0;
               if (++nb2 == nBlk) {
                  nb2 = 0;
                  ti2++;
               }
               did = true;
            }
            if (did)
               idle = 0;
            else
               ok = idle_step(idle, idleSince);
         }
         // MMAs still in flight finish before shared memory and TMEM go away
         if (!ok && issued > 0) {
            mma_commit(&drain);
            mbar_wait(&drain, 0);
         }
      }
   } else if (warp >= TW && warp < TW + TT / 32) {
      // ============================== tile warps (16-19) ==============================
      const int tt = tid - TW * 32;  // the position in the tile's 128-position block
      const int tq = warp & 3;       // TMEM lane quarter (= tt / 32)
      const float *win = reinterpret_cast<const float *>(smem + fp.offStage);
      float *fold = reinterpret_cast<float *>(smem + fp.offFold);
      const int yl = tt / g.v1Nx, xl = tt % g.v1Nx;
      // the residual window of tile t (summed from the bands in mode 1) and its BF16 im2col
      auto im2col = [&](int t) {
         if (tt == 0) wait_or_abort(&stFull, (uint32_t)(t & 1));
         if (named_bar_or(1, TT, abortFlag != 0)) return false;
         if (mode != 0) {
            // ---- the window from the bands (float4 runs: rows are RP floats, RP a multiple of
            // 4, so row r's run is [r * RP / 4, (r + 1) * RP / 4)) ----
            int b, mb, fh;
            tile_of(t, b, mb, fh);
            float4 *w4 = reinterpret_cast<float4 *>(smem + fp.offStage);
            const float4 *top4 = reinterpret_cast<const float4 *>(smem + fp.offTop);
            const float4 *bot4 = reinterpret_cast<const float4 *>(smem + fp.offBot);
            const int RP4 = RP / 4, bandF4 = (int)fp.bandFloats / 4, sliceF4 = (int)fp.sliceFloats / 4;
            const int nAll = RWR * RP4, topEnd = (P - S) * RP4, botStart = S * rpb * RP4;
            const bool hasTop = mb > 0, hasBot = mb < g.MB - 1;
            auto add4 = [](float4 a, float4 c) {
               return make_float4(__fadd_rn(a.x, c.x), __fadd_rn(a.y, c.y), __fadd_rn(a.z, c.z), __fadd_rn(a.w, c.w));
            };
            for (int i = tt; i < nAll; i += TT) {
               float4 v = w4[i];
               for (int f = 1; f < nFH; f++) v = add4(v, w4[f * bandF4 + i]);
               if (i < topEnd) {
                  if (hasTop) {  // the upper neighbour's rows first
                     float4 u = top4[i];
                     for (int f = 1; f < nFH; f++) u = add4(u, top4[f * sliceF4 + i]);
                     v = add4(u, v);
                  }
               } else if (i >= botStart && hasBot) {
                  const int j = i - botStart;
                  float4 u = bot4[j];
                  for (int f = 1; f < nFH; f++) u = add4(u, bot4[f * sliceF4 + j]);
                  v = add4(v, u);
               }
               w4[i] = v;
            }
         }
         // the operand is rewritten once tile t - 1's last GEMM1 has read it
         if (tt == 0 && t > 0) wait_or_abort(&imEmpty, (uint32_t)((t - 1) & 1));
         if (named_bar_or(1, TT, abortFlag != 0)) return false;
         const float *src0 = win + (S * yl) * RP + S * xl * C;
         if constexpr (IMT) {
            // ---- into TMEM: lane tt, K element k in column k / 2 ----
            constexpr int HALF = P * C / 2, COLS = KP / 2;
            static_assert((P * C) % 2 == 0 && COLS % 8 == 0, "im2col columns in groups of 8");
            tc_fence_after();
            const uint32_t t0 = tmem + ((uint32_t)(tq * 32) << 16) + colIM;
            uint32_t buf[8];
#pragma unroll
            for (int i = 0; i < COLS; i++) {
               const int ky = i / HALF, e = 2 * (i % HALF);
               const float2 t2 = *reinterpret_cast<const float2 *>(src0 + ky * RP + e);
               buf[i & 7] = pack2(t2.x, t2.y);
               if ((i & 7) == 7) tmem_st8(t0 + (i & ~7), buf);
            }
            tmem_wait_st();
            tc_fence_before();
         } else {
            // ---- into shared memory, K-major SW128 (as kernel P) ----
            constexpr int RUN = P * C;
            constexpr int CPR = RUN / 8;
            static_assert(RUN % 8 == 0, "patch rows must fill whole 16-byte chunks");
#pragma unroll 1
            for (int ky = 0; ky < P; ky++) {
               const float2 *src = reinterpret_cast<const float2 *>(src0 + ky * RP);
#pragma unroll
               for (int cc = 0; cc < CPR; cc++) {
                  float vals[8];
#pragma unroll
                  for (int jj = 0; jj < 4; jj++) {
                     const float2 t2 = src[cc * 4 + jj];
                     vals[2 * jj] = t2.x;
                     vals[2 * jj + 1] = t2.y;
                  }
                  const int c8 = ky * CPR + cc;
                  const uint32_t off = (c8 >> 3) * 16384 + sw128_offset(tt, (c8 & 7) * 8);
                  *reinterpret_cast<uint4 *>(smem + fp.offIM + off) =
                        make_uint4(pack2(vals[0], vals[1]), pack2(vals[2], vals[3]), pack2(vals[4], vals[5]),
                                   pack2(vals[6], vals[7]));
               }
            }
         }
         // on every path: the window sums above are generic-proxy writes into the stage, which
         // the next stage's bulk copy (async proxy) overwrites once stEmpty is signalled (and
         // the shared-memory im2col operand is read by the MMAs)
         fence_proxy_async_smem();
         named_bar_sync(1, TT);
         if (tt == 0) {
            mbar_arrive(&imFull);
            mbar_arrive(&stEmpty);
         }
         return true;
      };
      // the fold of tile t's D2 into its band (in the stage, which tile t + 1's im2col has
      // read), starting from x on the owned rows (a bulk copy) and 0 elsewhere, and the band store
      int xUses = 0;         // bulk copies of x waited for (thread 0): xFull's phase
      bool xPending = false;  // one issued and not yet waited for
      auto fold_tile = [&](int t) {
         int b, mb, fh;
         tile_of(t, b, mb, fh);
         // thread 0 passes this barrier only after the previous fold's band store has read the
         // stage (bulk_wait_read_all below); a CTA's last two folds follow each other directly
         named_bar_sync(1, TT);
         const int xRows = fh == 0 ? owned_rows(mb) : 0;
         if (tt == 0 && xRows > 0) {
            const uint32_t xb = (uint32_t)(xRows * RP * 4);
            mbar_arrive_expect_tx(&xFull, xb);
            bulk_load(fold, xpad + ((size_t)b * fp.rowsPad + (size_t)S * mb * rpb) * RP, xb, &xFull);
            xPending = true;
         }
         {
            const int n4 = (int)fp.bandFloats / 4;
            float4 *f4 = reinterpret_cast<float4 *>(fold);
            for (int i = xRows * RP / 4 + tt; i < n4; i += TT) f4[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
         }
         if (tt == 0) {
            if (xPending && wait_or_abort(&xFull, (uint32_t)(xUses & 1))) {
               xUses++;
               xPending = false;
            }
            wait_or_abort(&d2Full, (uint32_t)(t & 1));
         }
         if (named_bar_or(1, TT, abortFlag != 0)) return false;
         tc_fence_after();
         const uint32_t lanes = tmemD2 + ((uint32_t)(tq * 32) << 16);
         const int yImg0 = S * (mb * rpb + yl) - (P - S) / 2, xImg0 = S * xl - (P - S) / 2;
         constexpr int SEG = S * C, SEG2 = SEG / 2;  // floats of one patch row in one tap group
         // P/S x P/S tap groups (ty, tx), one barrier each; within a group no two threads touch
         // one pixel, and every pixel sees its taps in the order of the groups
#pragma unroll 1
         for (int ty = 0; ty < P / S; ty++) {
#pragma unroll 1
            for (int hf = 0; hf < FH; hf++) {
               float rowv[FD][P * C];
#pragma unroll
               for (int dd = 0; dd < FD; dd++)
                  tmem_ld_cols<P * C>(lanes + (uint32_t)((S * ty + hf * FD + dd) * P * C), rowv[dd]);
               if (ty == P / S - 1 && hf == FH - 1) {  // D2 read: the next tile's first GEMM2 may overwrite it
                  tc_fence_before();
                  __syncwarp();
                  if (lane == 0) mbar_arrive(&d2Empty);
               }
#pragma unroll
               for (int tx = 0; tx < P / S; tx++) {
                  // the group's pixels of this thread, S*C contiguous floats per patch row, read
                  // and written as pairs (they are distinct, so the adds need not wait on one
                  // another); pixels outside the image keep their value
                  float2 old[FD][SEG2];
                  bool rowIn[FD];
#pragma unroll
                  for (int dd = 0; dd < FD; dd++) {
                     const int ky = S * ty + hf * FD + dd;
                     const int py = yImg0 + ky;
                     rowIn[dd] = py >= 0 && py < g.inNy;
                     const float2 *o2 =
                           reinterpret_cast<const float2 *>(fold + (S * yl + ky) * RP + (S * xl + S * tx) * C);
#pragma unroll
                     for (int j = 0; j < SEG2; j++) old[dd][j] = rowIn[dd] ? o2[j] : make_float2(0.0f, 0.0f);
                  }
#pragma unroll
                  for (int dd = 0; dd < FD; dd++) {
                     const int ky = S * ty + hf * FD + dd;
                     if (rowIn[dd]) {
                        float2 *o2 = reinterpret_cast<float2 *>(fold + (S * yl + ky) * RP + (S * xl + S * tx) * C);
#pragma unroll
                        for (int j = 0; j < SEG2; j++) {
                           float e2[2] = {old[dd][j].x, old[dd][j].y};
#pragma unroll
                           for (int h = 0; h < 2; h++) {
                              const int e = 2 * j + h, dx = e / C;
                              const int px = xImg0 + S * tx + dx;
                              if (px >= 0 && px < g.inNx) e2[h] = __fadd_rn(e2[h], -rowv[dd][S * tx * C + e]);
                           }
                           o2[j] = make_float2(e2[0], e2[1]);
                        }
                     }
                  }
                  named_bar_sync(1, TT);
               }
            }
         }
         fence_proxy_async_smem();
         named_bar_sync(1, TT);
         if (tt == 0) {
            bulk_store(bandsOut + (((size_t)b * g.MB + mb) * nFH + fh) * fp.bandFloats, fold, bandBytes);
            bulk_commit();
            bulk_wait_read_all();
            mbar_arrive(&foldFree);
         }
         return true;
      };
      // im2col(0), then per tile: im2col(t + 1), fold(t).  The four warps take the same
      // decisions (named_bar_or), so they pass the same barriers and leave together.
      if (myTiles > 0) {
         bool ok = im2col(0);
         for (int t = 0; ok && t < myTiles; t++) {
            if (t + 1 < myTiles) ok = im2col(t + 1);
            if (ok) ok = fold_tile(t);
         }
      }
      if (tt == 0) {
         bulk_wait_all();
         // an x copy still in flight (a wait that gave up) lands before shared memory goes away
         if (xPending) mbar_wait(&xFull, (uint32_t)(xUses & 1));
      }
   } else if (warp < EW) {
      // ============================== epilogue (warps 0-15) ==============================
      const int gi = warp >> 3, qd = warp & 3, hh = (warp >> 2) & 1;
      const int pw = 32 * qd + lane;
      // this group's blocks q = gi, gi + 2, ...: the k-th is tile ti, block nb, V slot sv
      // (q % nV) in its use uv (q / nV); stepped, not divided
      int ti = 0, nb = gi, sv = gi, uv = 0, b = 0, mb = 0, fh = 0;
      while (nb >= nBlk) {
         nb -= nBlk;
         ti++;
      }
      if (ti < myTiles) tile_of(ti, b, mb, fh);
      bool dead = false;
      // with four V slots a slot is next loaded two of this group's blocks later, so its release
      // waits for the top of the group's next block (the store has long read it by then); with
      // two it is the group's next block's slot and goes back as soon as the store has read it
      int pendingV = -1;
      auto release_v = [&](int slot) {
         if (lane == 0) {
            bulk_wait_read_all();
            mbar_arrive(&vEmpty[slot]);
         }
      };
      for (int q = gi, k = 0; q < Q; q += 2, k++) {
         const int f0 = fh * fp.FT + nb * kPostNT, rowV = b * g.Npos + mb * 128;
         if (pendingV >= 0) release_v(pendingV);
         pendingV = -1;
         int okw = !dead;
         if (lane == 0 && okw)
            okw = wait_or_abort(&accFull[gi], (uint32_t)(k & 1)) && wait_or_abort(&vFull[sv], (uint32_t)(uv & 1));
         okw = __shfl_sync(0xffffffffu, okw, 0);
         dead = !okw;
         if (okw) {
            tc_fence_after();
            float d[32];
            tmem_ld32(tmem + gi * kPostNT + ((uint32_t)(32 * qd) << 16) + 32 * hh, d);
            tc_fence_before();
            if (lane == 0) mbar_arrive(&accEmpty[gi]);
            uint8_t *vsub = smem + fp.offVT[0] + sv * 32768u + hh * 16384 + 32 * qd * 128;
            uint8_t *vt = vsub + lane * 128;
            const float om = 1.0f - g.e;
            uint32_t ap[16];
#pragma unroll
            for (int sub = 0; sub < 2; sub++) {
               float v[16];
#pragma unroll
               for (int qq = 0; qq < 4; qq++) {
                  const float4 t4 = *reinterpret_cast<const float4 *>(vt + (((4 * sub + qq) ^ (pw & 7)) << 4));
                  v[4 * qq] = t4.x;
                  v[4 * qq + 1] = t4.y;
                  v[4 * qq + 2] = t4.z;
                  v[4 * qq + 3] = t4.w;
               }
               float an[16];
               if constexpr (SIMPLE) {
                  // element pairs on the packed FP32 pipe: t = d + si*ao, t = om*t, v = e*v + t
                  const float2 si2 = make_float2(g.si, g.si), om2 = make_float2(om, om), e2 = make_float2(g.e, g.e);
#pragma unroll
                  for (int jj = 0; jj < 16; jj += 2) {
                     const float ao0 = v[jj] < g.VThresh ? g.AMin : v[jj] - g.AShift;
                     const float ao1 = v[jj + 1] < g.VThresh ? g.AMin : v[jj + 1] - g.AShift;
                     float2 t = __ffma2_rn(si2, make_float2(ao0, ao1), make_float2(d[16 * sub + jj], d[16 * sub + jj + 1]));
                     t = __fmul2_rn(om2, t);
                     const float2 vn = __ffma2_rn(e2, make_float2(v[jj], v[jj + 1]), t);
                     v[jj] = vn.x;
                     v[jj + 1] = vn.y;
                     an[jj] = v[jj] < g.VThresh ? g.AMin : v[jj] - g.AShift;
                     an[jj + 1] = v[jj + 1] < g.VThresh ? g.AMin : v[jj + 1] - g.AShift;
                  }
               } else {
#pragma unroll
                  for (int jj = 0; jj < 16; jj++) {
                     v[jj] = fmaf(g.e, v[jj], om * (d[16 * sub + jj] + g.si * thresh(v[jj], g)));
                     an[jj] = thresh(v[jj], g);
                  }
               }
#pragma unroll
               for (int qq = 0; qq < 4; qq++)
                  *reinterpret_cast<float4 *>(vt + (((4 * sub + qq) ^ (pw & 7)) << 4)) =
                        make_float4(v[4 * qq], v[4 * qq + 1], v[4 * qq + 2], v[4 * qq + 3]);
#pragma unroll
               for (int j = 0; j < 8; j++) ap[8 * sub + j] = pack2(an[2 * j], an[2 * j + 1]);
               if constexpr (WRITEA) {  // the activity for the kernels of a later unfused step
                  const size_t o = (size_t)(rowV + pw) * g.F + f0 + 32 * hh + 16 * sub;
                  st_global_32B(A + o, make_uint4(ap[8 * sub], ap[8 * sub + 1], ap[8 * sub + 2], ap[8 * sub + 3]),
                                make_uint4(ap[8 * sub + 4], ap[8 * sub + 5], ap[8 * sub + 6], ap[8 * sub + 7]));
                  uint4 *lg = reinterpret_cast<uint4 *>(Alo + o);
#pragma unroll
                  for (int t = 0; t < 2; t++) {
                     float l[8];
#pragma unroll
                     for (int u = 0; u < 8; u++) l[u] = an[8 * t + u] - __bfloat162float(__float2bfloat16_rn(an[8 * t + u]));
                     lg[t] = make_uint4(pack2(l[0], l[1]), pack2(l[2], l[3]), pack2(l[4], l[5]), pack2(l[6], l[7]));
                  }
               }
            }
            // A into the group's TMEM A tile once GEMM2 of the group's previous block has read
            // it: lane pw, features 32 hh .. 32 hh + 31 as 16 columns of BF16 pairs
            int oka = 1;
            if (lane == 0 && k >= 1) oka = wait_or_abort(&aEmpty[gi], (uint32_t)((k - 1) & 1));
            oka = __shfl_sync(0xffffffffu, oka, 0);
            if (oka) {
               tc_fence_after();
               const uint32_t ta = tmem + ((uint32_t)(32 * qd) << 16) + colA + 32 * gi + 16 * hh;
               tmem_st8(ta, ap);
               tmem_st8(ta + 8, ap + 8);
               tmem_wait_st();
               tc_fence_before();
            }
            fence_proxy_async_smem();
            __syncwarp();
            if (lane == 0 && oka) {
               mbar_arrive(&aFull[gi]);
               // this warp's 32 x 32 part of the V chunk back to HBM; the slot is free once the
               // store has read it
               bulk_store(V + v_index(g, b, mb * 128 + 32 * qd, f0 + 32 * hh), vsub, 4096);
               bulk_commit();
            }
            if (oka) {
               if (nV == 2)
                  release_v(sv);
               else
                  pendingV = sv;
            }
            dead = !oka;
         }
         sv += 2;
         if (sv >= nV) {
            sv = gi;
            uv++;
         }
         nb += 2;
         while (nb >= nBlk) {
            nb -= nBlk;
            if (++ti < myTiles) tile_of(ti, b, mb, fh);
         }
      }
      if (pendingV >= 0) release_v(pendingV);
      if (lane == 0) bulk_wait_all();
   }
   __syncthreads();
   if (tid == 0 && abortFlag) atomicExch(err, 1);
   tc_fence_before();
   __syncthreads();
   if (warp == 0) tmem_dealloc(tmem, 512);
}

// x into the zero-bordered padded layout of the residual (kernel F starts its bands from it).
__global__ void pad_x_kernel(LcaGeom g, int C, int E, int rowsPad, int RP, const float *__restrict__ x,
                             float *__restrict__ xpad) {
   const size_t n = (size_t)g.nb * rowsPad * RP;
   const int rowElems = g.inNx * C;
   for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
      const int col = (int)(i % RP);
      const size_t r = i / RP;
      const int yp = (int)(r % rowsPad), b = (int)(r / rowsPad);
      const int ye = yp - E, j = col - E * C;
      xpad[i] = (ye >= 0 && ye < g.inNy && j >= 0 && j < rowElems) ? x[((size_t)b * g.inNy + ye) * rowElems + j] : 0.0f;
   }
}

// -------------------------------------------------------------------------------------------
// Probe energy: l2Coeff * sum r^2 + costCoeff * sum cost(T(V)), per image, FP64
// (ColumnEnergyProbe.cpp:60-70 over L2NormProbe and L1NormLCAProbe / FirmThresholdCostFnLCAProbe)
// -------------------------------------------------------------------------------------------
// The residual comes from the padded residual of kernel R (zero border) when rpad is given,
// else from x and the partial reconstructions of the FP32 form.
__global__ void __launch_bounds__(256) energy_kernel(LcaGeom g, int C, const float *__restrict__ x,
                                                     const float *__restrict__ partials,
                                                     const float *__restrict__ rpad, int padPerImage,
                                                     const float *__restrict__ V, double l2Coeff, int costKind,
                                                     double cp0, double cp1, double costCoeff,
                                                     double *__restrict__ out) {
   const int b = blockIdx.x;
   const int nPix = g.inNx * g.inNy * C;
   double l2 = 0.0, cost = 0.0;
   if (rpad) {
      const float *rb = rpad + (size_t)b * padPerImage;
      for (int i = threadIdx.x; i < padPerImage; i += 256) {
         double r = (double)rb[i];
         l2 += r * r;
      }
   } else {
      const float *pb = partials + (size_t)b * g.MB * nPix;
      for (int i = threadIdx.x; i < nPix; i += 256) {
         float rec = pb[i];
         for (int m = 1; m < g.MB; m++) rec = __fadd_rn(rec, pb[(size_t)m * nPix + i]);
         double r = (double)__fadd_rn(x[(size_t)b * nPix + i], -rec);
         l2 += r * r;
      }
   }
   const double tw = cp0 + cp1, maxc = 0.5 * tw, qc = 0.5 / tw;
   // V in 8-element runs (two float4; an image's V is a whole number of 64-feature chunks);
   // the L1 cost sums each run in FP32 (eight nonnegative terms) before the FP64 total
   const float4 *v4 = reinterpret_cast<const float4 *>(V + (size_t)b * g.Npos * g.F);
   const int n8 = g.Npos * g.F / 8;
   for (int i = threadIdx.x; i < n8; i += 256) {
      const float4 p = v4[2 * i], q = v4[2 * i + 1];
      const float e8[8] = {p.x, p.y, p.z, p.w, q.x, q.y, q.z, q.w};
      if (costKind == 1) {
         float s8 = 0.0f;
#pragma unroll
         for (int k = 0; k < 8; k++) s8 += fabsf(thresh(e8[k], g));
         cost += (double)s8;
      } else {
#pragma unroll
         for (int k = 0; k < 8; k++) {
            const double a = fabs((double)thresh(e8[k], g));
            cost += a < tw ? a * (1.0 - qc * a) : maxc;
         }
      }
   }
   __shared__ double s1[256], s2[256];
   s1[threadIdx.x] = l2;
   s2[threadIdx.x] = cost;
   __syncthreads();
   for (int w = 128; w > 0; w >>= 1) {
      if (threadIdx.x < w) {
         s1[threadIdx.x] += s1[threadIdx.x + w];
         s2[threadIdx.x] += s2[threadIdx.x + w];
      }
      __syncthreads();
   }
   if (threadIdx.x == 0) {
      double e = 0.0;
      e += l2Coeff * s1[0];
      e += costCoeff * s2[0];
      out[b] = e;
   }
}

// -------------------------------------------------------------------------------------------
// state / weight preparation
// -------------------------------------------------------------------------------------------
// W [F][KP] (FP32, the pre weights V1->error) -> BF16 hi/lo [F][KP] and transposed [KP][F]
__global__ void prep_weights_kernel(const float *__restrict__ w, int F, int KP, bf16 *Wh, bf16 *Wl, bf16 *Wth,
                                    bf16 *Wtl, float *W32, float *Wt32) {
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= F * KP) return;
   int f = i / KP, k = i % KP;
   float v = w[i];
   bf16 h = __float2bfloat16_rn(v);
   bf16 l = __float2bfloat16_rn(v - __bfloat162float(h));
   Wh[i] = h;
   Wl[i] = l;
   Wth[(size_t)k * F + f] = h;
   Wtl[(size_t)k * F + f] = l;
   W32[i] = v;
   Wt32[(size_t)k * F + f] = v;
}

// A = T(V) for the initial state, BF16 hi/lo and FP32
// (i indexes the reference layout [nb][Npos][F]; V is in the device layout of v_index)
__device__ __forceinline__ size_t v_of(const LcaGeom &g, size_t i) {
   const int f = (int)(i % g.F);
   const size_t bp = i / g.F;
   return v_index(g, (int)(bp / g.Npos), (int)(bp % g.Npos), f);
}

// eight features per thread: two float4 of V (each four features contiguous in its layout),
// 16-byte stores of A and its low half, two of the FP32 activity
__global__ void init_activity_kernel(LcaGeom g, const float *__restrict__ V, bf16 *A, bf16 *Alo, float *A32) {
   const size_t n8 = (size_t)g.nb * g.Npos * g.F / 8;
   for (size_t i8 = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i8 < n8; i8 += (size_t)gridDim.x * blockDim.x) {
      const size_t i = i8 * 8;
      const size_t bp = i / g.F;
      const int f = (int)(i % g.F);
      const int b = (int)(bp / g.Npos), pos = (int)(bp % g.Npos);
      const float4 p = *reinterpret_cast<const float4 *>(V + v_index(g, b, pos, f));
      const float4 q = *reinterpret_cast<const float4 *>(V + v_index(g, b, pos, f + 4));
      const float v8[8] = {p.x, p.y, p.z, p.w, q.x, q.y, q.z, q.w};
      float a[8], l[8];
#pragma unroll
      for (int k = 0; k < 8; k++) {
         a[k] = thresh(v8[k], g);
         l[k] = a[k] - __bfloat162float(__float2bfloat16_rn(a[k]));
      }
      *reinterpret_cast<uint4 *>(A + i) =
            make_uint4(pack2(a[0], a[1]), pack2(a[2], a[3]), pack2(a[4], a[5]), pack2(a[6], a[7]));
      *reinterpret_cast<uint4 *>(Alo + i) =
            make_uint4(pack2(l[0], l[1]), pack2(l[2], l[3]), pack2(l[4], l[5]), pack2(l[6], l[7]));
      *reinterpret_cast<float4 *>(A32 + i) = make_float4(a[0], a[1], a[2], a[3]);
      *reinterpret_cast<float4 *>(A32 + i + 4) = make_float4(a[4], a[5], a[6], a[7]);
   }
}

__global__ void activity_out_kernel(LcaGeom g, const float *__restrict__ V, float *__restrict__ out) {
   size_t n = (size_t)g.nb * g.Npos * g.F;
   for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
      out[i] = thresh(V[v_of(g, i)], g);
}

// V between the reference layout and the device layout
__global__ void v_layout_kernel(LcaGeom g, const float *__restrict__ src, float *__restrict__ dst, int toDevice) {
   size_t n = (size_t)g.nb * g.Npos * g.F;
   for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
      if (toDevice) dst[v_of(g, i)] = src[i];
      else dst[i] = src[v_of(g, i)];
   }
}

}  // namespace

// The SIMT FP32 form lives in lca_solver_fp32.cu and shares LcaGeom through this hook.
namespace pvgpu {
pvgpu_status lca_fp32_step(int S, int P, int C, const LcaGeom &g, const float *x, const float *W32, const float *Wt32,
                           float *partials, float *V, float *A32, cudaStream_t s, cudaEvent_t mid);
}

// Images [img0, img0 + g.nb) of the batch as a batch of their own: the geometry and the tensor
// maps of the activity rows they own (every other per-image array is addressed from a base
// pointer, shifted by img0 images at launch).
struct LcaHalf {
   LcaGeom g;
   int img0;
   CUtensorMap tmA, tmAlo, tmAst;
};

struct pvgpu_lca_solver {
   pvgpu_lca_solver_desc d;
   LcaGeom g;
   int S, P, C, KP;
   int stepsRun;
   float *V = nullptr, *partials = nullptr, *A32 = nullptr, *W32 = nullptr, *Wt32 = nullptr;
   float *rpad = nullptr;  // padded residual x - W^T a (kernel D -> kernel P)
   bf16 *A = nullptr, *Alo = nullptr, *W = nullptr, *Wlo = nullptr, *Wt = nullptr, *Wtlo = nullptr;
   int *err = nullptr;
   CUtensorMap tmA, tmAlo, tmWtH, tmWtloH, tmW, tmWlo, tmAst;  // tmWtH*: half-height W^T tiles
   PostPlan plan, planX3;
   ReconPlan rplan, rplanX3;
   FusePlan fplan;
   float *bands = nullptr;  // kernel F's bands, two buffers (a step reads one and writes the other)
   float *xpad = nullptr;   // x in the padded layout (kernel F)
   size_t bandsPerBuf = 0;  // floats in one band buffer (sized for 128-feature tiles)
   bool padValid = false;  // rpad holds the residual of the last step (BF16 form) rather than partials
   bool weightsSet = false;
   // optional per-kernel timing: events before kernel R, between R and P, after P
   std::vector<cudaEvent_t> ev;
   std::vector<uint8_t> evKind;  // per recorded step: 0 kernels R + P, 1 R + F, 2 F alone
   size_t evNext = 0;
   bool profiling = false;
   // the BF16 run as one CUDA graph: captured on capStream, replayed on the caller's stream;
   // rebuilt when the input pointer or the step counts change
   int maxRecon[2] = {0, 0};  // co-resident kernel-R CTAs (BF16, BF16x3)
   cudaStream_t capStream = nullptr;
   cudaGraphExec_t graph = nullptr;
   const float *graphX = nullptr;
   int graphSteps = -1, graphX3 = -1;
   // the graph's schedule: one chain of kernels over the batch, or two independent chains over
   // the two halves captured as parallel graph branches (one half's kernels fill the ramp and
   // tail of the other's); caps on the persistent grids; programmatic edges within a chain
   pvgpu_lca_schedule sched = {1, 0, 0, 1, 1};
   LcaHalf half[2];
   cudaStream_t capStream2 = nullptr;
   cudaEvent_t forkEv = nullptr, joinEv = nullptr;
};

namespace {

int g_num_sms = 0;

// Shared-memory layout of kernel P for a feature tile FT, ring depths nV / nW and A staging;
// total = 0 when FT does not divide the features.
PostPlan post_plan_for(const LcaGeom &g, int S, int P, int C, bool x3, int numSms, int FT, int nV, int nW, int stA) {
   const int KP = P * P * C, NKC = KP / 64, E = (P - S) / 2;
   auto al = [](uint32_t v) { return (v + 1023u) & ~1023u; };
   PostPlan pl;
   std::memset(&pl, 0, sizeof(pl));
   if (FT <= 0 || FT % 64 || g.F % FT || (stA && x3)) return pl;
   pl.RP = ((g.inNx + 2 * E) * C + 3) & ~3;
   pl.rowsPad = g.inNy + 2 * E;
   const uint32_t RWR = (uint32_t)rwin_rows(S, P, g.rowsPerBlock);
   const uint32_t wB = NKC * kPostNT * 128, imB = NKC * 16384, vtB = 2 * 16384;
   const uint32_t winB = RWR * (uint32_t)pl.RP * 4;
   uint32_t o = 0;
   pl.offIM = o;
   o = al(o + imB);
   pl.offIMlo = o;
   if (x3) o = al(o + imB);
   for (int sl = 0; sl < kMaxWSlots; sl++) {
      pl.offW[sl] = pl.offWlo[sl] = o;
      if (sl < nW) {
         o = al(o + wB);
         pl.offWlo[sl] = o;
         if (x3) o = al(o + wB);
      }
   }
   for (int sl = 0; sl < kMaxVSlots; sl++) {
      pl.offVT[sl] = o;
      if (sl < nV) o = al(o + vtB);
   }
   pl.wStride = (x3 ? 2u : 1u) * al(wB);
   pl.offWin = o;
   o = al(o + winB);
   pl.offA = o;
   if (stA) o = al(o + 8 * 2048);
   pl.total = o + 1024;
   pl.nV = nV;
   pl.nW = nW;
   pl.stageA = stA;
   pl.FT = FT;
   const int nTiles = g.nb * g.MB * (g.F / pl.FT);
   pl.G = numSms < nTiles ? numSms : nTiles;
   return pl;
}

constexpr uint32_t kSmemBudget = 227u * 1024u - 512u;  // dynamic shared memory; static shares the budget
constexpr uint32_t kSmemHalfSm = 116u * 1024u;         // more than half of an SM's 228 KB

// ring shapes, best first: V tiles first (they come from HBM), then weight tiles (from L2); A
// staged for TMA stores where it fits with at least two V slots (not in BF16x3 steps, which
// also write the low halves)
constexpr int kRings[][3] = {{3, 2, 1}, {3, 1, 1}, {2, 2, 1}, {2, 1, 1}, {3, 2, 0},
                             {3, 1, 0}, {2, 2, 0}, {2, 1, 0}, {1, 1, 0}};

// The default shape: 256-feature tiles (or the largest multiple of 64 dividing F) and the first
// ring shape that fits.
PostPlan make_post_plan(const LcaGeom &g, int S, int P, int C, bool x3, int numSms) {
   int FT = g.F < 256 ? g.F : 256;
   while (g.F % FT) FT -= 64;
   PostPlan pl;
   std::memset(&pl, 0, sizeof(pl));
   for (const auto &r : kRings) {
      pl = post_plan_for(g, S, P, C, x3, numSms, FT, r[0], r[1], r[2]);
      if (pl.total && pl.total <= kSmemBudget) return pl;
   }
   return pl;
}

ReconPlan recon_plan_for(const LcaGeom &g, int S, int P, int C, bool x3, int maxCtas, int nStage) {
   const int KP = P * P * C, E = (P - S) / 2;
   auto al = [](uint32_t v) { return (v + 1023u) & ~1023u; };
   ReconPlan rp;
   std::memset(&rp, 0, sizeof(rp));
   rp.RP = ((g.inNx + 2 * E) * C + 3) & ~3;
   rp.rowsPad = g.inNy + 2 * E;
   rp.stageBytes = al((x3 ? 2u : 1u) * (128u * 64u * 2u + (uint32_t)KP * 64u * 2u));
   const uint32_t imgB = al((uint32_t)(g.inNx * g.inNy * C) * 4u);
   rp.nStage = nStage;
   uint32_t o = nStage * rp.stageBytes;
   rp.offRec = o;
   o += imgB;
   rp.offX[0] = o;
   o += imgB;
   rp.offX[1] = o;
   rp.xStride = imgB;
   o += imgB;
   rp.total = o + 1024;
   rp.G = maxCtas < g.nb ? maxCtas : g.nb;
   return rp;
}

// The default shape: the deepest ring that fits.
ReconPlan make_recon_plan(const LcaGeom &g, int S, int P, int C, bool x3, int maxCtas) {
   ReconPlan rp = recon_plan_for(g, S, P, C, x3, maxCtas, 2);
   for (int n = kMaxRStages; n >= 2; n--) {
      rp = recon_plan_for(g, S, P, C, x3, maxCtas, n);
      if (rp.total <= kSmemBudget) break;
   }
   return rp;
}

// Shared-memory layout of kernel F for a feature tile FT, nV V slots and nW weight slots;
// total = 0 when the geometry does not allow it (FT not a multiple of 64 dividing F, an odd V
// ring -- each epilogue group owns every other slot --, or bands reaching past the
// neighbouring blocks).
FusePlan fuse_plan_for(const LcaGeom &g, int S, int P, int C, int numSms, int FT, int nV, int nW) {
   const int KP = P * P * C, NKC = KP / 64, E = (P - S) / 2;
   auto al = [](uint32_t v) { return (v + 1023u) & ~1023u; };
   FusePlan fp;
   std::memset(&fp, 0, sizeof(fp));
   if (FT < 64 || FT % 64 || g.F % FT || (nV != 2 && nV != 4) || nW < 2 || nW > 4 ||
       P - S > S * g.rowsPerBlock || g.MB < 1)
      return fp;
   const int nFH = g.F / FT;
   fp.FT = FT;
   fp.nV = nV;
   fp.nW = nW;
   fp.RP = ((g.inNx + 2 * E) * C + 3) & ~3;
   fp.rowsPad = g.inNy + 2 * E;
   fp.RWR = rwin_rows(S, P, g.rowsPerBlock);
   fp.bandFloats = (uint32_t)(fp.RWR * fp.RP);
   fp.sliceFloats = (uint32_t)((P - S) * fp.RP);
   const uint32_t wB = NKC * kPostNT * 128;
   // the im2col operand lives in TMEM when it fits beside the accumulators and the A tiles
   // (kernel F's column budget: 2 x 64 + KP + 2 x 32 + KP / 2 <= 512), else in shared memory
   const bool imTmem = 2 * kPostNT + KP + 64 + KP / 2 <= 512;
   uint32_t o = 0;
   fp.offIM = o;
   if (!imTmem) o = al(o + NKC * 16384);
   fp.wStride = al(wB);
   for (int sl = 0; sl < 4; sl++) {
      fp.offW[sl] = o;
      if (sl < nW) o = al(o + wB);
   }
   for (int sl = 0; sl < 4; sl++) {
      fp.offVT[sl] = o;
      if (sl < nV) o = al(o + 32768);
   }
   fp.offStage = o;
   o += nFH * fp.bandFloats * 4;
   fp.offTop = o;
   o += nFH * fp.sliceFloats * 4;
   fp.offBot = o;
   o += nFH * fp.sliceFloats * 4;
   fp.offFold = fp.offStage;  // the fold runs in the stage once the next tile's im2col has read it
   o = al(o);
   fp.total = o + 1024;
   const int nTiles = g.nb * g.MB * nFH;
   fp.G = numSms < nTiles ? numSms : nTiles;
   return fp;
}

// The default: 256-feature tiles (or the largest multiple of 64 dividing F), the deepest V ring
// (4 or 2 slots) that fits with two weight slots.
FusePlan make_fuse_plan(const LcaGeom &g, int S, int P, int C, int numSms) {
   FusePlan fp;
   std::memset(&fp, 0, sizeof(fp));
   for (int FT = std::min(256, g.F); FT >= 64; FT -= 64) {
      if (g.F % FT || FT % 64) continue;
      for (int nV = 4; nV >= 2; nV -= 2) {
         fp = fuse_plan_for(g, S, P, C, numSms, FT, nV, 2);
         if (fp.total && fp.total <= kSmemBudget) return fp;
      }
   }
   std::memset(&fp, 0, sizeof(fp));
   return fp;
}

// The launch arguments of one timestep over a batch view (the whole batch or one half).
struct StepArgs {
   LcaGeom g;
   ReconPlan rp;
   PostPlan pl;
   FusePlan fp;
   const CUtensorMap *tmA, *tmAlo, *tmAst, *tmWtH, *tmWtloH, *tmW, *tmWlo;
   const float *x;
   float *rpad, *V;
   bf16 *A, *Alo;
   float *bands[2];
   float *xpad;
   int *err;
};

// Kernel R's and kernel P's persistent grids for nb images under the schedule's caps.
void size_grids(const pvgpu_lca_solver *s, int nb, bool x3, ReconPlan &rp, PostPlan &pl) {
   int rctas = std::min(s->maxRecon[x3 ? 1 : 0], nb);
   if (s->sched.reconCtas > 0) rctas = std::min(rctas, s->sched.reconCtas);
   rp.G = std::max(rctas, 1);
   const int nTiles = nb * s->g.MB * (s->g.F / pl.FT);
   int ctas = g_num_sms;
   if (s->sched.postCtas > 0) ctas = std::min(ctas, s->sched.postCtas);
   pl.G = std::min(ctas, nTiles);
}

void size_fuse_grid(const pvgpu_lca_solver *s, int nb, FusePlan &fp) {
   if (!fp.FT) return;
   const int nTiles = nb * s->g.MB * (s->g.F / fp.FT);
   int ctas = g_num_sms;
   if (s->sched.postCtas > 0) ctas = std::min(ctas, s->sched.postCtas);
   fp.G = std::min(ctas, nTiles);
}

// view = -1: the whole batch; 0 / 1: that half.
StepArgs step_args(const pvgpu_lca_solver *s, int view, const float *x, bool x3) {
   StepArgs a;
   const LcaHalf *h = view >= 0 ? &s->half[view] : nullptr;
   a.g = h ? h->g : s->g;
   a.rp = x3 ? s->rplanX3 : s->rplan;
   a.pl = x3 ? s->planX3 : s->plan;
   size_grids(s, a.g.nb, x3, a.rp, a.pl);
   a.fp = s->fplan;
   size_fuse_grid(s, a.g.nb, a.fp);
   // Kernels R and F take all 512 TMEM columns, whose allocation waits without a bound: a CTA
   // of either never shares an SM (more than half of the SM's shared memory per CTA), so no CTA
   // waits for TMEM that another CTA holds while it waits on the first.  With two chains kernel P (256 columns)
   // gets an SM to itself as well: a CTA of one chain must not wait for TMEM held by a CTA that
   // waits, through its own chain, on the first one.
   a.rp.total = std::max(a.rp.total, kSmemHalfSm);
   a.fp.total = std::max(a.fp.total, kSmemHalfSm);
   if (h) a.pl.total = std::max(a.pl.total, kSmemHalfSm);
   const size_t i0 = h ? (size_t)h->img0 : 0;
   const size_t state = (size_t)s->g.Npos * s->g.F;
   a.tmA = h ? &h->tmA : &s->tmA;
   a.tmAlo = h ? &h->tmAlo : &s->tmAlo;
   a.tmAst = h ? &h->tmAst : &s->tmAst;
   a.tmWtH = &s->tmWtH;
   a.tmWtloH = &s->tmWtloH;
   a.tmW = &s->tmW;
   a.tmWlo = &s->tmWlo;
   a.x = x + i0 * (size_t)s->g.inNx * s->g.inNy * s->C;
   a.rpad = s->rpad + i0 * (size_t)a.rp.rowsPad * a.rp.RP;
   a.V = s->V + i0 * state;
   a.A = s->A + i0 * state;
   a.Alo = s->Alo + i0 * state;
   // bands: [image][block][feature tile][RWR x RP] per buffer
   const size_t perImage = a.fp.FT ? (size_t)s->g.MB * (s->g.F / a.fp.FT) * a.fp.bandFloats : 0;
   for (int k = 0; k < 2; k++) a.bands[k] = s->bands ? s->bands + k * s->bandsPerBuf + i0 * perImage : nullptr;
   a.xpad = s->xpad ? s->xpad + i0 * (size_t)a.rp.rowsPad * a.rp.RP : nullptr;
   a.err = s->err;
   return a;
}

template <int S, int P, int C>
struct Launcher {
   // shared-memory limits of both kernels (once, at create: not inside a stream capture)
   static pvgpu_status set_attrs(const pvgpu_lca_solver *) {
      const void *fns[10] = {reinterpret_cast<const void *>(recon_tc_kernel<S, P, C, false>),
                            reinterpret_cast<const void *>(recon_tc_kernel<S, P, C, true>),
                            reinterpret_cast<const void *>(post_tc_kernel<S, P, C, false, false>),
                            reinterpret_cast<const void *>(post_tc_kernel<S, P, C, true, false>),
                            reinterpret_cast<const void *>(post_tc_kernel<S, P, C, false, true>),
                            reinterpret_cast<const void *>(post_tc_kernel<S, P, C, true, true>),
                            reinterpret_cast<const void *>(step_tc_kernel<S, P, C, false, false>),
                            reinterpret_cast<const void *>(step_tc_kernel<S, P, C, false, true>),
                            reinterpret_cast<const void *>(step_tc_kernel<S, P, C, true, false>),
                            reinterpret_cast<const void *>(step_tc_kernel<S, P, C, true, true>)};
      for (int i = 0; i < 10; i++) {
         cudaError_t e = cudaFuncSetAttribute(fns[i], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBudget);
         if (e != cudaSuccess) return pvgpu::record_cuda_error(e, "lca kernel attributes");
      }
      return PVGPU_OK;
   }
   // Launches over a batch view, each with programmatic stream serialisation unless the
   // schedule (or per-kernel timing, which keeps the kernels apart) turns it off, so that its
   // set-up overlaps the tail of the kernel before it.
   static cudaLaunchConfig_t config(int grid, uint32_t smem, cudaStream_t st, bool programmatic,
                                    cudaLaunchAttribute *attr, int threads = 320) {
      attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
      attr[0].val.programmaticStreamSerializationAllowed = 1;
      cudaLaunchConfig_t c = {};
      c.gridDim = dim3(grid);
      c.blockDim = dim3(threads);
      c.dynamicSmemBytes = smem;
      c.stream = st;
      c.attrs = attr;
      c.numAttrs = programmatic ? 1 : 0;
      return c;
   }
   // kernel R: the residual x - W^T a into the padded layout
   static pvgpu_status launch_R(const StepArgs &a, bool x3, cudaStream_t st, bool programmatic) {
      cudaLaunchAttribute attr[1];
      cudaLaunchConfig_t c = config(a.rp.G, a.rp.total, st, programmatic, attr);
      cudaError_t e = x3 ? cudaLaunchKernelEx(&c, recon_tc_kernel<S, P, C, true>, *a.tmA, *a.tmAlo, *a.tmWtH,
                                              *a.tmWtloH, a.g, a.rp, a.x, a.rpad, a.err)
                         : cudaLaunchKernelEx(&c, recon_tc_kernel<S, P, C, false>, *a.tmA, *a.tmAlo, *a.tmWtH,
                                              *a.tmWtloH, a.g, a.rp, a.x, a.rpad, a.err);
      return e == cudaSuccess ? PVGPU_OK : pvgpu::record_cuda_error(e, "lca recon");
   }
   // kernel P: post delivery of the residual and the LCA update
   static pvgpu_status launch_P(const StepArgs &a, bool x3, cudaStream_t st, bool programmatic) {
      cudaLaunchAttribute attr[1];
      cudaLaunchConfig_t c = config(a.pl.G, a.pl.total, st, programmatic, attr);
      auto fn = x3 ? (a.g.simple ? post_tc_kernel<S, P, C, true, true> : post_tc_kernel<S, P, C, true, false>)
                   : (a.g.simple ? post_tc_kernel<S, P, C, false, true> : post_tc_kernel<S, P, C, false, false>);
      cudaError_t e = cudaLaunchKernelEx(&c, fn, *a.tmW, *a.tmWlo, *a.tmAst, a.g, a.pl, (const float *)a.rpad, a.V,
                                         a.A, a.Alo, a.err);
      return e == cudaSuccess ? PVGPU_OK : pvgpu::record_cuda_error(e, "lca post");
   }
   // kernel F: a whole timestep; mode 0 reads kernel R's residual, mode 1 the bands in rin
   static pvgpu_status launch_F(const StepArgs &a, int mode, int writeA, const float *rin, float *bout,
                                cudaStream_t st, bool programmatic) {
      cudaLaunchAttribute attr[1];
      cudaLaunchConfig_t c = config(a.fp.G, a.fp.total, st, programmatic, attr, kFuseThreads);
      auto fn = a.g.simple ? (writeA ? step_tc_kernel<S, P, C, true, true> : step_tc_kernel<S, P, C, true, false>)
                           : (writeA ? step_tc_kernel<S, P, C, false, true> : step_tc_kernel<S, P, C, false, false>);
      cudaError_t e = cudaLaunchKernelEx(&c, fn, *a.tmW, a.g, a.fp, mode, rin, bout, (const float *)a.xpad, a.V, a.A,
                                         a.Alo, a.err);
      return e == cudaSuccess ? PVGPU_OK : pvgpu::record_cuda_error(e, "lca fused step");
   }
   // recon CTAs that can be resident at once (one CTA per SM)
   static int max_recon_ctas(const ReconPlan &rp, bool x3) {
      const void *fn = x3 ? reinterpret_cast<const void *>(recon_tc_kernel<S, P, C, true>)
                          : reinterpret_cast<const void *>(recon_tc_kernel<S, P, C, false>);
      if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rp.total) != cudaSuccess) {
         cudaGetLastError();
         return 0;
      }
      int n = 0;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, 320, rp.total) != cudaSuccess) {
         cudaGetLastError();
         return 0;
      }
      return std::min(n, 1) * g_num_sms;
   }
   static bool fits(const pvgpu_lca_solver *s, bool x3) {
      const uint32_t pt = x3 ? s->planX3.total : s->plan.total;
      return (x3 ? s->rplanX3.total : s->rplan.total) <= kSmemBudget && pt && pt <= kSmemBudget;
   }

};

template <typename Fn>
pvgpu_status dispatch(int S, int P, int C, Fn &&fn) {
   if (S == 2 && P == 8 && C == 1) return fn(Launcher<2, 8, 1>());
   if (S == 2 && P == 8 && C == 3) return fn(Launcher<2, 8, 3>());
   if (S == 4 && P == 16 && C == 1) return fn(Launcher<4, 16, 1>());
   return PVGPU_ERR_UNSUPPORTED_SHAPE;
}

// Whether a BF16 run of n steps (the last m BF16x3) takes kernel F: it needs the fused plan,
// the schedule's consent and at least two fused steps (the run's final BF16 step and its
// BF16x3 steps run as kernels R + P, which leave the residual for the energy probe).
bool use_fusion(const pvgpu_lca_solver *s, int n, int m) {
   const int nF = n - m - (m == 0 ? 1 : 0);
   return s->sched.fused && s->bands && s->fplan.total && s->fplan.total <= kSmemBudget && nF >= 2;
}

// One BF16 run over a batch view, launched on st.  With kernel F: x padded once; timestep 1 =
// kernel R + kernel F reading R's residual (mode 0); then kernel F alone reading the bands of
// the step before (mode 1); the last fused step also writes A and its low half for the
// kernels R that follow.  Every other step is kernel R + kernel P.  With prof, three events
// per timestep: before it, after its kernel R (or at once), after it.
pvgpu_status enqueue_run(pvgpu_lca_solver *s, const float *x, int n, int m, int view, cudaStream_t st, bool prof) {
   const bool fuse = use_fusion(s, n, m);
   const int nF = fuse ? n - m - (m == 0 ? 1 : 0) : 0;
   return dispatch(s->S, s->P, s->C, [&](auto L) -> pvgpu_status {
      const StepArgs a16 = step_args(s, view, x, false), a3 = step_args(s, view, x, true);
      const bool pg = s->sched.programmatic != 0 && !prof;
      if (fuse) {
         const int E = (s->P - s->S) / 2;
         pad_x_kernel<<<g_num_sms * 4, 256, 0, st>>>(a16.g, s->C, E, a16.rp.rowsPad, a16.rp.RP, a16.x, a16.xpad);
         cudaError_t e = cudaGetLastError();
         if (e != cudaSuccess) return pvgpu::record_cuda_error(e, "lca pad x");
      }
      pvgpu_status r = PVGPU_OK;
      for (int t = 0; t < n && r == PVGPU_OK; t++) {
         const bool x3 = t >= n - m;
         const StepArgs &a = x3 ? a3 : a16;
         const bool rec = prof && s->evNext + 3 <= s->ev.size();
         if (rec) cudaEventRecord(s->ev[s->evNext], st);
         uint8_t kind = 0;
         if (t < nF) {
            if (t == 0) r = L.launch_R(a, false, st, pg);
            if (rec) cudaEventRecord(s->ev[s->evNext + 1], st);
            if (r == PVGPU_OK)
               r = L.launch_F(a, t == 0 ? 0 : 1, t == nF - 1 ? 1 : 0, t == 0 ? a.rpad : a.bands[(t - 1) & 1],
                              a.bands[t & 1], st, pg);
            kind = t == 0 ? 1 : 2;
         } else {
            r = L.launch_R(a, x3, st, pg);
            if (rec) cudaEventRecord(s->ev[s->evNext + 1], st);
            if (r == PVGPU_OK) r = L.launch_P(a, x3, st, pg);
         }
         if (rec) {
            cudaEventRecord(s->ev[s->evNext + 2], st);
            s->evKind[s->evNext / 3] = kind;
            s->evNext += 3;
         }
      }
      return r;
   });
}

void free_solver(pvgpu_lca_solver *s) {
   for (cudaEvent_t e : s->ev) cudaEventDestroy(e);
   if (s->graph) cudaGraphExecDestroy(s->graph);
   if (s->capStream) cudaStreamDestroy(s->capStream);
   if (s->capStream2) cudaStreamDestroy(s->capStream2);
   if (s->forkEv) cudaEventDestroy(s->forkEv);
   if (s->joinEv) cudaEventDestroy(s->joinEv);
   void *ptrs[] = {s->V,   s->partials, s->rpad, s->A32, s->W32, s->Wt32,  s->A,
                   s->Alo, s->W,        s->Wlo,  s->Wt,  s->Wtlo, s->bands, s->xpad, s->err};
   for (void *p : ptrs)
      if (p) cudaFree(p);
   delete s;
}

// ---- autotuning -------------------------------------------------------------------------
// The shapes picked for one geometry: kernel P {FT, nV, nW, stageA} and kernel R {nStage}, for
// the BF16 form [0] and the BF16x3 form [1].  Kept per process, keyed by the geometry and the
// SM count, and applied to every solver created afterwards with the same geometry.
struct TunedShapes {
   int post[2][4];
   int recon[2];
   int fuse[3];  // kernel F {FT, nV, nW}; FT = 0: none
   pvgpu_lca_schedule sched;
};

std::mutex g_tune_mu;
std::map<std::array<int, 10>, TunedShapes> g_tuned;

std::array<int, 10> tune_key(const pvgpu_lca_solver *s) {
   const LcaGeom &g = s->g;
   return {s->S, s->P, s->C, g.nb, g.inNx, g.inNy, g.v1Nx, g.v1Ny, g.F, g_num_sms};
}

void set_shapes(pvgpu_lca_solver *s, const TunedShapes &t) {
   if (t.fuse[0] && s->bands) {
      FusePlan fp = fuse_plan_for(s->g, s->S, s->P, s->C, g_num_sms, t.fuse[0], t.fuse[1], t.fuse[2]);
      if (fp.total && fp.total <= kSmemBudget) s->fplan = fp;
   }
   for (int x3 = 0; x3 < 2; x3++) {
      const int *q = t.post[x3];
      PostPlan pl = post_plan_for(s->g, s->S, s->P, s->C, x3 != 0, g_num_sms, q[0], q[1], q[2], q[3]);
      if (pl.total && pl.total <= kSmemBudget) (x3 ? s->planX3 : s->plan) = pl;
      ReconPlan rp = recon_plan_for(s->g, s->S, s->P, s->C, x3 != 0, s->maxRecon[x3], t.recon[x3]);
      if (rp.total <= kSmemBudget) (x3 ? s->rplanX3 : s->rplan) = rp;
   }
   if (t.sched.chains == 1 || (s->g.nb >= 2 && s->capStream2)) s->sched = t.sched;
   if (s->graph) cudaGraphExecDestroy(s->graph);
   s->graph = nullptr;
}

void apply_tuned(pvgpu_lca_solver *s) {
   std::lock_guard<std::mutex> lk(g_tune_mu);
   auto it = g_tuned.find(tune_key(s));
   if (it != g_tuned.end()) set_shapes(s, it->second);
}

}  // namespace

extern "C" pvgpu_status pvgpu_lca_solver_create(const pvgpu_lca_solver_desc *d, pvgpu_lca_solver **out) {
   if (!d || !out) return PVGPU_ERR_BAD_ARG;
   *out = nullptr;
   if (d->nbatch <= 0 || d->inNx <= 0 || d->inNy <= 0 || d->inNf <= 0 || d->v1Nx <= 0 || d->v1Ny <= 0 ||
       d->v1Nf <= 0 || d->nxp <= 0 || d->tau <= 0.0f)
      return PVGPU_ERR_BAD_ARG;
   if (d->inNx % d->v1Nx || d->inNy % d->v1Ny || d->inNx / d->v1Nx != d->inNy / d->v1Ny) return PVGPU_ERR_UNSUPPORTED_SHAPE;
   const int S = d->inNx / d->v1Nx;
   if (!pvgpu::axis_legal(d->v1Nx, d->inNx, d->nxp)) return PVGPU_ERR_ILLEGAL_GEOMETRY;
   const int P = d->nxp, C = d->inNf, KP = P * P * C;
   const int Npos = d->v1Nx * d->v1Ny;
   if (Npos % 128 || 128 % d->v1Nx || KP % 64 || KP > 256 || d->v1Nf % 64) return PVGPU_ERR_UNSUPPORTED_SHAPE;
   if ((d->inNx * d->inNy * d->inNf) % 4) return PVGPU_ERR_UNSUPPORTED_SHAPE;  // an image is bulk-copied (16-byte multiple)
   if (dispatch(S, P, C, [](auto) { return PVGPU_OK; }) != PVGPU_OK) return PVGPU_ERR_UNSUPPORTED_SHAPE;
   pvgpu_lca_solver *s = new (std::nothrow) pvgpu_lca_solver();
   if (!s) return PVGPU_ERR_OOM;
   s->d = *d;
   s->S = S;
   s->P = P;
   s->C = C;
   s->KP = KP;
   s->stepsRun = 0;
   LcaGeom &g = s->g;
   g.nb = d->nbatch;
   g.inNx = d->inNx;
   g.inNy = d->inNy;
   g.v1Nx = d->v1Nx;
   g.v1Ny = d->v1Ny;
   g.F = d->v1Nf;
   g.Npos = Npos;
   g.MB = Npos / 128;
   g.rowsPerBlock = 128 / d->v1Nx;
   g.NT = kPostNT;
   float vt = d->VThresh, vw = d->VWidth;
   if (vw < 0) {
      vt += vw;
      vw = -vw;
   }
   g.VThresh = vt;
   g.AMin = d->AMin;
   g.AMax = d->AMax;
   g.AShift = d->AShift;
   g.VWidth = vw;
   g.e = (float)exp(-(double)d->dt / (double)d->tau);
   g.si = d->selfInteract ? 1.0f : 0.0f;
   g.simple = (vw == 0.0f && !(d->AMax < FLT_MAX) && vt > -FLT_MAX) ? 1 : 0;
   const size_t nState = (size_t)g.nb * Npos * g.F;
   const size_t nPart = (size_t)g.nb * g.MB * d->inNx * d->inNy * C;
   const size_t nW = (size_t)g.F * KP;
   const int E = (P - S) / 2;
   const size_t nPad = (size_t)g.nb * (d->inNy + 2 * E) * (((d->inNx + 2 * E) * C + 3) & ~3);
   bool ok = cudaMalloc(&s->V, nState * 4) == cudaSuccess && cudaMalloc(&s->A32, nState * 4) == cudaSuccess &&
             cudaMalloc(&s->A, nState * 2) == cudaSuccess && cudaMalloc(&s->Alo, nState * 2) == cudaSuccess &&
             cudaMalloc(&s->partials, nPart * 4) == cudaSuccess && cudaMalloc(&s->W, nW * 2) == cudaSuccess &&
             cudaMalloc(&s->Wlo, nW * 2) == cudaSuccess && cudaMalloc(&s->Wt, nW * 2) == cudaSuccess &&
             cudaMalloc(&s->Wtlo, nW * 2) == cudaSuccess && cudaMalloc(&s->W32, nW * 4) == cudaSuccess &&
             cudaMalloc(&s->Wt32, nW * 4) == cudaSuccess && cudaMalloc(&s->err, sizeof(int)) == cudaSuccess &&
             cudaMalloc(&s->rpad, nPad * 4) == cudaSuccess;
   if (!ok) {
      cudaGetLastError();
      free_solver(s);
      return PVGPU_ERR_OOM;
   }
   cudaMemset(s->err, 0, sizeof(int));
   // the activity maps of images [i0, i0 + n): A and its low half as 128-row MMA tiles, and A as
   // one epilogue warp's 32 x 32 part (64-byte swizzle) for the staged stores
   auto activity_maps = [&](int i0, int n, CUtensorMap *tA, CUtensorMap *tAlo, CUtensorMap *tAst) {
      const uint64_t rows = (uint64_t)n * Npos;
      bf16 *a = s->A + (size_t)i0 * Npos * g.F, *alo = s->Alo + (size_t)i0 * Npos * g.F;
      if (!pvgpu::make_tmap_bf16_sw128(tA, a, rows, g.F, g.F, 128) ||
          !pvgpu::make_tmap_bf16_sw128(tAlo, alo, rows, g.F, g.F, 128))
         return false;
      pvgpu::EncodeTiledFn enc = pvgpu::encode_tiled_fn();
      cuuint64_t dims[2] = {(cuuint64_t)g.F, rows};
      cuuint64_t strides[1] = {(cuuint64_t)g.F * 2};
      cuuint32_t box[2] = {32, 32};
      cuuint32_t estr[2] = {1, 1};
      return enc && enc(tAst, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, a, dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
   };
   ok = activity_maps(0, g.nb, &s->tmA, &s->tmAlo, &s->tmAst) &&
        pvgpu::make_tmap_bf16_sw128(&s->tmWtH, s->Wt, KP, g.F, g.F, KP / 2) &&
        pvgpu::make_tmap_bf16_sw128(&s->tmWtloH, s->Wtlo, KP, g.F, g.F, KP / 2) &&
        pvgpu::make_tmap_bf16_sw128(&s->tmW, s->W, g.F, KP, KP, g.NT) &&
        pvgpu::make_tmap_bf16_sw128(&s->tmWlo, s->Wlo, g.F, KP, KP, g.NT);
   if (ok && g.nb >= 2) {
      // the two halves: an even first half where that leaves images for the second
      int n0 = (g.nb / 2 + 1) & ~1;
      if (n0 >= g.nb) n0 = g.nb / 2;
      for (int c = 0; c < 2 && ok; c++) {
         LcaHalf &h = s->half[c];
         h.g = g;
         h.img0 = c ? n0 : 0;
         h.g.nb = c ? g.nb - n0 : n0;
         ok = activity_maps(h.img0, h.g.nb, &h.tmA, &h.tmAlo, &h.tmAst);
      }
   }
   if (!ok) {
      free_solver(s);
      return PVGPU_ERR_LAUNCH;
   }
   if (!g_num_sms) {
      int dev = 0, n = 0;
      cudaGetDevice(&dev);
      if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 148;
      g_num_sms = n;
   }
   s->plan = make_post_plan(g, S, P, C, false, g_num_sms);
   s->planX3 = make_post_plan(g, S, P, C, true, g_num_sms);
   s->fplan = make_fuse_plan(g, S, P, C, g_num_sms);
   if (s->fplan.total) {
      // band buffers sized for the smallest feature tile that divides F (the most bands)
      int ftMin = 0;
      for (int FT = 64; FT <= g.F && !ftMin; FT += 64)
         if (g.F % FT == 0) ftMin = FT;
      s->bandsPerBuf = (size_t)g.nb * g.MB * (g.F / ftMin) * s->fplan.bandFloats;
      if (cudaMalloc(&s->bands, 2 * s->bandsPerBuf * 4) != cudaSuccess ||
          cudaMalloc(&s->xpad, nPad * 4) != cudaSuccess) {
         cudaGetLastError();  // no fused steps
         if (s->bands) cudaFree(s->bands);
         if (s->xpad) cudaFree(s->xpad);
         s->bands = nullptr;
         s->xpad = nullptr;
         std::memset(&s->fplan, 0, sizeof(s->fplan));
      }
   }
   s->rplan = make_recon_plan(g, S, P, C, false, g_num_sms);
   s->rplanX3 = make_recon_plan(g, S, P, C, true, g_num_sms);
   s->maxRecon[0] = s->maxRecon[1] = g_num_sms;
   dispatch(S, P, C, [&](auto L) {
      // as many CTAs as can be resident together (the kernel is persistent)
      for (int x3 = 0; x3 < 2; x3++) {
         ReconPlan &rp = x3 ? s->rplanX3 : s->rplan;
         const int n = L.max_recon_ctas(rp, x3 != 0);
         if (n > 0) {
            s->maxRecon[x3] = std::min(n, g_num_sms);
            rp = make_recon_plan(g, S, P, C, x3 != 0, s->maxRecon[x3]);
         }
      }
      return PVGPU_OK;
   });
   bool fits = true;
   dispatch(S, P, C, [&](auto L) {
      fits = L.fits(s, false);
      return PVGPU_OK;
   });
   if (!fits) {
      free_solver(s);
      return PVGPU_ERR_UNSUPPORTED_SHAPE;
   }
   pvgpu_status ra = dispatch(S, P, C, [&](auto L) { return L.set_attrs(s); });
   if (ra == PVGPU_OK && cudaStreamCreateWithFlags(&s->capStream, cudaStreamNonBlocking) != cudaSuccess) {
      cudaGetLastError();
      s->capStream = nullptr;  // runs then launch kernel by kernel
   }
   if (s->capStream && (cudaStreamCreateWithFlags(&s->capStream2, cudaStreamNonBlocking) != cudaSuccess ||
                        cudaEventCreateWithFlags(&s->forkEv, cudaEventDisableTiming) != cudaSuccess ||
                        cudaEventCreateWithFlags(&s->joinEv, cudaEventDisableTiming) != cudaSuccess)) {
      cudaGetLastError();  // one chain only
      if (s->capStream2) cudaStreamDestroy(s->capStream2);
      s->capStream2 = nullptr;
   }
   apply_tuned(s);  // shapes (only ones that fit) and schedule an earlier autotune picked, if any
   if (ra != PVGPU_OK) {
      free_solver(s);
      return ra;
   }
   *out = s;
   return PVGPU_OK;
}

extern "C" pvgpu_status pvgpu_lca_solver_destroy(pvgpu_lca_solver *s) {
   if (!s) return PVGPU_ERR_BAD_ARG;
   free_solver(s);
   return PVGPU_OK;
}

extern "C" pvgpu_status pvgpu_lca_solver_set_weights(pvgpu_lca_solver *s, const float *w, void *stream) {
   if (!s || !w) return PVGPU_ERR_BAD_ARG;
   int n = s->g.F * s->KP;
   prep_weights_kernel<<<(n + 255) / 256, 256, 0, pvgpu::as_stream(stream)>>>(w, s->g.F, s->KP, s->W, s->Wlo, s->Wt,
                                                                           s->Wtlo, s->W32, s->Wt32);
   PVGPU_CHECK_LAUNCH("lca set_weights");
   s->weightsSet = true;
   return PVGPU_OK;
}

extern "C" pvgpu_status pvgpu_lca_solver_reset(pvgpu_lca_solver *s, const float *v0, void *stream) {
   if (!s) return PVGPU_ERR_BAD_ARG;
   cudaStream_t st = pvgpu::as_stream(stream);
   size_t n = (size_t)s->g.nb * s->g.Npos * s->g.F;
   if (v0) {
      v_layout_kernel<<<152 * 8, 256, 0, st>>>(s->g, v0, s->V, 1);
      PVGPU_CHECK_LAUNCH("lca reset");
   } else {
      PVGPU_CUDA(cudaMemsetAsync(s->V, 0, n * 4, st), "lca reset");
   }
   init_activity_kernel<<<152 * 8, 256, 0, st>>>(s->g, s->V, s->A, s->Alo, s->A32);
   PVGPU_CHECK_LAUNCH("lca reset");
   PVGPU_CUDA(cudaMemsetAsync(s->err, 0, sizeof(int), st), "lca reset");
   s->stepsRun = 0;
   s->padValid = false;
   return PVGPU_OK;
}

extern "C" pvgpu_status pvgpu_lca_solver_run(pvgpu_lca_solver *s, const float *x, int numSteps, int numX3Steps,
                                             int precision, void *stream) {
   if (!s || !x || numSteps < 0 || numX3Steps < 0 || numX3Steps > numSteps) return PVGPU_ERR_BAD_ARG;
   if (!s->weightsSet) return PVGPU_ERR_BAD_ARG;
   cudaStream_t st = pvgpu::as_stream(stream);
   if (precision == PVGPU_LCA_FP32) {
      for (int t = 0; t < numSteps; t++) {
         const bool rec = s->profiling && s->evNext + 3 <= s->ev.size();
         if (rec) cudaEventRecord(s->ev[s->evNext], st);
         pvgpu_status r = pvgpu::lca_fp32_step(s->S, s->P, s->C, s->g, x, s->W32, s->Wt32, s->partials, s->V, s->A32,
                                               st, rec ? s->ev[s->evNext + 1] : nullptr);
         if (r != PVGPU_OK) return r;
         if (rec) {
            cudaEventRecord(s->ev[s->evNext + 2], st);
            s->evNext += 3;
         }
      }
      s->stepsRun += numSteps;
      if (numSteps > 0) s->padValid = false;
      return PVGPU_OK;
   }
   if (precision != PVGPU_LCA_BF16) return PVGPU_ERR_BAD_ARG;
   bool x3ok = true;
   if (numX3Steps > 0) {
      dispatch(s->S, s->P, s->C, [&](auto L) {
         x3ok = L.fits(s, true);
         return PVGPU_OK;
      });
      if (!x3ok) return PVGPU_ERR_UNSUPPORTED_SHAPE;
   }
   if (numSteps > 0 && !s->profiling && s->capStream) {
      // the whole run as one CUDA graph (programmatic edges between the kernels of a chain)
      if (!s->graph || s->graphX != x || s->graphSteps != numSteps || s->graphX3 != numX3Steps) {
         if (s->graph) cudaGraphExecDestroy(s->graph);
         s->graph = nullptr;
         PVGPU_CUDA(cudaStreamBeginCapture(s->capStream, cudaStreamCaptureModeThreadLocal), "lca graph capture");
         pvgpu_status r = PVGPU_OK;
         if (s->sched.chains == 2) {  // the second half's chain on a branch of its own, joined at the end
            cudaEventRecord(s->forkEv, s->capStream);
            cudaStreamWaitEvent(s->capStream2, s->forkEv, 0);
            r = enqueue_run(s, x, numSteps, numX3Steps, 0, s->capStream, false);
            if (r == PVGPU_OK) r = enqueue_run(s, x, numSteps, numX3Steps, 1, s->capStream2, false);
            cudaEventRecord(s->joinEv, s->capStream2);
            cudaStreamWaitEvent(s->capStream, s->joinEv, 0);
         } else {
            r = enqueue_run(s, x, numSteps, numX3Steps, -1, s->capStream, false);
         }
         cudaGraph_t g = nullptr;
         cudaError_t ee = cudaStreamEndCapture(s->capStream, &g);
         if (r != PVGPU_OK || ee != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            if (r == PVGPU_OK) r = pvgpu::record_cuda_error(ee, "lca graph capture");
            return r;
         }
         cudaError_t ei = cudaGraphInstantiate(&s->graph, g, 0);
         cudaGraphDestroy(g);
         if (ei != cudaSuccess) {
            s->graph = nullptr;
            return pvgpu::record_cuda_error(ei, "lca graph instantiate");
         }
         s->graphX = x;
         s->graphSteps = numSteps;
         s->graphX3 = numX3Steps;
      }
      PVGPU_CUDA(cudaGraphLaunch(s->graph, st), "lca graph launch");
   } else {
      pvgpu_status r = enqueue_run(s, x, numSteps, numX3Steps, -1, st, s->profiling);
      if (r != PVGPU_OK) return r;
   }
   s->stepsRun += numSteps;
   if (numSteps > 0) s->padValid = true;
   return PVGPU_OK;
}

extern "C" pvgpu_status pvgpu_lca_solver_energy(pvgpu_lca_solver *s, const float *x, double l2Coeff, int costKind,
                                                double costThresh, double costWidth, double costCoeff,
                                                double *energy, void *stream) {
   if (!s || !x || !energy || (costKind != 1 && costKind != 2)) return PVGPU_ERR_BAD_ARG;
   energy_kernel<<<s->g.nb, 256, 0, pvgpu::as_stream(stream)>>>(s->g, s->C, x, s->partials,
                                                                s->padValid ? s->rpad : nullptr, s->rplan.rowsPad * s->rplan.RP,
                                                                s->V, l2Coeff, costKind, costThresh, costWidth,
                                                                costCoeff, energy);
   PVGPU_CHECK_LAUNCH("lca energy");
   return PVGPU_OK;
}

extern "C" pvgpu_status pvgpu_lca_solver_state(pvgpu_lca_solver *s, float *v, float *a, void *stream) {
   if (!s) return PVGPU_ERR_BAD_ARG;
   cudaStream_t st = pvgpu::as_stream(stream);
   if (v) {
      v_layout_kernel<<<152 * 8, 256, 0, st>>>(s->g, s->V, v, 0);
      PVGPU_CHECK_LAUNCH("lca state");
   }
   if (a) {
      activity_out_kernel<<<152 * 8, 256, 0, st>>>(s->g, s->V, a);
      PVGPU_CHECK_LAUNCH("lca state");
   }
   return PVGPU_OK;
}

extern "C" pvgpu_status pvgpu_lca_solver_error_flag(pvgpu_lca_solver *s, int *hostFlag) {
   if (!s || !hostFlag) return PVGPU_ERR_BAD_ARG;
   PVGPU_CUDA(cudaMemcpy(hostFlag, s->err, sizeof(int), cudaMemcpyDeviceToHost), "lca error flag");
   return PVGPU_OK;
}

extern "C" pvgpu_status pvgpu_lca_solver_profile_begin(pvgpu_lca_solver *s, int maxSteps) {
   if (!s || maxSteps < 0) return PVGPU_ERR_BAD_ARG;
   size_t need = (size_t)maxSteps * 3;
   while (s->ev.size() < need) {
      cudaEvent_t e;
      PVGPU_CUDA(cudaEventCreate(&e), "lca profile");
      s->ev.push_back(e);
   }
   s->evKind.assign((size_t)maxSteps, 0);
   s->evNext = 0;
   s->profiling = true;
   return PVGPU_OK;
}

namespace {

// Kernel R and kernel P times summed over n timesteps of x, launched one by one with events.
pvgpu_status time_steps(pvgpu_lca_solver *s, const float *x, int n, bool x3, void *stream, double *r, double *p,
                        double *f = nullptr) {
   pvgpu_status st = pvgpu_lca_solver_profile_begin(s, n);
   if (st != PVGPU_OK) return st;
   st = pvgpu_lca_solver_run(s, x, n, x3 ? n : 0, PVGPU_LCA_BF16, stream);
   int k = 0, kf = 0;
   double fm = 0.0;
   pvgpu_status st2 = pvgpu_lca_solver_profile_end_fused(s, r, p, &fm, &k, &kf);
   if (f) *f = kf > 0 ? fm / kf : 1e30;
   return st != PVGPU_OK ? st : st2;
}

}  // namespace

extern "C" pvgpu_status pvgpu_lca_solver_autotune(pvgpu_lca_solver *s, const float *x, int trialSteps, void *stream) {
   if (!s || !x || trialSteps <= 0 || !s->weightsSet) return PVGPU_ERR_BAD_ARG;
   TunedShapes best;
   const PostPlan keepP[2] = {s->plan, s->planX3};
   const ReconPlan keepR[2] = {s->rplan, s->rplanX3};
   const int fusedKeep = s->sched.fused;
   s->sched.fused = 0;  // kernels R and P on every step while their shapes are timed
   best.fuse[0] = s->fplan.FT;
   best.fuse[1] = s->fplan.nV;
   best.fuse[2] = s->fplan.nW;
   for (int x3 = 0; x3 < 2; x3++) {
      PostPlan &cur = x3 ? s->planX3 : s->plan;
      ReconPlan &curR = x3 ? s->rplanX3 : s->rplan;
      const PostPlan p0 = cur;
      const ReconPlan r0 = curR;
      best.post[x3][0] = p0.FT;
      best.post[x3][1] = p0.nV;
      best.post[x3][2] = p0.nW;
      best.post[x3][3] = p0.stageA;
      best.recon[x3] = r0.nStage;
      if (!p0.total || p0.total > kSmemBudget || r0.total > kSmemBudget) continue;  // form not offered
      // kernel P: every feature tile and ring shape that fits
      double bestMs = 1e30;
      for (int FT = 64; FT <= 512 && FT <= s->g.F; FT += 64) {
         if (s->g.F % FT || (FT & (FT - 1))) continue;  // 64, 128, 256, 512 dividing F
         for (const auto &rg : kRings) {
            PostPlan pl = post_plan_for(s->g, s->S, s->P, s->C, x3 != 0, g_num_sms, FT, rg[0], rg[1], rg[2]);
            if (!pl.total || pl.total > kSmemBudget) continue;
            cur = pl;
            double r = 0, p = 0;
            pvgpu_status st = time_steps(s, x, 1, x3 != 0, stream, &r, &p);  // warm-up
            if (st == PVGPU_OK) st = time_steps(s, x, trialSteps, x3 != 0, stream, &r, &p);
            if (st != PVGPU_OK) {
               s->plan = keepP[0];
               s->planX3 = keepP[1];
               s->sched.fused = fusedKeep;
               return st;
            }
            if (p < bestMs) {
               bestMs = p;
               best.post[x3][0] = FT;
               best.post[x3][1] = rg[0];
               best.post[x3][2] = rg[1];
               best.post[x3][3] = rg[2];
            }
         }
      }
      cur = post_plan_for(s->g, s->S, s->P, s->C, x3 != 0, g_num_sms, best.post[x3][0], best.post[x3][1],
                          best.post[x3][2], best.post[x3][3]);
      // kernel R: every ring depth that fits
      bestMs = 1e30;
      for (int n = 2; n <= kMaxRStages; n++) {
         ReconPlan rp = recon_plan_for(s->g, s->S, s->P, s->C, x3 != 0, s->maxRecon[x3], n);
         if (rp.total > kSmemBudget) continue;
         curR = rp;
         double r = 0, p = 0;
         pvgpu_status st = time_steps(s, x, 1, x3 != 0, stream, &r, &p);
         if (st == PVGPU_OK) st = time_steps(s, x, trialSteps, x3 != 0, stream, &r, &p);
         if (st != PVGPU_OK) {
            s->rplan = keepR[0];
            s->rplanX3 = keepR[1];
            s->sched.fused = fusedKeep;
            return st;
         }
         if (r < bestMs) {
            bestMs = r;
            best.recon[x3] = n;
         }
      }
   }
   s->sched.fused = fusedKeep;
   // kernel F: every feature tile (multiple of 64 dividing F), V and weight ring depth that fits,
   // timed on trialSteps + 2 BF16 steps (all but the first and last fused)
   if (s->bands && s->fplan.total) {
      const FusePlan keepF = s->fplan;
      const int fusedWas = s->sched.fused;
      s->sched.fused = 1;
      double bestMs = 1e30;
      for (int FT = 64; FT <= 512 && FT <= s->g.F; FT += 64) {
         for (int nV = 2; nV <= 4; nV += 2) {
            for (int nW = 2; nW <= 4; nW++) {
               FusePlan fp = fuse_plan_for(s->g, s->S, s->P, s->C, g_num_sms, FT, nV, nW);
               if (!fp.total || fp.total > kSmemBudget) continue;
               if ((size_t)s->g.nb * s->g.MB * (s->g.F / FT) * fp.bandFloats > s->bandsPerBuf) continue;
               s->fplan = fp;
               double r = 0, p = 0, f = 0;
               pvgpu_status st = time_steps(s, x, 3, false, stream, &r, &p, &f);  // warm-up
               if (st == PVGPU_OK) st = time_steps(s, x, trialSteps + 2, false, stream, &r, &p, &f);
               if (st != PVGPU_OK) {
                  s->fplan = keepF;
                  s->sched.fused = fusedWas;
                  return st;
               }
               if (f < bestMs) {
                  bestMs = f;
                  best.fuse[0] = FT;
                  best.fuse[1] = nV;
                  best.fuse[2] = nW;
               }
            }
         }
      }
      s->sched.fused = fusedWas;
   }
   best.sched = s->sched;
   set_shapes(s, best);
   // the graph schedule: each candidate replayed as a graph of max(trialSteps, 16) BF16 steps,
   // best of two replays
   {
      const int n = std::max(trialSteps, 16);
      // one or two chains, with and without programmatic edges, and two chains with the persistent
      // grids of kernels P and F capped (each chain's last wave then leaves whole SMs to the other)
      const int fz = s->sched.fused;
      const int cap1 = (g_num_sms * 5 / 6) & ~1, cap2 = (g_num_sms * 2 / 3) & ~1;
      const pvgpu_lca_schedule cands[6] = {{1, 0, 0, 1, fz}, {1, 0, 0, 0, fz},    {2, 0, 0, 1, fz},
                                           {2, 0, 0, 0, fz}, {2, 0, cap1, 1, fz}, {2, 0, cap2, 1, fz}};
      cudaStream_t st = pvgpu::as_stream(stream);
      cudaEvent_t e0 = nullptr, e1 = nullptr;
      if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
         if (e0) cudaEventDestroy(e0);
         return pvgpu::record_cuda_error(cudaGetLastError(), "lca autotune events");
      }
      double bestMs = 1e30;
      pvgpu_status st2 = PVGPU_OK;
      for (const pvgpu_lca_schedule &c : cands) {
         if (pvgpu_lca_solver_set_schedule(s, &c) != PVGPU_OK) continue;  // no second half
         st2 = pvgpu_lca_solver_run(s, x, n, 0, PVGPU_LCA_BF16, stream);  // captures the graph
         for (int rep = 0; rep < 2 && st2 == PVGPU_OK; rep++) {
            cudaEventRecord(e0, st);
            st2 = pvgpu_lca_solver_run(s, x, n, 0, PVGPU_LCA_BF16, stream);
            cudaEventRecord(e1, st);
            float ms = 0.0f;
            if (st2 == PVGPU_OK && cudaEventSynchronize(e1) == cudaSuccess &&
                cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess && ms < bestMs) {
               bestMs = ms;
               best.sched = c;
            }
         }
         if (st2 != PVGPU_OK) break;
      }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      s->sched = best.sched;
      if (s->graph) cudaGraphExecDestroy(s->graph);
      s->graph = nullptr;
      if (st2 != PVGPU_OK) return st2;
   }
   std::lock_guard<std::mutex> lk(g_tune_mu);
   g_tuned[tune_key(s)] = best;
   return PVGPU_OK;
}

extern "C" pvgpu_status pvgpu_lca_solver_plan_info(const pvgpu_lca_solver *s, int *out) {
   if (!s || !out) return PVGPU_ERR_BAD_ARG;
   for (int x3 = 0; x3 < 2; x3++) {
      const PostPlan &pl = x3 ? s->planX3 : s->plan;
      const ReconPlan &rp = x3 ? s->rplanX3 : s->rplan;
      int *o = out + 5 * x3;
      o[0] = pl.FT;
      o[1] = pl.nV;
      o[2] = pl.nW;
      o[3] = pl.stageA;
      o[4] = rp.nStage;
   }
   return PVGPU_OK;
}

extern "C" pvgpu_status pvgpu_lca_solver_fused_plan_info(const pvgpu_lca_solver *s, int *out) {
   if (!s || !out) return PVGPU_ERR_BAD_ARG;
   const bool ok = s->bands && s->fplan.total && s->fplan.total <= kSmemBudget;
   out[0] = ok ? s->fplan.FT : 0;
   out[1] = ok ? s->fplan.nV : 0;
   out[2] = ok ? s->fplan.nW : 0;
   return PVGPU_OK;
}

extern "C" pvgpu_status pvgpu_lca_solver_set_fused_plan(pvgpu_lca_solver *s, int featureTile, int vSlots, int wSlots) {
   if (!s) return PVGPU_ERR_BAD_ARG;
   if (!s->bands) return PVGPU_ERR_UNSUPPORTED_SHAPE;
   FusePlan fp = fuse_plan_for(s->g, s->S, s->P, s->C, g_num_sms, featureTile, vSlots, wSlots);
   if (!fp.total || fp.total > kSmemBudget ||
       (size_t)s->g.nb * s->g.MB * (s->g.F / featureTile) * fp.bandFloats > s->bandsPerBuf)
      return PVGPU_ERR_UNSUPPORTED_SHAPE;
   s->fplan = fp;
   if (s->graph) cudaGraphExecDestroy(s->graph);
   s->graph = nullptr;
   return PVGPU_OK;
}

extern "C" pvgpu_status pvgpu_lca_solver_set_schedule(pvgpu_lca_solver *s, const pvgpu_lca_schedule *sc) {
   if (!s || !sc || (sc->chains != 1 && sc->chains != 2) || sc->reconCtas < 0 || sc->postCtas < 0 ||
       (sc->programmatic != 0 && sc->programmatic != 1) || (sc->fused != 0 && sc->fused != 1))
      return PVGPU_ERR_BAD_ARG;
   if (sc->chains == 2 && (s->g.nb < 2 || !s->capStream2)) return PVGPU_ERR_UNSUPPORTED_SHAPE;
   s->sched = *sc;
   if (s->graph) cudaGraphExecDestroy(s->graph);
   s->graph = nullptr;
   return PVGPU_OK;
}

extern "C" pvgpu_status pvgpu_lca_solver_get_schedule(const pvgpu_lca_solver *s, pvgpu_lca_schedule *sc) {
   if (!s || !sc) return PVGPU_ERR_BAD_ARG;
   *sc = s->sched;
   return PVGPU_OK;
}

extern "C" pvgpu_status pvgpu_lca_solver_profile_end_fused(pvgpu_lca_solver *s, double *reconMs, double *postMs,
                                                           double *fusedMs, int *steps, int *fusedSteps) {
   if (!s || !reconMs || !postMs || !fusedMs || !steps || !fusedSteps) return PVGPU_ERR_BAD_ARG;
   s->profiling = false;
   double r = 0.0, p = 0.0, f = 0.0;
   int n = (int)(s->evNext / 3), nf = 0;
   if (n > 0) PVGPU_CUDA(cudaEventSynchronize(s->ev[s->evNext - 1]), "lca profile");
   for (int i = 0; i < n; i++) {
      float a = 0.0f, b = 0.0f;
      PVGPU_CUDA(cudaEventElapsedTime(&a, s->ev[3 * i], s->ev[3 * i + 1]), "lca profile");
      PVGPU_CUDA(cudaEventElapsedTime(&b, s->ev[3 * i + 1], s->ev[3 * i + 2]), "lca profile");
      r += a;
      if (s->evKind[i] == 0) {
         p += b;
      } else {
         f += b;
         nf++;
      }
   }
   *reconMs = r;
   *postMs = p;
   *fusedMs = f;
   *steps = n;
   *fusedSteps = nf;
   s->evNext = 0;
   return PVGPU_OK;
}

extern "C" pvgpu_status pvgpu_lca_solver_profile_end(pvgpu_lca_solver *s, double *reconMs, double *postMs, int *steps) {
   if (!s || !reconMs || !postMs || !steps) return PVGPU_ERR_BAD_ARG;
   double f = 0.0;
   int nf = 0;
   pvgpu_status st = pvgpu_lca_solver_profile_end_fused(s, reconMs, postMs, &f, steps, &nf);
   *postMs += f;
   return st;
}
