// tc_ptx.cuh -- inline-PTX building blocks for the Blackwell (sm_103a) tensor-core path:
// mbarriers with bounded waits, TMA tile loads, tcgen05 TMEM allocation, tcgen05.mma
// (kind::f16, BF16 inputs, FP32 accumulation in TMEM), tcgen05.commit and tcgen05.ld.
//
// Shared-memory operand layout: K-major, 128-byte swizzle (the layout a TMA load with
// CU_TENSOR_MAP_SWIZZLE_128B writes for a box whose inner extent is 64 BF16 elements).
// Rows are 128 B; the 16-byte chunk c of row r sits at chunk c ^ (r % 8); 8-row atoms are
// 1024 B apart.  Tiles start on 1024-byte boundaries.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <stdint.h>

namespace pvgpu {
namespace tc {

// Time limit of every device-side wait, in ns of the global timer: far beyond any legitimate
// latency inside one launch (the longest waits here are a few microseconds); after it the
// kernel records a timeout and returns.  Waits are bounded by elapsed time, not by a count of
// probes, because one mbarrier.try_wait may suspend the thread for a system-dependent interval.
constexpr uint64_t kWaitNs = 200ull * 1000ull * 1000ull;

__device__ __forceinline__ uint64_t global_ns() {
   uint64_t t;
   asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
   return t;
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
   return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// ---- mbarrier -------------------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
   asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
   asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
   asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
   uint32_t ok;
   asm volatile(
         "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
         : "=r"(ok)
         : "r"(smem_u32(bar)), "r"(parity)
         : "memory");
   return ok != 0;
}

// Non-blocking test of the phase with the given parity (never suspends the thread).
__device__ __forceinline__ bool mbar_test(uint64_t *bar, uint32_t parity) {
   uint32_t ok;
   asm volatile(
         "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
         : "=r"(ok)
         : "r"(smem_u32(bar)), "r"(parity)
         : "memory");
   return ok != 0;
}

// Wait for the phase with the given parity, for at most limitNs of elapsed time (the clock is
// read once per 64 probes); false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint64_t limitNs = kWaitNs) {
   if (mbar_try_wait(bar, parity)) return true;
   const uint64_t t0 = global_ns();
   for (;;) {
      for (int i = 0; i < 64; i++)
         if (mbar_try_wait(bar, parity)) return true;
      if (global_ns() - t0 > limitNs) return false;
   }
}

// ---- TMA -------------------------------------------------------------------------------
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int c0, int c1) {
   asm volatile(
         "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
         ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(smem_u32(bar))
         : "memory");
}

__device__ __forceinline__ void prefetch_tmap(const CUtensorMap *map) {
   asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// Generic-proxy shared-memory writes become visible to the async proxy (tcgen05.mma operands).
__device__ __forceinline__ void fence_proxy_async_smem() {
   asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ---- TMEM ------------------------------------------------------------------------------
// Whole warp: allocate ncols (power of two, >= 32) TMEM columns; the address lands in *dst.
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
   asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
                : "memory");
   asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
   asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
   asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_after() {
   asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// ---- descriptors -------------------------------------------------------------------------
// Shared-memory matrix descriptor, K-major with 128-byte swizzle: start address, leading
// byte offset (unused for this layout, 16 B), stride byte offset 1024 B between 8-row
// atoms, descriptor version 1, swizzle mode 2 (128B).
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t smem_addr) {
   uint64_t d = 0;
   d |= (uint64_t)((smem_addr >> 4) & 0x3FFFu);
   d |= (uint64_t)(16u >> 4) << 16;
   d |= (uint64_t)(1024u >> 4) << 32;
   d |= (uint64_t)1 << 46;
   d |= (uint64_t)2 << 61;
   return d;
}

// Descriptor of an MN-major operand in 128-byte swizzled tiles: 128-byte rows along K (64 BF16
// values of consecutive M / N each), 8-row swizzle atoms 1024 B apart along K (SBO), and groups
// of 64 M / N values lbo bytes apart (LBO) -- a K-major SW128 tile of the transposed matrix read
// the other way round.
__device__ __forceinline__ uint64_t sdesc_sw128_mn(uint32_t smem_addr, uint32_t lbo) {
   uint64_t d = 0;
   d |= (uint64_t)((smem_addr >> 4) & 0x3FFFu);
   d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
   d |= (uint64_t)(1024u >> 4) << 32;
   d |= (uint64_t)1 << 46;
   d |= (uint64_t)2 << 61;
   return d;
}

// Instruction descriptor, kind::f16: D = FP32, A = B = BF16, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
   return (1u << 4)                        // D format F32
          | (1u << 7)                      // A format BF16
          | (1u << 10)                     // B format BF16
          | ((uint32_t)(N >> 3) << 17)     // N / 8
          | ((uint32_t)(M >> 4) << 24);    // M / 16
}

// The same with B MN-major (transpose-B bit).
__host__ __device__ constexpr uint32_t idesc_bf16_bmn(int M, int N) { return idesc_bf16(M, N) | (1u << 16); }

// D[tmem] (+)= A[smem] * B[smem]^T, one instruction (M x N x 16), issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
   asm volatile(
         "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
         " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
         "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
         : "memory");
}

// Arrive on *bar once every tcgen05.mma this thread issued so far has completed.
// D[tmem] (+)= A[tmem] * B[smem]^T (M x N x 16, kind::f16): A is read from tensor memory, row m
// in lane m, two consecutive K elements per 32-bit column (8 columns per instruction).
__device__ __forceinline__ void mma_bf16_ta(uint32_t d_tmem, uint32_t a_tmem, uint64_t bdesc, uint32_t idesc,
                                            uint32_t accumulate) {
   asm volatile(
         "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
         " tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}\n" ::"r"(d_tmem),
         "r"(a_tmem), "l"(bdesc), "r"(idesc), "r"(accumulate)
         : "memory");
}

// Warp-collective: 8 consecutive 32-bit columns of this warp's 32 TMEM lanes from registers.
__device__ __forceinline__ void tmem_st8(uint32_t taddr, const uint32_t *r) {
   asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr), "r"(r[0]),
                "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7])
                : "memory");
}

// Stores issued by this thread have completed (before a fence and the hand-off to the MMA).
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
   asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                : "memory");
}

// Warp-collective: 32 consecutive FP32 columns of this warp's 32 TMEM lanes.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float *v) {
   uint32_t r[32];
   asm volatile(
         "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
         "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
         : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
           "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
           "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
           "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
         : "r"(taddr));
   asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
   for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// Byte offset of element (row, k) of a K-major SW128 BF16 tile with 64-element rows.
__host__ __device__ __forceinline__ uint32_t sw128_offset(int row, int k) {
   int chunk = k >> 3;  // 8 BF16 = 16 B
   return (uint32_t)(row * 128 + (((chunk ^ (row & 7)) << 4)) + ((k & 7) << 1));
}

}  // namespace tc
}  // namespace pvgpu

namespace pvgpu {
namespace tc {

// ---- bulk copies and TMA stores ------------------------------------------------------------
// Contiguous global -> shared copy (16-byte aligned addresses, size a multiple of 16) that
// completes on an mbarrier.
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
   asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(smem_u32(bar))
                : "memory");
}

// Contiguous shared -> global copy (16-byte aligned addresses, size a multiple of 16),
// bulk-group completion.
__device__ __forceinline__ void bulk_store(void *dst, const void *src, uint32_t bytes) {
   asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(reinterpret_cast<uint64_t>(dst)),
                "r"(smem_u32(src)), "r"(bytes)
                : "memory");
}

// Tiled shared -> global store through a tensor map (bulk-group completion).
__device__ __forceinline__ void tma_store_2d(const CUtensorMap *map, const void *src, int c0, int c1) {
   asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%2, %3}], [%1];"
                ::"l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(src)), "r"(c0), "r"(c1)
                : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }

// Wait until the bulk stores committed by this thread have finished reading shared memory.
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }

// Wait until all but the most recent bulk-store group of this thread have read shared memory.
__device__ __forceinline__ void bulk_wait_read_1() { asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory"); }

// Wait until the bulk stores committed by this thread have completed.
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

}  // namespace tc
}  // namespace pvgpu

namespace pvgpu {
namespace tc {

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
   asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// One 32-byte global store (address 32-byte aligned).
__device__ __forceinline__ void st_global_32B(void *p, uint4 a, uint4 b) {
   asm volatile("st.global.v8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"l"(p), "r"(a.x), "r"(a.y), "r"(a.z), "r"(a.w),
                "r"(b.x), "r"(b.y), "r"(b.z), "r"(b.w)
                : "memory");
}

// ---- programmatic dependent launch ---------------------------------------------------------
// Let the next kernel in the stream be scheduled once every CTA of this grid has passed here
// (or exited); its CTAs then occupy SMs as this grid's CTAs leave them.
__device__ __forceinline__ void griddep_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Wait until the grids this one depends on have completed and their memory is visible.
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }


// Barrier among `count` threads (a multiple of 32) on hardware barrier `id` (1..15).
__device__ __forceinline__ void named_bar_sync(int id, int count) {
   asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}

// Barrier like named_bar_sync that also returns the OR of `pred` over the participating
// threads, so a decision taken after it is the same in every thread.
__device__ __forceinline__ bool named_bar_or(int id, int count, bool pred) {
   uint32_t r;
   asm volatile(
         "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.or.pred q, %2, %3, p;\n selp.u32 %0, 1, 0, q;\n}\n"
         : "=r"(r)
         : "r"((uint32_t)pred), "r"(id), "r"(count)
         : "memory");
   return r != 0;
}

}  // namespace tc
}  // namespace pvgpu

namespace pvgpu {
namespace tc {

// ---- TF32 operands (kind::tf32) ------------------------------------------------------------
// 3-D TMA tile load (coordinates innermost first) completing on an mbarrier.
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, uint64_t *bar, int c0, int c1, int c2) {
   asm volatile(
         "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
         ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
         : "memory");
}

// FP32 -> TF32 (round to nearest, ties away from zero), returned as an FP32 whose low 13
// mantissa bits are zero.
__device__ __forceinline__ float to_tf32(float x) {
   uint32_t r;
   asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
   return __uint_as_float(r);
}

// K-major descriptor without swizzle: 8-row x 16-byte core matrices, `lbo` bytes between core
// matrices along K, `sbo` bytes between 8-row groups along M/N.  With sbo = 128 the rows of a
// 16-byte K chunk sit 16 B apart, so an operand may start at any row of such a column.
__device__ __forceinline__ uint64_t sdesc_noswizzle(uint32_t smem_addr, uint32_t lbo, uint32_t sbo) {
   uint64_t d = 0;
   d |= (uint64_t)((smem_addr >> 4) & 0x3FFFu);
   d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
   d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
   d |= (uint64_t)1 << 46;
   return d;  // swizzle mode 0
}

// Warp-collective: 16 consecutive FP32 columns of this warp's 32 TMEM lanes.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
   uint32_t r[16];
   asm volatile(
         "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
         : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
           "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
         : "r"(taddr));
   asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
   for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// Instruction descriptor, kind::tf32: D = FP32, A = B = TF32, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
   return (1u << 4)                        // D format F32
          | (2u << 7)                      // A format TF32
          | (2u << 10)                     // B format TF32
          | ((uint32_t)(N >> 3) << 17)     // N / 8
          | ((uint32_t)(M >> 4) << 24);    // M / 16
}

// D[tmem] (+)= A[smem] * B[smem]^T, one instruction (M x N x 8, TF32), issued by one thread.
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
   asm volatile(
         "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
         " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
         "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
         : "memory");
}

}  // namespace tc
}  // namespace pvgpu
