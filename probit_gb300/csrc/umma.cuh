// Blackwell (sm_100a / sm_103a) tensor-core primitives in inline PTX:
// tensor-memory allocation, tcgen05.mma (kind::tf32) with shared-memory
// operand descriptors, commit to mbarriers, and tcgen05.ld of the fp32
// accumulator.  Used by the 3xTF32 tile products of the factorisation.
//
// Operand layout: K-major, 128-byte swizzle (the canonical SW128 layout):
// a 128-row x 32-fp32 (128 B) chunk is stored row after row at a 128-byte
// pitch, 8-row groups 1024 B apart, and inside each row the 16-byte unit u is
// stored at position u ^ (row & 7).  The chunk base must be 1024-byte aligned.
#pragma once

#include <stdint.h>

#include "common.cuh"

namespace pgb {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// ---------------------------------------------------------------- TMEM
// One full warp allocates `ncols` columns (power of two >= 32) and writes the
// base address to shared memory.
__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst_smem)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Make this thread's generic-proxy shared-memory writes visible to the async
// proxy (tcgen05.mma operand reads).
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ---------------------------------------------------------------- descriptors
// Instruction descriptor of kind::tf32: D = F32, A = B = TF32, both K-major,
// dense, M x N with M in {64, 128}, N multiple of 8 (<= 256).
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4)                        // D format: F32
         | (2u << 7)                      // A format: TF32
         | (2u << 10)                     // B format: TF32
         | ((uint32_t)(N >> 3) << 17)     // N / 8
         | ((uint32_t)(M >> 4) << 24);    // M / 16
}

// Shared-memory matrix descriptor for a K-major SW128 operand starting at
// `saddr` (byte address in shared memory).  SBO = 1024 B between 8-row
// groups; LBO is not used by swizzled K-major layouts (set to 1); version 1.
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1u << 16;                  // LBO (unused for SW128 K-major)
  d |= (uint64_t)(1024u >> 4) << 32;        // SBO
  d |= (uint64_t)1u << 46;                  // descriptor version
  d |= (uint64_t)2u << 61;                  // layout: SWIZZLE_128B
  return d;
}

// The same for a K-major SW64 operand (64-byte rows, 8-row groups 512 B
// apart; the chunk base 512-byte aligned).
__device__ __forceinline__ uint64_t sdesc_sw64(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1u << 16;                  // LBO (unused for swizzled K-major)
  d |= (uint64_t)(512u >> 4) << 32;         // SBO
  d |= (uint64_t)1u << 46;                  // descriptor version
  d |= (uint64_t)4u << 61;                  // layout: SWIZZLE_64B
  return d;
}

// ---------------------------------------------------------------- MMA
__device__ __forceinline__ void umma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// Same with the A operand in tensor memory at `a_tmem` (M lanes x K columns,
// one 32-bit element per column).
__device__ __forceinline__ void umma_tf32_ts(uint32_t d_tmem, uint32_t a_tmem, uint64_t bdesc, uint32_t idesc,
                                             uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "r"(a_tmem), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// The mbarrier receives one arrive when every tcgen05 operation issued so far
// by this thread has completed.
__device__ __forceinline__ void umma_commit(uint64_t* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
               : "memory");
}

// ---------------------------------------------------------------- TMEM -> registers
// 32 lanes x 32 consecutive fp32 columns: thread t of the warp receives lane
// (taddr lane + t), columns taddr col .. col+31.
__device__ __forceinline__ void tmem_ld_32x32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// registers -> TMEM: thread t of the warp writes lane (taddr lane + t),
// columns taddr col .. col+31.
__device__ __forceinline__ void tmem_st_32x32(uint32_t taddr, const float (&v)[32]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], "
      "{%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, "
      "%17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, %32};" ::"r"(taddr),
      "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])), "r"(__float_as_uint(v[3])),
      "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])), "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])),
      "r"(__float_as_uint(v[8])), "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),
      "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])), "r"(__float_as_uint(v[15])),
      "r"(__float_as_uint(v[16])), "r"(__float_as_uint(v[17])), "r"(__float_as_uint(v[18])), "r"(__float_as_uint(v[19])),
      "r"(__float_as_uint(v[20])), "r"(__float_as_uint(v[21])), "r"(__float_as_uint(v[22])), "r"(__float_as_uint(v[23])),
      "r"(__float_as_uint(v[24])), "r"(__float_as_uint(v[25])), "r"(__float_as_uint(v[26])), "r"(__float_as_uint(v[27])),
      "r"(__float_as_uint(v[28])), "r"(__float_as_uint(v[29])), "r"(__float_as_uint(v[30])), "r"(__float_as_uint(v[31]))
      : "memory");
}
// 16 consecutive columns of this warp's 32 lanes (lane = thread's lane).
__device__ __forceinline__ void tmem_st_32x32_x16(uint32_t taddr, const float (&v)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
      "{%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16};" ::"r"(taddr),
      "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])), "r"(__float_as_uint(v[3])),
      "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])), "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])),
      "r"(__float_as_uint(v[8])), "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),
      "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])), "r"(__float_as_uint(v[15]))
      : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// ---------------------------------------------------------------- mbarrier
__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_u32(mbar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for the phase of `parity` to complete; false after the time
// limit (the caller raises the abort word).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* mbar, uint32_t parity, uint64_t limit_ns) {
  if (mbar_try_wait(mbar, parity)) return true;
  const uint64_t t0 = global_ns();
  while (!mbar_try_wait(mbar, parity)) {
    if (global_ns() - t0 > limit_ns) return false;
  }
  return true;
}

// One arrive that also announces `bytes` of transaction count (TMA loads
// complete the phase when their bytes land).
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)), "r"(bytes)
               : "memory");
}
// Plain arrive (count 1).
__device__ __forceinline__ void mbar_arrive(uint64_t* mbar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(mbar)) : "memory");
}
__device__ __forceinline__ void mbar_inval(uint64_t* mbar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(mbar)) : "memory");
}

// ---------------------------------------------------------------- TMA
// 2-D tiled load of the box at (x = column, y = row) of the tensor map into
// shared memory; completes `bytes` of transaction count on `mbar`.  x * 4
// bytes must be a multiple of 16 (every caller passes a multiple of 32).
__device__ __forceinline__ void tma_load_2d(void* dst_smem, const void* tmap, int x, int y, uint64_t* mbar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
          "r"(smem_u32(dst_smem)),
      "l"(tmap), "r"(x), "r"(y), "r"(smem_u32(mbar))
      : "memory");
}
// A tensor map written to global memory by ordinary stores (or copied there
// from the host) is made visible to the tensor-copy unit by this fence.
__device__ __forceinline__ void fence_tensormap_acquire(const void* tmap) {
  asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(tmap) : "memory");
}
// Order this thread's earlier generic-proxy global accesses (and those it
// acquired from other threads) before its later async-proxy (TMA) accesses.
__device__ __forceinline__ void fence_proxy_async_global() {
  asm volatile("fence.proxy.async.global;" ::: "memory");
}

// ---------------------------------------------------------------- 3xTF32 split
// Round to the nearest TF32 value (10 explicit mantissa bits, ties away from
// zero); the result is an fp32 bit pattern whose 13 low mantissa bits are 0.
__device__ __forceinline__ float round_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// x ~ hi + lo with hi and lo both TF32 values (what the tensor core reads):
// hi = x rounded to TF32 (|x - hi| <= 2^-11 |x|), lo = (x - hi) rounded to
// TF32 (x - hi is exact in fp32), so |x - hi - lo| <= 2^-22 |x|.  (Clearing
// the 13 low bits instead and letting the tensor core truncate lo is 16x
// coarser; it tripled the gradient error of the factorisation path.)
__device__ __forceinline__ void split_tf32(float x, float& hi, float& lo) {
  hi = round_tf32(x);
  lo = round_tf32(x - hi);
}

// Split layout of an operand matrix: the TF32 hi and lo parts of every
// 128-column tile side by side, hi in the tile's first 128 columns of the
// split row and lo in the next 128, so a split matrix of a logical rows x ld
// fp32 matrix has 2 ld columns.  Logical column `col` has its hi part at
// split column split_col(col) and its lo part 128 columns further on; a
// 32-column chunk of either part is one 128 x 32 tensor-map box.
__host__ __device__ __forceinline__ int split_col(int col) { return ((col >> 7) << 8) + (col & 127); }

// x as its hi/lo pair at p[0] (hi) and p[128] (lo).
__device__ __forceinline__ void put_split(float* p, float x) {
  float hi, lo;
  split_tf32(x, hi, lo);
  p[0] = hi;
  p[128] = lo;
}

__device__ __forceinline__ uint32_t sw128_offset(int row, int unit) {
  return (uint32_t)(row * 128 + ((unit ^ (row & 7)) << 4));
}

}  // namespace pgb
