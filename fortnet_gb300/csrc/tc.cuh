// Blackwell (sm_103a) tensor-core primitives written as inline PTX: tensor memory (TMEM)
// allocation, tcgen05.mma of kind::f16 (BF16 operands, FP32 accumulators in TMEM), its commit
// to an mbarrier, TMEM loads into registers, and bulk global->shared copies completed on an
// mbarrier.  Every wait on an mbarrier is bounded: it gives up after a fixed number of polls
// and reports it, so that a kernel can record an error and return instead of hanging.
//
// Operand layout (no swizzle).  A matrix of BF16 values is stored in "core matrices" of 8 rows
// x 16 bytes (8 values), each core matrix 128 contiguous bytes, rows 16 bytes apart.  For an
// R x C matrix Z (element (r, c)) this library always uses
//     byte(r, c) = ((c / 8) * (R / 8) + r / 8) * 128 + (r % 8) * 16 + (c % 8) * 2,
// i.e. column groups of 8 outermost, then row groups.  The same buffer serves as
//   * a K-major operand with K = columns (the 16-byte rows run along K): leading-byte offset
//     (the K-direction core-matrix stride) = 16 R, stride-byte offset (M/N direction) = 128;
//   * an MN-major operand with K = rows (the 16-byte rows run along M/N): leading-byte offset
//     (K direction: row groups) = 128, stride-byte offset (M/N direction) = 16 R.
// One kind::f16 instruction consumes K = 16: the operand's start address advances by two
// K-direction core matrices per instruction.
#pragma once

#include <stdint.h>

namespace fnetg {
namespace tc {

constexpr int kPollLimit = 1 << 22;  // polls of one mbarrier wait before it gives up

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// byte offset of element (r, c) of an R-row BF16 matrix in the core-matrix layout
__host__ __device__ __forceinline__ uint32_t core_off(int r, int c, int R) {
  return (uint32_t)((((c >> 3) * (R >> 3) + (r >> 3)) << 7) + ((r & 7) << 4) + ((c & 7) << 1));
}

// shared-memory matrix descriptor: start address, leading / stride byte offsets, version 1
// (tcgen05), no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version for tcgen05
  return d;
}

// instruction descriptor of kind::f16: BF16 A and B, FP32 accumulator, M x N, each operand
// K-major (0) or MN-major (1)
__host__ __device__ __forceinline__ uint32_t idesc_bf16(int M, int N, int a_mn, int b_mn) {
  uint32_t d = 0;
  d |= 1u << 4;                      // accumulator format F32
  d |= 1u << 7;                      // A format BF16
  d |= 1u << 10;                     // B format BF16
  d |= (uint32_t)(a_mn & 1) << 15;   // A major-ness
  d |= (uint32_t)(b_mn & 1) << 16;   // B major-ness
  d |= (uint32_t)((N >> 3) & 0x3F) << 17;
  d |= (uint32_t)((M >> 4) & 0x1F) << 24;
  return d;
}

// ---- TMEM allocation (one full warp) --------------------------------------------------------
__device__ __forceinline__ void tmem_alloc(uint32_t *dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                   smem_u32(dst_smem)),
               "r"(ncols));
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols));
}

// ---- MMA (one thread) ---------------------------------------------------------------------
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate));
}
// arrive (once) on the mbarrier when every tcgen05 operation issued so far by this thread is done
__device__ __forceinline__ void mma_commit(uint64_t *mbar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
          smem_u32(mbar)));
}
__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}
// generic-proxy shared-memory writes made visible to the async proxy (the MMA's operand reads)
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

// ---- TMEM -> registers (one warp: its 32 lanes, 16 consecutive columns) ---------------------
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int k = 0; k < 16; k++) v[k] = __uint_as_float(r[k]);
}
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7])
      : "r"(taddr));
#pragma unroll
  for (int k = 0; k < 8; k++) v[k] = __uint_as_float(r[k]);
}
// CH consecutive accumulator columns of this warp's lanes (CH = 8, 16 or 32), one wait
template <int CH> __device__ __forceinline__ void tmem_ld_cols(uint32_t taddr, float (&v)[CH]) {
  static_assert(CH == 8 || CH % 16 == 0, "column count");
  if constexpr (CH == 8) {
    tmem_ld8(taddr, v);
  } else {
#pragma unroll
    for (int c0 = 0; c0 < CH; c0 += 16)
      tmem_ld16(taddr + c0, *reinterpret_cast<float(*)[16]>(&v[c0]));
  }
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
}

// ---- mbarriers --------------------------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t *mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(mbar)), "r"(count));
}
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(mbar)),
               "r"(bytes)
               : "memory");
}
// wait for the phase with the given parity to complete; false if the poll limit ran out
__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, uint32_t parity) {
  const uint32_t a = smem_u32(mbar);
  for (int it = 0; it < kPollLimit; it++) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// ---- bulk copy global -> shared (one thread), completion counted in bytes on the mbarrier ---
// dst, src 16-byte aligned; bytes a multiple of 16
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         uint64_t *mbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(mbar))
      : "memory");
}

}  // namespace tc
}  // namespace fnetg
