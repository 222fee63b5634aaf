// Fifth-generation tensor core (tcgen05) building blocks for sm_103a, in
// inline PTX: shared-memory matrix descriptors, the kind::f16 instruction
// descriptor, TMEM allocation, MMA issue/commit, TMEM loads, mbarriers with
// bounded waits.
//
// Operand layouts (no swizzle).  A "core matrix" is 8 rows of 16 bytes
// (8 x 8 BF16), stored as 128 contiguous bytes.
//   K-major (rows = M or N, K contiguous):
//     element (r, k) at  (r % 8) * 16 + (k % 8) * 2 + (r / 8) * SBO + (k / 8) * LBO
//   MN-major (rows = K, M or N contiguous):
//     element (m, k) at  (m % 8) * 2 + (k % 8) * 16 + (m / 8) * MNO + (k / 8) * KO
//     where the descriptor's (LBO, SBO) carry (MNO, KO) in the order that
//     tc_selftest establishes on the device (kMnMajorSwap below).
// Accumulators live in TMEM: row i of an M = 128 tile is lane i, column j
// of an FP32 accumulator is TMEM column base + j.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace phafd {
namespace tc {

PHAFD_D uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor, no swizzle (layout type 0), version 1
PHAFD_HD uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor of tcgen05.mma kind::f16: BF16 x BF16 -> FP32,
// M x N tile; a_mn / b_mn select MN-major operands
PHAFD_HD uint32_t idesc_bf16(int M, int N, int a_mn, int b_mn) {
  return (1u << 4)                      // D format FP32
         | (1u << 7) | (1u << 10)       // A, B BF16
         | ((uint32_t)a_mn << 15) | ((uint32_t)b_mn << 16) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

PHAFD_D void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
PHAFD_D void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }
PHAFD_D bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait: false when `limit` polls passed without the phase completing
PHAFD_D bool mbar_wait(uint64_t* bar, uint32_t parity, int limit = 1 << 22) {
  for (int i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// TMEM allocation: one full warp executes these
PHAFD_D void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(dst)), "r"(ncols)
               : "memory");
}
PHAFD_D void tmem_relinquish() { asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory"); }
PHAFD_D void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols) : "memory");
}

PHAFD_D void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
PHAFD_D void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
// make generic-proxy shared-memory writes visible to the tensor core
PHAFD_D void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// D (TMEM) (+)= A (smem desc) * B (smem desc); one thread issues
PHAFD_D void mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, int accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// arrive on `bar` once every MMA issued so far by this thread has completed
PHAFD_D void commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(smem_u32(bar))
               : "memory");
}

// 32 lanes x 16 consecutive FP32 columns: thread i of the warp gets lane
// (32 * (warp % 4) + i), columns [col, col + 16)
PHAFD_D void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

}  // namespace tc
}  // namespace phafd
