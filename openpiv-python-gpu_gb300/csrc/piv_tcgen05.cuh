// tcgen05 (5th-generation tensor core) primitives for sm_103a, inline PTX.
//
// * TMEM allocation / release (one warp), tcgen05.ld of fp32 accumulators;
// * kind::f16 MMA with operands in shared memory, issued by one thread;
// * commit to an mbarrier and a bounded wait on it (the wait gives up after a
//   fixed number of polls and reports failure instead of spinning forever);
// * shared-memory matrix descriptors for the no-swizzle ("interleaved")
//   canonical layout: core matrices of 8 rows x 16 bytes.
#pragma once

#include <stdint.h>

#include "piv_common.cuh"

namespace piv {
namespace tc {

PIV_D uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// ---- mbarrier ---------------------------------------------------------------
PIV_D void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

PIV_D bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// One arrival (release semantics, CTA scope) on `bar`.
PIV_D void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Polls until the phase with `parity` completes; gives up after max_polls and
// returns false (each try_wait itself suspends for a hardware-defined time).
PIV_D bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t max_polls) {
  for (uint32_t i = 0; i < max_polls; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// ---- proxy / tcgen05 fences ---------------------------------------------------
// Makes generic-proxy shared-memory writes visible to the tensor core (async proxy).
PIV_D void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
PIV_D void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
PIV_D void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// ---- TMEM -------------------------------------------------------------------
// Allocates `ncols` (power of two, 32..512) TMEM columns; the base address is
// written to *dst (shared memory). Called by one full warp.
PIV_D void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

PIV_D void tmem_free(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// Loads 16 consecutive fp32 columns of this thread's TMEM lane. `taddr` must
// carry the warp's lane quarter in bits 16..31 (lane 32 * (warp % 4)).
PIV_D void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

PIV_D void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Register fence for the destinations of tcgen05.ld: after tmem_ld_wait(),
// pass the loaded array through this so that the compiler sees its values
// produced at the fence and cannot move their uses above the wait.
template <int K>
PIV_D void reg_fence(float (&v)[K]) {
  static_assert(K % 8 == 0, "reg_fence takes multiples of 8 registers");
#pragma unroll
  for (int i = 0; i < K; i += 8)
    asm volatile(""
                 : "+f"(v[i]), "+f"(v[i + 1]), "+f"(v[i + 2]), "+f"(v[i + 3]), "+f"(v[i + 4]), "+f"(v[i + 5]),
                   "+f"(v[i + 6]), "+f"(v[i + 7]));
}

// ---- MMA --------------------------------------------------------------------
// Instruction descriptor of kind::f16 with fp16 A/B and fp32 D.
// a_mn / b_mn: 1 when the operand is stored MN-major (transposed), 0 K-major.
PIV_HD uint32_t idesc_f16(int M, int N, int a_mn, int b_mn) {
  return (1u << 4)                      // D format: f32
         | (0u << 7) | (0u << 10)       // A, B format: f16
         | ((uint32_t)a_mn << 15) | ((uint32_t)b_mn << 16)
         | ((uint32_t)(N >> 3) << 17)   // N / 8
         | ((uint32_t)(M >> 4) << 24);  // M / 16
}

// Shared-memory descriptor, no-swizzle layout. lbo / sbo in bytes.
PIV_D uint64_t sdesc(uint32_t smem_addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((smem_addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// D[tmem] (+)= A * B. kWarp false: issued by the one calling thread. kWarp
// true: called by all 32 lanes of a converged warp with the same operands
// (warp-uniform values) and issued by one elected lane; this keeps the
// descriptor arithmetic on the uniform datapath, which pays off where a
// stage issues many MMAs (the hi/lo split form).
template <bool kWarp = false>
PIV_D void mma_f16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc, uint32_t accumulate) {
  if (kWarp)
    asm volatile(
        "{\n"
        ".reg .pred p, e;\n"
        "elect.sync _|e, 0xffffffff;\n"
        "setp.ne.b32 p, %4, 0;\n"
        "@e tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
        "}\n" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
  else
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "setp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
        "}\n" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Arrives on `bar` once every MMA issued so far by the issuing thread (kWarp:
// the lane elect.sync picks in the same converged warp) has completed.
template <bool kWarp = false>
PIV_D void mma_commit(uint64_t* bar) {
  if (kWarp)
    asm volatile(
        "{\n"
        ".reg .pred e;\n"
        "elect.sync _|e, 0xffffffff;\n"
        "@e tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n"
        "}\n" ::"r"(smem_u32(bar))
        : "memory");
  else
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

}  // namespace tc
}  // namespace piv
