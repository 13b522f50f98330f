// qbg_tcgen05.cuh -- inline-PTX helpers shared by the tensor-core GEMMs
// (qbg_tc.cu, qbg_ozaki.cu): mbarriers with bounded waits, 1-D bulk async
// copies into shared memory, tcgen05 shared-memory descriptors for the
// canonical no-swizzle K-major layout, kind::f16 MMAs into tensor memory,
// commits and tensor-memory loads.  sm_100a/sm_103a only.
#pragma once
#include <cstdint>

namespace qbg {

constexpr int TC_SPIN = 1 << 21;  // polls per bounded wait (~0.2 s with backoff, ~2 s at most
                                   // with try_wait)

// ------------------------------------------------------------ PTX helpers
static __device__ __forceinline__ uint32_t su32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
static __device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(count));
}
static __device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(b)), "r"(bytes)
               : "memory");
}
static __device__ __forceinline__ void mbar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(b)) : "memory");
}
// One poll of an mbarrier phase.  By default mbarrier.try_wait with a 1 us
// suspend-time hint: the hardware wakes the thread when the phase completes,
// which hands the pipeline stages over sooner than test_wait with a 64 ns
// sleep (GEMM1 3.84 -> 3.71 ms, the FP64-accurate GEMMs 4.7% faster on the
// 216-atom cell); QBG_MBAR_TRYWAIT=0 selects test_wait, which backs off by
// 64 ns per poll after QBG_SPIN_SLEEP_AFTER polls.
#ifndef QBG_MBAR_TRYWAIT
#define QBG_MBAR_TRYWAIT 1
#endif
#ifndef QBG_SPIN_SLEEP_AFTER
#define QBG_SPIN_SLEEP_AFTER 64
#endif
static __device__ __forceinline__ bool mbar_poll(uint64_t* b, uint32_t par) {
  uint32_t ok;
#if QBG_MBAR_TRYWAIT
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
      "selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(su32(b)), "r"(par), "r"(1000u)
      : "memory");
#else
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(su32(b)), "r"(par)
      : "memory");
#endif
  return ok != 0;
}
static __device__ __forceinline__ void mbar_backoff(int it) {
  if (!QBG_MBAR_TRYWAIT && it > QBG_SPIN_SLEEP_AFTER) __nanosleep(64);
}
// bounded wait for the phase with parity `par` to complete; false on timeout
// or when another CTA has already raised the grid-wide error word
static __device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t par, const int* gstatus,
                                          int limit = TC_SPIN) {
  for (int it = 0; it < limit; ++it) {
    if (mbar_poll(b, par)) return true;
    mbar_backoff(it);
    if ((it & 4095) == 4095 && *(volatile const int*)gstatus) return false;
  }
  return false;
}
// bounded wait for this CTA's own copies or MMAs to land before its shared
// or tensor memory is released: it does not give up early when another CTA
// has failed (its own operations are still in flight then)
static __device__ __forceinline__ bool mbar_wait_drain(uint64_t* b, uint32_t par) {
  for (int it = 0; it < TC_SPIN; ++it) {
    if (mbar_poll(b, par)) return true;
    mbar_backoff(it);
  }
  return false;
}
static __device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          su32(dst)),
      "l"(src), "r"(bytes), "r"(su32(bar))
      : "memory");
}
static __device__ __forceinline__ uint64_t sdesc(uint32_t addr) {
  // no-swizzle K-major canonical layout: LBO (K direction) 128 B, SBO (8-row
  // groups) 256 B, descriptor version 1
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)(128 >> 4) << 16) |
         ((uint64_t)(256 >> 4) << 32) | ((uint64_t)1 << 46);
}
static __device__ __forceinline__ uint32_t idesc_f16_f32(int m, int n) {
  // D F32 (bit 4), A/B F16 (format 0), K-major, N>>3 at bit 17, M>>4 at 24
  return (1u << 4) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}
static __device__ __forceinline__ void mma_f16(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc,
                                        uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(da), "l"(db), "r"(idesc), "r"(acc));
}
static __device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
      su32(bar))
               : "memory");
}
static __device__ __forceinline__ void tmem_ld32(uint32_t ta, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(ta));
}
static __device__ __forceinline__ void tmem_ld16(uint32_t ta, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(ta));
}
static __device__ __forceinline__ void tmem_st16(uint32_t ta, const uint32_t* r) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15,%16};" ::"r"(ta),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
      "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]),
      "r"(r[15]));
}
static __device__ __forceinline__ void tmem_st32(uint32_t ta, const uint32_t* r) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(ta),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
      "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]),
      "r"(r[15]), "r"(r[16]), "r"(r[17]), "r"(r[18]), "r"(r[19]), "r"(r[20]), "r"(r[21]),
      "r"(r[22]), "r"(r[23]), "r"(r[24]), "r"(r[25]), "r"(r[26]), "r"(r[27]), "r"(r[28]),
      "r"(r[29]), "r"(r[30]), "r"(r[31]));
}


}  // namespace qbg
