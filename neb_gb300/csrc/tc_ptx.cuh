// Blackwell (sm_103a) building blocks written as inline PTX: mbarriers, TMA
// tile loads, tcgen05 tensor-memory allocation, MMA issue / commit and
// tensor-memory loads.  Every wait is bounded: after kMaxSpins failed polls
// the waiter records an error bit in a global status word and carries on, so
// a kernel always terminates.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cstdint>

namespace neb {
namespace tc {

constexpr uint32_t kMaxSpins = 1u << 21;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// ------------------------------------------------------------- mbarrier
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: returns false (and sets bit 0 of *status) after `limit`
// polls, or soon after another wait of this launch has already given up.
// A caller that gets false issues no further copies or MMAs.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* status,
                                          uint32_t limit = kMaxSpins) {
  uint32_t spins = 0;
  while (!mbar_try_wait(bar, parity)) {
    if ((++spins & 1023u) == 0u &&
        (spins >= limit || *reinterpret_cast<volatile int*>(status) != 0)) {
      atomicOr(status, 1);
      return false;
    }
  }
  return true;
}
// The same wait for the shutdown of a CTA that gave up: it is not cut short
// by the status word (copies or MMAs this CTA issued must land before it
// exits), still bounded by kMaxSpins; a wait that runs out sets bit 1.
__device__ __forceinline__ void mbar_wait_drain(uint64_t* bar, uint32_t parity, int* status) {
  uint32_t spins = 0;
  while (!mbar_try_wait(bar, parity)) {
    if (++spins >= kMaxSpins) {
      atomicOr(status, 2);
      return;
    }
  }
}
// Waits until the last copy issued into each of the `stages` stages of a
// ring (issue count `issued`, stage = issue % stages, phase = issue /
// stages) has completed on its `full` barrier.
__device__ __forceinline__ void drain_ring(uint64_t* full, int stages, int issued, int* status) {
  for (int j = issued > stages ? issued - stages : 0; j < issued; ++j)
    mbar_wait_drain(&full[j % stages], (uint32_t)((j / stages) & 1), status);
}

// ------------------------------------------------------------------ TMA
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar,
                                            int32_t x, int32_t y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4}], [%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y)
      : "memory");
}

// -------------------------------------------------------------- tcgen05
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(dst)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T, bf16 x bf16 -> f32, both K-major.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// Arrive on *bar once every MMA issued so far by this thread has completed.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

// 16 consecutive 32-bit columns of this thread's TMEM lane, without the
// wait: several loads can be in flight before one
// tmem_ld_wait; tmem_ld_fence then orders the registers after the wait.
__device__ __forceinline__ void tmem_ld16_issue(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld8_issue(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld4_issue(uint32_t taddr, uint32_t* r) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(taddr));
}
template <int W>
__device__ __forceinline__ void tmem_ld_issue(uint32_t taddr, uint32_t* r) {
  static_assert(W == 4 || W == 8 || W == 16, "TMEM load width");
  if constexpr (W == 16) tmem_ld16_issue(taddr, r);
  else if constexpr (W == 8) tmem_ld8_issue(taddr, r);
  else tmem_ld4_issue(taddr, r);
}
__device__ __forceinline__ void tmem_ld_wait() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_ld_fence(uint32_t* r) {
#pragma unroll
  for (int i = 0; i < 16; ++i) asm volatile("" : "+r"(r[i]));
}

// Shared-memory matrix descriptor of a K-major bf16 tile stored as rows of
// 128 bytes (64 elements) with the 128-byte swizzle (the layout a TMA load
// with CU_TENSOR_MAP_SWIZZLE_128B writes): 8-row core groups 1024 bytes
// apart (stride byte offset), descriptor version 1, layout code 2.
__device__ __forceinline__ uint64_t desc_sw128(uint32_t smem_addr) {
  uint64_t d = 0;
  d |= (uint64_t)((smem_addr >> 4) & 0x3FFF);
  d |= (uint64_t)(1) << 16;                  // leading byte offset (unused when swizzled)
  d |= (uint64_t)((1024 >> 4) & 0x3FFF) << 32;  // stride byte offset
  d |= (uint64_t)1 << 46;                    // descriptor version (tcgen05)
  d |= (uint64_t)2 << 61;                    // SWIZZLE_128B
  return d;
}

// Shared-memory matrix descriptor of an MN-major bf16 tile with the 128-byte
// swizzle: each K row holds 64 MN-contiguous elements (128 bytes, the layout
// a TMA box {64 MN elements, K rows} with CU_TENSOR_MAP_SWIZZLE_128B writes),
// 8-row K groups 1024 bytes apart (stride byte offset) and 64-element MN
// blocks mn_stride bytes apart (leading byte offset).
__device__ __forceinline__ uint64_t desc_mn_sw128(uint32_t smem_addr, uint32_t mn_stride) {
  uint64_t d = 0;
  d |= (uint64_t)((smem_addr >> 4) & 0x3FFF);
  d |= (uint64_t)((mn_stride >> 4) & 0x3FFF) << 16;  // leading byte offset: MN blocks
  d |= (uint64_t)((1024 >> 4) & 0x3FFF) << 32;        // stride byte offset: K groups
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// Instruction descriptor: kind::f16 with bf16 A and B, f32 D, K-major B; A
// K-major, or MN-major when a_mn (bit 15, transpose A).
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N, bool a_mn = false) {
  return (1u << 4)                         // D = f32
         | (1u << 7)                       // A = bf16
         | (1u << 10)                      // B = bf16
         | ((a_mn ? 1u : 0u) << 15)        // A major-ness
         | ((uint32_t)(N >> 3) << 17)      // N / 8
         | ((uint32_t)(M >> 4) << 24);     // M / 16
}

// Split x into bf16 hi + lo with x ~= hi + lo (16 significant bits).
__device__ __forceinline__ void split_bf16(float x, __nv_bfloat16& hi, __nv_bfloat16& lo) {
  hi = __float2bfloat16_rn(x);
  lo = __float2bfloat16_rn(x - __bfloat162float(hi));
}

}  // namespace tc
}  // namespace neb
