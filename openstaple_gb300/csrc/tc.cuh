// tc.cuh -- fifth-generation tensor core (tcgen05) primitives for sm_103a:
// tensor-memory allocation, shared-memory operand descriptors, BF16 MMA with
// FP32 accumulation in TMEM, completion through an mbarrier, and TMEM loads.
//
// Operand layout used throughout: "K-major, no swizzle".  A matrix of R rows
// and K columns (BF16) is stored as 8x8 core matrices of 128 contiguous bytes
// (8 rows of 16 bytes); element (r, k) lives at
//     (r / 8) * SBO + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2
// with SBO = (K / 8) * 128.  The descriptor's leading byte offset (between
// core matrices along K) is 128 and its stride byte offset (between 8-row
// groups) is SBO.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>
#include "common.cuh"

namespace ost {
namespace tc {

OST_D uint32_t smem_u32(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

OST_D uint32_t kmajor_offset(int r, int k, int K) { return (r >> 3) * (K * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2; }

// tcgen05 shared-memory matrix descriptor (no swizzle)
OST_D uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= uint64_t((saddr & 0x3FFFF) >> 4);
  d |= uint64_t((lbo & 0x3FFFF) >> 4) << 16;
  d |= uint64_t((sbo & 0x3FFFF) >> 4) << 32;
  d |= uint64_t(1) << 46;          // fixed 0b001 field of the tcgen05 descriptor
  return d;                        // base offset 0, relative LBO mode, no swizzle
}

// instruction descriptor of kind::f16: BF16 x BF16 -> FP32, both K-major
OST_HD constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4)                      // D: FP32
         | (1u << 7)                    // A: BF16
         | (1u << 10)                   // B: BF16
         | (uint32_t(N >> 3) << 17)     // N / 8
         | (uint32_t(M >> 4) << 24);    // M / 16
}

// one warp allocates ncols TMEM columns; the base address is written to *slot
OST_D void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(slot)),
               "r"(ncols));
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
}
OST_D void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols));
}

OST_D void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
OST_D void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
OST_D void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

// D[tmem] (+)= A[smem] * B[smem]^T, one elected thread
OST_D void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, int accumulate) {
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "setp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
      "}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

// arrive on the mbarrier once all previously issued MMAs of this thread complete
OST_D void mma_commit(uint64_t* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                   smem_u32(mbar))
               : "memory");
}

OST_D void mbar_init(uint64_t* mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
}

// Waits for phase `parity` of the mbarrier with an iteration limit; returns
// false (without hanging) if the limit is reached.
OST_D bool mbar_wait_bounded(uint64_t* mbar, uint32_t parity, long max_iter) {
  for (long it = 0; it < max_iter; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(ok)
        : "r"(smem_u32(mbar)), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// 32 lanes x 16 consecutive 32-bit columns: thread i of the warp receives
// lane (lane_base + i), columns col .. col+15
OST_D void tmem_ld16(uint32_t taddr, float v[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc
}  // namespace ost
