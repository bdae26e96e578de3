// Helpers shared by the kernels that drive the 5th-generation tensor cores
// (tcgen05) from inline PTX: the denoiser's convolutions (conv_tc.cuh) and
// the radiance cache's MLP (nrc.cu).
#pragma once

#include <cstdint>

namespace mrt {

constexpr uint32_t kTcSpin = 1u << 20;  // mbarrier wait cap (polls; a poll may suspend ~1 us)

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor: start, leading (K) and stride (M/N) byte
// offsets, descriptor version 1, no swizzle.  The operand layout this
// describes is the canonical K-major one: a core matrix is 8 rows of 16
// bytes stored contiguously (SBO = 128 B between row groups when the rows of
// a K chunk are consecutive), and the next 16-byte K chunk sits LBO bytes
// further.
__device__ __forceinline__ uint64_t tc_sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return uint64_t((saddr >> 4) & 0x3FFFu) | (uint64_t((lbo >> 4) & 0x3FFFu) << 16) |
           (uint64_t((sbo >> 4) & 0x3FFFu) << 32) | (uint64_t(1) << 46);
}

// Bounded wait for phase `parity` of an mbarrier; false when the cap ran out.
__device__ __forceinline__ bool tc_wait(uint32_t mbar, uint32_t parity) {
    uint32_t done = 0;
    for (uint32_t spins = 0; !done && spins < kTcSpin; ++spins)
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
    return done != 0;
}

} // namespace mrt
