// Read-bandwidth sweep for roofline denominators.  The traversal kernels
// read a scene that stays resident in L2, so the roof that binds them is
// L2 read bandwidth, which no generated peak gives: this sweep reads
// a caller's buffer `passes` times with 16-byte loads that bypass L1
// (ld.global.cg).  On a buffer well inside L2 every pass after the first
// is served by L2.
#include "internal.hpp"

namespace {

__global__ void __launch_bounds__(256) k_read_sweep(const uint4* __restrict__ buf, size_t n16, uint32_t passes,
                                                    uint32_t* sink) {
    const size_t stride = size_t(gridDim.x) * blockDim.x;
    uint32_t acc = 0u;
    for (uint32_t p = 0; p < passes; ++p) {
        for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n16; i += stride) {
            const uint4 v = __ldcg(buf + i);
            acc ^= v.x ^ v.y ^ v.z ^ v.w;
        }
    }
    // one word per block keeps the loads live
    acc = __reduce_xor_sync(0xFFFFFFFFu, acc);
    if ((threadIdx.x & 31u) == 0u) atomicXor(sink + blockIdx.x, acc);
}

} // namespace

extern "C" int mrt_cuda_read_sweep(mrt_ctx* ctx, const void* buf, size_t bytes, uint32_t passes, uint32_t* sink,
                                   uint32_t sink_words, void* stream) {
    if (!ctx || !buf || !sink || bytes < 16 || passes == 0 || sink_words == 0) return MRT_EINVAL;
    if (reinterpret_cast<uintptr_t>(buf) % 16u != 0u) return MRT_EINVAL;
    cudaSetDevice(ctx->device);
    const uint32_t blocks = std::min<uint32_t>(sink_words, uint32_t(ctx->sm_count) * 8u);
    k_read_sweep<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(static_cast<const uint4*>(buf), bytes / 16,
                                                                         passes, sink);
    if (cudaGetLastError() != cudaSuccess) return MRT_ECUDA;
    return MRT_OK;
}
