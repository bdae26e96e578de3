// Weight and bias gradients of the denoiser's 3x3 convolutions on the
// tcgen05 tensor cores (included inside denoise.cu's anonymous namespace,
// after conv_tc.cuh).
//
//   gw[co][tap][ci] += sum_p dz[p][co] * x[p + off(tap)][ci]
//   gbias[co]       += sum_p dz[p][co]
//
// is a GEMM whose reduction runs over the pixels: D[(tap, ci)][co] +=
// im2col(x)^T (M = (tap, ci) rows x K = 16 pixels) * dz (K x N = cout) per
// MMA.  A tcgen05 MMA costs a fixed ~46 cycles up to N = 64, so the rows are
// the (tap, input channel) pairs of a 32-channel chunk — 9 x 32 = 288 plus a
// block of ones whose rows accumulate the bias gradient, three M = 128 tiles
// — and each 16 pixels take 3 MMAs of N = cout.  Both operands are stored
// with their channels contiguous (MN-major, selected by the instruction
// descriptor's transpose bits): the im2col is staged in shared memory as
// 256-byte blocks of 16 pixels x 8 channels, one block per (tap, 8-channel
// group), gathered from the NHWC input with cp.async (zero-filled outside
// the image; the nearest-upsampled first source of the decoder's layers and
// the skip concatenation resolved in the gather), so no tap needs a shifted
// operand; dz is staged the same way, one block per 8 output channels.
//
// A CTA owns one 32-channel (16 for the first layer) input chunk and a
// contiguous range of 64-pixel row segments; the partial sums stay in
// tensor memory until the range is done and are then added to the FP32
// gradients with atomics (lanes = consecutive input channels, so each
// output channel's adds are coalesced).  Warps 0-3 gather the stages,
// completing on the stage's `full` mbarrier with no-increment arrivals; one
// thread of warp 4 issues the MMAs and releases a stage through its `empty`
// mbarrier with tcgen05.commit.  Every wait is bounded and ends when
// another role has given up (a shared abort word).
#pragma once

struct WgArgs {
    const bf16* dz;  // N x H x W x cout: gradient at the layer's pre-activation
    const bf16* a;   // source A: N x Ha x Wa x ca (nearest-upsampled when ups)
    const bf16* b;   // source B (skip): N x H x W x cb, or null
    float* gw;       // cout x 9 x (ca + cb), accumulated
    float* gbias;    // cout, accumulated
    int n, h, w, ca, cb, cout, ups;
};

// MN-major no-swizzle matrix descriptor: byte strides between core matrices
// along M/N (8-channel blocks) and along K (8-pixel halves).  As for the
// K-major layout, the leading byte offset is the K stride and the stride byte
// offset the M/N stride (checked on the device with an MMA of known integer
// operands whose layout keeps either reading inside the operand buffers).
__device__ __forceinline__ uint64_t tc_sdesc_mn(uint32_t saddr, uint32_t mn_stride, uint32_t k_stride) {
    return tc_sdesc(saddr, k_stride, mn_stride);
}

constexpr int kWgSeg = 64;  // pixels of a row segment (one stage): 4 MMA K steps

template <int COUT, int NC>
struct WgShape {
    static constexpr int kCo8 = COUT / 8, kNc8 = NC / 8;
    static constexpr int kGroups = 9 * kNc8 + 1;           // (tap, 8 channels) blocks + the ones block
    static constexpr int kTiles = (kGroups + 15) / 16;     // M = 128 tiles (16 blocks each)
    static constexpr int kKSteps = kWgSeg / 16;
    // per K step: kTiles x 16 blocks of 256 B (blocks past kGroups are never
    // written: they only feed accumulator rows that are not read), then dz
    static constexpr uint32_t kA = uint32_t(kKSteps * kTiles * 16 * 256);
    static constexpr uint32_t kB = uint32_t(kKSteps * kCo8 * 256);
    static constexpr uint32_t kStage = (kA + kB + 127u) & ~127u;
    static constexpr int kAccCols = kTiles * COUT;
    static constexpr int kCols = kAccCols <= 32 ? 32 : (kAccCols <= 64 ? 64 : (kAccCols <= 128 ? 128 : (kAccCols <= 256 ? 256 : 512)));
    static constexpr int kStages = 3;
    static constexpr size_t kSmem = size_t(kStages) * kStage + size_t(2 * kStages + 1) * 8 + 32;
};

template <int COUT, int NC>
__global__ void __launch_bounds__(160) k_conv_wgrad(WgArgs a, int chunks, int slices, uint32_t* status) {
    using S = WgShape<COUT, NC>;
    constexpr int kStages = S::kStages;
    static_assert(S::kAccCols <= 512, "tensor memory columns");
    extern __shared__ __align__(128) unsigned char tsm[];
    uint64_t* full = reinterpret_cast<uint64_t*>(tsm + kStages * S::kStage);
    uint64_t* empty = full + kStages;
    uint64_t* fin = empty + kStages;
    uint32_t* slot = reinterpret_cast<uint32_t*>(fin + 1);
    volatile uint32_t* abort = slot + 1;
    volatile uint32_t* prod_go = slot + 2;  // [2]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int chunk = blockIdx.x % chunks, slice = blockIdx.x / chunks;
    const int cin = a.ca + a.cb, c0 = chunk * NC;
    const int segs_x = (a.w + kWgSeg - 1) / kWgSeg;
    const int rows = a.n * a.h * segs_x;
    const int r0 = int((long long)rows * slice / slices), r1 = int((long long)rows * (slice + 1) / slices);
    const uint32_t smem0 = smem_u32(tsm);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                     "r"(uint32_t(S::kCols))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    // the ones block of every K step of every stage: written once, never
    // overwritten by the gathers (16 pixels x 8 channels of BF16 1.0)
    for (int i = tid; i < kStages * S::kKSteps * 64; i += blockDim.x) {
        const int e = i & 63, ks = i >> 6;  // ks = stage * kKSteps + K step
        const int s = ks / S::kKSteps, j = ks % S::kKSteps;
        reinterpret_cast<uint32_t*>(tsm + size_t(s) * S::kStage + size_t(j * S::kTiles * 16 + 9 * S::kNc8) * 256)[e] =
            0x3F803F80u;
    }
    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 128;" ::"r"(smem_u32(full + s)) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(empty + s)) : "memory");
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(fin)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *abort = (*reinterpret_cast<volatile uint32_t*>(status) & MRT_STATUS_PIPE_TIMEOUT) != 0u ? 2u : 0u;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the ones blocks, for the tensor cores
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = *slot;
    auto give_up = [&]() {
        if (*abort == 0u) atomicOr(status, MRT_STATUS_PIPE_TIMEOUT);
        *abort = 1u;
    };

    bool mma_any = false;
    if (warp < 4) {
        // producers: one stage per 64-pixel row segment.  A thread keeps one
        // pixel of each group of eight (tid % 8) and one 8-channel group:
        // eight consecutive threads write eight consecutive 16-byte rows of
        // a block (the 32 banks once) and a warp reads whole 64-byte pixel
        // chunks across its channel groups; the source, its channel offset
        // and its resolution are fixed per thread, so an element costs one
        // address computation.
        const int plo = tid & 7;
        const int c8 = (tid >> 3) % S::kNc8, r_off = (tid >> 3) / S::kNc8;
        constexpr int kRStep = 16 / S::kNc8;  // (tap, pixel group) pairs between a thread's elements
        const int c = c0 + 8 * c8;
        const bool from_a = c < a.ca;
        const bf16* base = from_a ? a.a + c : a.b + (c - a.ca);
        const int cstride = from_a ? a.ca : a.cb;
        const int sh = (from_a && a.ups) ? 1 : 0;
        const int hs = a.h >> sh, wsz = a.w >> sh;
        const int d8 = (tid >> 3) % S::kCo8, dph0 = (tid >> 3) / S::kCo8;
        constexpr int kDStep = 16 / S::kCo8 > 0 ? 16 / S::kCo8 : 1;
        // the element maps below cover a segment exactly once only when the
        // steps divide its pixel groups (a thread's first group r_off or
        // dph0 is below its step)
        static_assert(16 % S::kNc8 == 0 && (kWgSeg / 8) % kRStep == 0, "im2col gather covers the segment");
        static_assert(16 % S::kCo8 == 0 && (kWgSeg / 8) % kDStep == 0, "dz gather covers the segment");
        for (int g = 0, r = r0; r < r1; ++r, ++g) {
            const int s = g % kStages;
            const uint32_t u = uint32_t(g / kStages);
            const int xs = r % segs_x, y = (r / segs_x) % a.h, n = r / (segs_x * a.h);
            const int x0 = xs * kWgSeg;
            const uint32_t st = smem0 + uint32_t(s) * S::kStage;
            if (tid == 0) {
                if (!ws_wait(smem_u32(empty + s), (u & 1u) ^ 1u, abort)) give_up();
                prod_go[g & 1] = *abort == 0u ? 1u : 0u;
            }
            asm volatile("bar.sync 1, 128;" ::: "memory");
            if (prod_go[g & 1] == 0u) break;
            // im2col: element (tap t, pixel p, channel group c8) -> block
            // (K step p / 16, t * NC8 + c8), row p % 16.  Taps unrolled: the
            // three source rows are addressed once per stage
            const bf16* srow[3];
            bool rin[3];
#pragma unroll
            for (int ky = 0; ky < 3; ++ky) {
                const int yy = y + ky - 1;
                rin[ky] = unsigned(yy) < unsigned(a.h);
                srow[ky] = base + size_t(n * hs + (rin[ky] ? yy >> sh : 0)) * size_t(wsz) * size_t(cstride);
            }
#pragma unroll
            for (int t = 0; t < 9; ++t) {
#pragma unroll
                for (int ph = 0; ph < kWgSeg / 8; ph += kRStep) {
                    const int p = (ph + r_off) * 8 + plo;  // r_off < kRStep: (tap, group) pairs stay in order
                    const int xx = x0 + p + t % 3 - 1;
                    const bool in = rin[t / 3] && unsigned(xx) < unsigned(a.w);
                    cp16(st + uint32_t(((p >> 4) * S::kTiles * 16 + t * S::kNc8 + c8) * 256 + (p & 15) * 16),
                         in ? srow[t / 3] + size_t(xx >> sh) * size_t(cstride) : a.dz, in);
                }
            }
            // dz: element (pixel p, channel group d8) -> block (K step, d8), row p % 16
            {
                const bf16* drow = a.dz + (size_t(n * a.h + y) * a.w + x0) * COUT + 8 * d8;
                for (int ph = dph0; ph < kWgSeg / 8; ph += kDStep) {
                    const int p = ph * 8 + plo;
                    const bool in = x0 + p < a.w;
                    cp16(st + S::kA + uint32_t(((p >> 4) * S::kCo8 + d8) * 256 + (p & 15) * 16),
                         in ? drow + size_t(p) * COUT : a.dz, in);
                }
            }
            asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(full + s)) : "memory");
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
    } else if (lane == 0 && *abort == 0u) {
        // MMA issuer: per K step, tile m of (tap, channel) rows into columns
        // [m * COUT, (m + 1) * COUT)
        constexpr uint32_t idesc = tc_idesc(128, COUT) | (1u << 15) | (1u << 16);  // A and B MN-major
        bool ok = true;
        // stage-0 descriptors; the others add (byte offset / 16) to the
        // 14-bit start field (shared addresses stay below 2^18: no carry)
        const uint64_t a00 = tc_sdesc_mn(smem0, 256u, 128u);
        const uint64_t b00 = tc_sdesc_mn(smem0 + S::kA, 256u, 128u);
        for (int g = 0, r = r0; r < r1; ++r, ++g) {
            const int s = g % kStages;
            const uint32_t u = uint32_t(g / kStages);
            if (!ws_wait(smem_u32(full + s), u & 1u, abort)) { ok = false; break; }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint64_t sd = uint64_t((uint32_t(s) * S::kStage) >> 4);
#pragma unroll
            for (int j = 0; j < S::kKSteps; ++j) {
                const uint32_t acc = (g > 0 || j > 0) ? 1u : 0u;
                const uint64_t bd = b00 + sd + uint64_t((j * S::kCo8 * 256) >> 4);
#pragma unroll
                for (int m = 0; m < S::kTiles; ++m) {
                    const uint64_t ad = a00 + sd + uint64_t(((j * S::kTiles + m) * 16 * 256) >> 4);
                    asm volatile(
                        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(taddr + uint32_t(m * COUT)),
                        "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                        : "memory");
                }
            }
            mma_any = true;
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(empty + s))
                         : "memory");
        }
        if (!ok) give_up();
        if (mma_any)
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(fin))
                         : "memory");
        else if (r0 < r1)
            give_up();
    }
    // epilogue (warps 0-3): tile m, TMEM lane 32 warp + lane = block
    // 16 m + (32 warp + lane) / 8, channel (32 warp + lane) % 8 of it
    if (warp < 4 && r0 < r1) {
        const bool ok = ws_wait(smem_u32(fin), 0u, abort);
        if (__all_sync(0xFFFFFFFFu, ok)) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            for (int m = 0; m < S::kTiles; ++m) {
                if (16 * m + 4 * warp >= S::kGroups) break;  // the warp's 4 blocks all lie past the ones block
                const int blk = 16 * m + (32 * warp + lane) / 8, cc = (32 * warp + lane) % 8;
                const bool wrow = blk < 9 * S::kNc8;
                const bool brow = blk == 9 * S::kNc8 && cc == 0 && chunk == 0;
                const int t = blk / S::kNc8, ci = c0 + (blk % S::kNc8) * 8 + cc;
#pragma unroll
                for (int c = 0; c < COUT; c += 16) {
                    uint32_t v[16];
                    asm volatile(
                        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                        "[%16];\n"
                        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                          "=r"(v[15])
                        : "r"(taddr + (uint32_t(32 * warp) << 16) + uint32_t(m * COUT + c)));
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                    if (wrow) {
#pragma unroll
                        for (int q = 0; q < 16; ++q)
                            atomicAdd(a.gw + (size_t(c + q) * 9 + t) * cin + ci, __uint_as_float(v[q]));
                    } else if (brow) {
#pragma unroll
                        for (int q = 0; q < 16; ++q) atomicAdd(a.gbias + c + q, __uint_as_float(v[q]));
                    }
                }
            }
        } else if (lane == 0) {
            give_up();
        }
    }
    __syncthreads();
    // every MMA issued has completed before the tensor memory and the shared
    // memory are released; copies issued but never consumed have landed
    // (cp.async.wait_all above)
    if (warp == 4 && lane == 0 && mma_any && !tc_wait(smem_u32(fin), 0u)) atomicOr(status, MRT_STATUS_PIPE_TIMEOUT);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(uint32_t(S::kCols))
                     : "memory");
}

// Grid: `chunks` input-channel chunks x `slices` row ranges, about one CTA
// per SM, at least 4 row segments per CTA so the atomics stay a small share
// of the work.
template <int COUT, int NC>
cudaError_t launch_conv_wgrad(const WgArgs& wa, uint32_t* status, int sm_count, cudaStream_t s) {
    using S = WgShape<COUT, NC>;
    static uint64_t configured = 0;
    cudaError_t e = tc_configure(k_conv_wgrad<COUT, NC>, S::kSmem, configured);
    if (e != cudaSuccess) return e;
    const int cin = wa.ca + wa.cb;
    if (cin % NC || wa.cout != COUT) return cudaErrorInvalidValue;
    const int chunks = cin / NC;
    const int rows = wa.n * wa.h * ((wa.w + kWgSeg - 1) / kWgSeg);
    const int slices = std::max(1, std::min((rows + 3) / 4, std::max(1, sm_count / chunks)));
    k_conv_wgrad<COUT, NC><<<chunks * slices, 160, S::kSmem, s>>>(wa, chunks, slices, status);
    return cudaGetLastError();
}
