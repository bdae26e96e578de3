// Weight and bias gradients of the denoiser's 3x3 convolutions on the
// tcgen05 tensor cores (included inside denoise.cu's anonymous namespace,
// after conv_tc.cuh).
//
//   gw[co][tap][ci] += sum_p dz[p][co] * x[p + off(tap)][ci]
//   gbias[co]       += sum_p dz[p][co]
//
// is a GEMM whose reduction runs over the pixels: per tap, D (M = output
// channel, N = input channel) += dz^T (M x K) * x_tap (K x N) with K = 16
// consecutive pixels of an image row per MMA.  Both operands are stored with
// their channels contiguous (NHWC), i.e. MN-major, which the instruction
// descriptor's transpose bits select, so neither is transposed in memory.  In
// shared memory an operand is a set of 256-byte blocks of 16 pixels x 8
// channels (a pixel's 8 channels are one 16-byte row; the two 8-pixel core
// matrices of an MMA's K sit 128 bytes apart).  The input is staged as a halo
// (image rows y-1..y+1, pixels x0-1..x0+128) whose 8-channel planes hold the
// pixels consecutively, so a tap's operand is the plane shifted by its column
// (16 bytes a pixel) and row: the im2col never exists.  M is 128 lanes; the
// rows at and above cout read whatever follows in the stage (the stage is
// padded so that stays inside it) and their accumulators are never read.
// The bias gradient is one more MMA per K step against a block of ones.
//
// A CTA accumulates one 16- or 32-channel input chunk (NC) of all 9 taps
// (9 x NC tensor-memory columns) plus the bias (16 columns) over a contiguous
// range of image row segments (up to 128 pixels each), so the partial sums of
// a CTA never leave tensor memory until its range is done; the epilogue then
// adds them to the FP32 gradients with atomics (one per weight per CTA).
// Warps 0-3 gather the stages with cp.async (zero-filled outside the image;
// the nearest-upsampled first source of the decoder's layers and the skip
// concatenation are resolved in the gather), completing on the stage's
// `full` mbarrier with no-increment arrivals; one thread of warp 4 issues the
// MMAs and releases a stage through its `empty` mbarrier with
// tcgen05.commit.  Every wait is bounded and ends when another role has
// given up (a shared abort word), as in the forward kernels.
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

constexpr int kWgPix = 128;               // pixels of an image row segment (one stage)
constexpr int kWgHalo = kWgPix + 2;       // halo pixels per row
constexpr uint32_t kWgPlane = kWgHalo * 16;  // one 8-channel plane of a halo row

template <int COUT, int NC>
struct WgShape {
    static constexpr int kCo8 = COUT / 8, kNc8 = NC / 8;
    // dz: [segment (8)][8-channel block][16 pixels][8 channels], padded so the
    // M = 128 operand of the last segment stays inside the stage
    static constexpr uint32_t kA = uint32_t(kWgPix * COUT * 2) + (kCo8 < 16 ? uint32_t(16 - kCo8) * 256u : 0u);
    static constexpr uint32_t kRow = uint32_t(kNc8) * kWgPlane;  // one halo row: [block][pixel][8 channels]
    static constexpr uint32_t kB = 3u * kRow;
    static constexpr uint32_t kStage = (kA + kB + 127u) & ~127u;
    static constexpr int kTapCols = 9 * NC;
    static constexpr int kCols = kTapCols + 16 <= 256 ? 256 : 512;  // taps + bias, a power of 2
    static constexpr int kStages = 3;
    static constexpr size_t kUsed = size_t(kStages) * kStage + 512 + size_t(2 * kStages + 1) * 8 + 32;
    // a CTA holding all 512 tensor-memory columns asks for enough shared
    // memory that no second one is placed on its SM (it would only wait in
    // tcgen05.alloc)
    static constexpr size_t kSmem = kCols == 512 && kUsed < 120u * 1024u ? 120u * 1024u : kUsed;
};

template <int COUT, int NC>
__global__ void __launch_bounds__(160) k_conv_wgrad(WgArgs a, int chunks, int slices, uint32_t* status) {
    using S = WgShape<COUT, NC>;
    constexpr int kStages = S::kStages;
    extern __shared__ __align__(128) unsigned char tsm[];
    unsigned char* ones = tsm + kStages * S::kStage;  // 16 pixels x 16 channels of BF16 1.0
    uint64_t* full = reinterpret_cast<uint64_t*>(ones + 512);
    uint64_t* empty = full + kStages;
    uint64_t* fin = empty + kStages;
    uint32_t* slot = reinterpret_cast<uint32_t*>(fin + 1);
    volatile uint32_t* abort = slot + 1;
    volatile uint32_t* prod_go = slot + 2;  // [2]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int chunk = blockIdx.x % chunks, slice = blockIdx.x / chunks;
    const int cin = a.ca + a.cb, c0 = chunk * NC;
    const int tiles_x = (a.w + kWgPix - 1) / kWgPix;
    const int rows = a.n * a.h * tiles_x;
    const int r0 = int((long long)rows * slice / slices), r1 = int((long long)rows * (slice + 1) / slices);
    const uint32_t smem0 = smem_u32(tsm), ones_s = smem_u32(ones);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                     "r"(uint32_t(S::kCols))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid < 128) reinterpret_cast<uint16_t*>(ones)[2 * tid] = reinterpret_cast<uint16_t*>(ones)[2 * tid + 1] =
        uint16_t(0x3F80u);  // BF16 1.0
    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 128;" ::"r"(smem_u32(full + s)) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(empty + s)) : "memory");
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(fin)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *abort = (*reinterpret_cast<volatile uint32_t*>(status) & MRT_STATUS_PIPE_TIMEOUT) != 0u ? 2u : 0u;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the ones block, for the tensor cores
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = *slot;
    auto give_up = [&]() {
        if (*abort == 0u) atomicOr(status, MRT_STATUS_PIPE_TIMEOUT);
        *abort = 1u;
    };
    auto segments = [&](int x0) { return (min(kWgPix, a.w - x0) + 15) >> 4; };

    bool mma_any = false;
    if (warp < 4) {
        // producers: one stage per image row segment
        const int ha = a.ups ? a.h >> 1 : a.h, wa = a.ups ? a.w >> 1 : a.w;
        for (int g = 0, r = r0; r < r1; ++r, ++g) {
            const int s = g % kStages;
            const uint32_t u = uint32_t(g / kStages);
            const int xt = r % tiles_x, y = (r / tiles_x) % a.h, n = r / (tiles_x * a.h);
            const int x0 = xt * kWgPix, segs = segments(x0);
            const uint32_t st = smem0 + uint32_t(s) * S::kStage;
            if (tid == 0) {
                if (!ws_wait(smem_u32(empty + s), (u & 1u) ^ 1u, abort)) give_up();
                prod_go[g & 1] = *abort == 0u ? 1u : 0u;
            }
            asm volatile("bar.sync 1, 128;" ::: "memory");
            if (prod_go[g & 1] == 0u) break;
            // dz: pixels x0 .. x0 + 16 segs - 1 of row y, all COUT channels
            for (int i = tid; i < 16 * segs * S::kCo8; i += 128) {
                const int c8 = i % S::kCo8, px = i / S::kCo8, xx = x0 + px;
                const bool in = xx < a.w;
                const bf16* src = in ? a.dz + ((size_t(n) * a.h + y) * a.w + xx) * COUT + 8 * c8 : a.dz;
                cp16(st + uint32_t(((px >> 4) * S::kCo8 + c8) * 256 + (px & 15) * 16), src, in);
            }
            // input halo: rows y-1 .. y+1, pixels x0-1 .. x0 + 16 segs, channels c0 .. c0 + NC - 1
            const int hx = 16 * segs + 2;
            for (int i = tid; i < 3 * hx * S::kNc8; i += 128) {
                const int c8 = i % S::kNc8, q = i / S::kNc8, px = q % hx, rr = q / hx;
                const int yy = y - 1 + rr, xx = x0 - 1 + px, c = c0 + 8 * c8;
                const bool in = yy >= 0 && yy < a.h && xx >= 0 && xx < a.w;
                const bf16* src = a.dz;  // any valid address when zero-filling
                if (in) {
                    if (c < a.ca) {
                        const int ya = a.ups ? yy >> 1 : yy, xa = a.ups ? xx >> 1 : xx;
                        src = a.a + ((size_t(n) * ha + ya) * wa + xa) * a.ca + c;
                    } else {
                        src = a.b + ((size_t(n) * a.h + yy) * a.w + xx) * a.cb + (c - a.ca);
                    }
                }
                cp16(st + S::kA + uint32_t(rr) * S::kRow + uint32_t(c8) * kWgPlane + uint32_t(px * 16), src, in);
            }
            asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(full + s)) : "memory");
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
    } else if (lane == 0 && *abort == 0u) {
        // MMA issuer: per segment, 9 taps into columns [tap * NC, ...) and
        // the bias into columns [9 NC, 9 NC + 16) (chunk 0 only)
        constexpr uint32_t idesc = tc_idesc(128, NC) | (1u << 15) | (1u << 16);    // A and B MN-major
        constexpr uint32_t idesc_b = tc_idesc(128, 16) | (1u << 15) | (1u << 16);
        bool ok = true;
        // descriptors of stage 0, segment 0, tap 0: the others differ only in
        // the start address, so they are these plus the byte offset / 16
        // (smem addresses stay below 2^18: no carry out of the 14-bit field)
        const uint64_t a00 = tc_sdesc_mn(smem0, 256u, 128u);
        const uint64_t b00 = tc_sdesc_mn(smem0 + S::kA, kWgPlane, 128u);
        const uint64_t od = tc_sdesc_mn(ones_s, 256u, 128u);
        for (int g = 0, r = r0; r < r1; ++r, ++g) {
            const int s = g % kStages;
            const uint32_t u = uint32_t(g / kStages);
            if (!ws_wait(smem_u32(full + s), u & 1u, abort)) { ok = false; break; }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int segs = segments((r % tiles_x) * kWgPix);
            const uint64_t sd = uint64_t((uint32_t(s) * S::kStage) >> 4);
            const uint64_t a0 = a00 + sd, b0 = b00 + sd;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                if (j >= segs) break;
                const uint64_t ad = a0 + uint64_t((j * S::kCo8 * 256) >> 4);
                const uint32_t acc = (g > 0 || j > 0) ? 1u : 0u;
#pragma unroll
                for (int t = 0; t < 9; ++t) {
                    const uint64_t bd = b0 + uint64_t(((t / 3) * S::kRow + uint32_t(16 * j + t % 3) * 16u) >> 4);
                    asm volatile(
                        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(taddr + uint32_t(t * NC)),
                        "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                        : "memory");
                }
                if (chunk == 0)
                    asm volatile(
                        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
                            taddr + uint32_t(S::kTapCols)),
                        "l"(ad), "l"(od), "r"(idesc_b), "r"(acc)
                        : "memory");
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
    // epilogue (warps 0-3, TMEM lanes 32 warp ..): lane = output channel
    if (warp < 4 && r0 < r1 && 32 * warp < a.cout) {
        const bool ok = ws_wait(smem_u32(fin), 0u, abort);
        if (__all_sync(0xFFFFFFFFu, ok)) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int co = 32 * warp + lane;
            const int ncol = chunk == 0 ? S::kTapCols + 16 : S::kTapCols;
            for (int c = 0; c < ncol; c += 16) {
                uint32_t v[16];
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                    "[%16];\n"
                    : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                      "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                      "=r"(v[15])
                    : "r"(taddr + (uint32_t(32 * warp) << 16) + uint32_t(c)));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if (co < a.cout) {
                    if (c < S::kTapCols) {
                        const int t = c / NC, ci = c0 + c % NC;
                        float* dst = a.gw + (size_t(co) * 9 + t) * cin + ci;
#pragma unroll
                        for (int q = 0; q < 16; ++q) atomicAdd(dst + q, __uint_as_float(v[q]));
                    } else {
                        atomicAdd(a.gbias + co, __uint_as_float(v[0]));
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
// per SM (a CTA holds up to 512 tensor-memory columns), at least 4 row
// segments per CTA so the atomics stay a small share of the work.
template <int COUT, int NC>
cudaError_t launch_conv_wgrad(const WgArgs& wa, uint32_t* status, int sm_count, cudaStream_t s) {
    using S = WgShape<COUT, NC>;
    static uint64_t configured = 0;
    cudaError_t e = tc_configure(k_conv_wgrad<COUT, NC>, S::kSmem, configured);
    if (e != cudaSuccess) return e;
    const int cin = wa.ca + wa.cb;
    if (cin % NC || wa.cout != COUT) return cudaErrorInvalidValue;
    const int chunks = cin / NC;
    const int rows = wa.n * wa.h * ((wa.w + kWgPix - 1) / kWgPix);
    const int slices = std::max(1, std::min((rows + 3) / 4, std::max(1, sm_count / chunks)));
    k_conv_wgrad<COUT, NC><<<chunks * slices, 160, S::kSmem, s>>>(wa, chunks, slices, status);
    return cudaGetLastError();
}
