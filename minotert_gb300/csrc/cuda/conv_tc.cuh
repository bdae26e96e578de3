// tcgen05 implicit-GEMM 3x3 convolution for the denoiser (included inside
// denoise.cu's anonymous namespace, after ConvArgs), in two forms that share
// the shared-memory operand layout, the MMAs and the epilogue: k_conv_tc
// gathers the halo with per-thread cp.async (any source, including the
// nearest-upsampled one), k_conv_tma with tensor copies (sources at the
// output's resolution).
//
// One CTA (4 warps) computes ROWS output rows x 128 consecutive pixels x all
// COUT channels as ROWS GEMMs on the 5th-generation tensor cores: M = 128
// pixels per row, N = COUT, K = 9 taps x Cin, FP32 accumulators in tensor
// memory (row r in columns [r * COUT, (r + 1) * COUT)).  The input is walked
// in 16-channel slices of the virtual, concatenated, possibly upsampled
// input; for each slice the CTA stages the (ROWS + 2)-row x 130-pixel halo and
// the slice's 9 x COUT weights in shared memory, in the canonical no-swizzle
// K-major layout: each 8-channel half is a plane of 16-byte rows, so a core
// matrix is 8 consecutive rows (SBO = 128 B) and the second K half sits one
// plane further (LBO = the plane size).  A tap's A operand is the halo plane
// of its input row shifted by its column, i.e. a start address 16 * dx bytes
// later: the im2col never exists, and the output rows share the weight
// slice.  Slices stream through STAGES shared-memory stages with cp.async
// (16-byte copies, zero-filled outside the image): while the tensor cores
// run the 9 x ROWS MMAs of slice k (issued by one thread and committed to that
// stage's mbarrier) the copies of the next STAGES - 1 slices are in flight.
// The epilogue reads the accumulators with tcgen05.ld (warp w owns TMEM
// lanes 32w..32w+31 = pixels 32w..32w+31), adds the bias, applies ReLU and
// stores BF16 with 16-byte stores.
#pragma once

constexpr int kTcPix = 128;             // output pixels per row of a CTA (MMA M)
constexpr int kTcHalo = kTcPix + 2;     // input pixels per halo row
constexpr int kTcPlane = kTcHalo * 16;  // bytes of one 8-channel halo plane
__host__ __device__ constexpr int tc_abytes(int rows) { return (rows + 2) * 2 * kTcPlane; }
// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N and M
__host__ __device__ constexpr uint32_t tc_idesc(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(n >> 3) << 17) | (uint32_t(m >> 4) << 24);
}
// Output rows per CTA and pipeline depth per COUT, from a sweep on the 1080p
// denoiser (ms per frame: 2 rows everywhere 2.19, 4 rows up to COUT 64 1.77,
// 8 rows below COUT 64 and 4 above with two stages 1.70).  More rows share
// each weight slice and amortise the 2-row halo; COUT <= 64 keeps two CTAs
// per SM (<= 113 KB of shared memory, <= 256 tensor-memory columns each),
// COUT 128 runs one (512 columns).
__host__ __device__ constexpr int tc_rows(int cout) { return cout >= 64 ? 4 : 8; }
__host__ __device__ constexpr int tc_stages(int) { return 2; }
__host__ __device__ constexpr size_t tc_stage_bytes(int cout, int rows) {
    return size_t(tc_abytes(rows)) + size_t(9) * 2 * cout * 16;
}
__host__ __device__ constexpr size_t tc_smem_bytes(int cout, int rows, int stages) {
    return stages * tc_stage_bytes(cout, rows) + 64;
}

// 16-byte asynchronous copy global -> shared; zero-filled when !valid (the
// source is then not read)
__device__ __forceinline__ void cp16(uint32_t saddr, const void* g, bool valid) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(saddr), "l"(g), "r"(valid ? 16 : 0)
                 : "memory");
}

template <int COUT, int ROWS>
__device__ __forceinline__ void tc_load_slice(const ConvArgs& a, uint32_t As, uint32_t Bs, int n, int y0, int x0,
                                              int c0, int cin, int ha, int wa) {
    const int tid = threadIdx.x;
    // halo: input rows y0-1..y0+ROWS, pixels x0-1..x0+128, channels c0..c0+15
    for (int i = tid; i < (ROWS + 2) * 2 * kTcHalo; i += 128) {
        const int hf = i & 1, p = (i >> 1) % kTcHalo, r = (i >> 1) / kTcHalo;
        const int yy = y0 - 1 + r, xx = x0 - 1 + p, c = c0 + 8 * hf;
        const bool in = yy >= 0 && yy < a.h && xx >= 0 && xx < a.w_;
        const bf16* src = a.w;  // any valid address when zero-filling
        if (in) {
            if (c < a.ca) {
                const int ya = a.ups ? yy >> 1 : yy, xa = a.ups ? xx >> 1 : xx;
                src = a.a + ((size_t(n) * ha + ya) * wa + xa) * a.ca + c;
            } else {
                src = a.b + ((size_t(n) * a.h + yy) * a.w_ + xx) * a.cb + (c - a.ca);
            }
        }
        cp16(As + uint32_t((r * 2 + hf) * kTcPlane + p * 16), src, in);
    }
    // weights: 9 taps x 2 halves x COUT rows of 16 B
    for (int i = tid; i < 9 * 2 * COUT; i += 128) {
        const int co = i % COUT, hf = (i / COUT) & 1, t = i / (2 * COUT);
        cp16(Bs + uint32_t(((t * 2 + hf) * COUT + co) * 16), a.w + (size_t(co) * 9 + t) * cin + c0 + 8 * hf, true);
    }
}

// Epilogue shared by the convolution kernels: warp w reads TMEM lanes
// 32w..32w+31 (pixels x0 + 32w ..), ROWS x COUT FP32 accumulators, adds the
// bias, applies ReLU, zeroes the outputs whose gate is not positive (when the
// arguments carry a gate tensor) and stores BF16 with 16-byte stores.
template <int COUT, int ROWS>
__device__ __forceinline__ void tc_epilogue(const ConvArgs& a, uint32_t taddr, int n, int y0, int x0, int warp,
                                            int lane) {
    const int m = 32 * warp + lane, x = x0 + m;
    // per 16-channel group: its biases read once for the tile, and the
    // accumulators of up to four rows loaded before one wait
    constexpr int kBatch = ROWS < 4 ? ROWS : 4;
    static_assert(ROWS % kBatch == 0, "row batches");
#pragma unroll
    for (int jj = 0; jj < COUT / 16; ++jj) {
        float bias[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) bias[k] = a.bias[16 * jj + k];
#pragma unroll
        for (int r0 = 0; r0 < ROWS; r0 += kBatch) {
            uint32_t v[kBatch][16];
#pragma unroll
            for (int rr = 0; rr < kBatch; ++rr) {
                const uint32_t ta = taddr + (uint32_t(32 * warp) << 16) + uint32_t((r0 + rr) * COUT + 16 * jj);
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                    "[%16];\n"
                    : "=r"(v[rr][0]), "=r"(v[rr][1]), "=r"(v[rr][2]), "=r"(v[rr][3]), "=r"(v[rr][4]), "=r"(v[rr][5]),
                      "=r"(v[rr][6]), "=r"(v[rr][7]), "=r"(v[rr][8]), "=r"(v[rr][9]), "=r"(v[rr][10]), "=r"(v[rr][11]),
                      "=r"(v[rr][12]), "=r"(v[rr][13]), "=r"(v[rr][14]), "=r"(v[rr][15])
                    : "r"(ta));
            }
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int rr = 0; rr < kBatch; ++rr) {
                const int y = y0 + r0 + rr;
                if (x < a.w_ && y < a.h) {
                    bf16* dst = a.y + ((size_t(n) * a.h + y) * a.w_ + x) * COUT;
                    uint32_t packed[8], gv[8];
                    if (a.gate) {
                        const uint4* gp = reinterpret_cast<const uint4*>(
                            a.gate + ((size_t(n) * a.h + y) * a.w_ + x) * COUT + 16 * jj);
                        const uint4 g0 = gp[0], g1 = gp[1];
                        gv[0] = g0.x; gv[1] = g0.y; gv[2] = g0.z; gv[3] = g0.w;
                        gv[4] = g1.x; gv[5] = g1.y; gv[6] = g1.z; gv[7] = g1.w;
                    }
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        float f0 = __uint_as_float(v[rr][2 * q]) + bias[2 * q];
                        float f1 = __uint_as_float(v[rr][2 * q + 1]) + bias[2 * q + 1];
                        if (a.relu) {
                            f0 = fmaxf(f0, 0.0f);
                            f1 = fmaxf(f1, 0.0f);
                        }
                        if (a.gate) {
                            const float2 g = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&gv[q]));
                            if (!(g.x > 0.0f)) f0 = 0.0f;
                            if (!(g.y > 0.0f)) f1 = 0.0f;
                        }
                        const __nv_bfloat162 hv = __floats2bfloat162_rn(f0, f1);
                        packed[q] = *reinterpret_cast<const uint32_t*>(&hv);
                    }
                    uint4* o = reinterpret_cast<uint4*>(dst + 16 * jj);
                    o[0] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
                    o[1] = make_uint4(packed[4], packed[5], packed[6], packed[7]);
                }
            }
        }
    }
}

template <int COUT, int ROWS, int STAGES>
__global__ void __launch_bounds__(128) k_conv_tc(ConvArgs a, uint32_t* status) {
    constexpr int kAcc = ROWS * COUT;
    constexpr int kCols = kAcc < 32 ? 32 : kAcc;  // TMEM columns (power of 2, >= 32)
    static_assert(kCols <= 512 && (kCols & (kCols - 1)) == 0, "tensor memory columns");
    constexpr int kStages = STAGES;
    constexpr int kTcAbytes = tc_abytes(ROWS);
    constexpr uint32_t kStage = uint32_t(tc_stage_bytes(COUT, ROWS));
    extern __shared__ __align__(128) unsigned char tsm[];
    uint64_t* mbar = reinterpret_cast<uint64_t*>(tsm + kStages * kStage);  // one per stage
    uint32_t* slot = reinterpret_cast<uint32_t*>(mbar + kStages);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tiles_x = (a.w_ + kTcPix - 1) / kTcPix, rows_per_img = (a.h + ROWS - 1) / ROWS;
    const int tx = blockIdx.x % tiles_x, rb = blockIdx.x / tiles_x;
    const int y0 = (rb % rows_per_img) * ROWS, n = rb / rows_per_img;
    const int x0 = tx * kTcPix;
    const int cin = a.ca + a.cb, nk = cin / 16;
    const int ha = a.ups ? a.h >> 1 : a.h, wa = a.ups ? a.w_ >> 1 : a.w_;
    const uint32_t smem0 = smem_u32(tsm);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                     "r"(uint32_t(kCols))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < kStages; ++s)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar + s)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // prologue: slices 0 .. kStages-2 in flight
    for (int s = 0; s < kStages - 1; ++s) {
        if (s < nk) tc_load_slice<COUT, ROWS>(a, smem0 + s * kStage, smem0 + s * kStage + kTcAbytes, n, y0, x0, 16 * s, cin,
                                        ha, wa);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = *slot;
    constexpr uint32_t idesc = tc_idesc(kTcPix, COUT);
    bool timed_out = false;
    int issued = 0;  // slices whose MMAs were committed

    for (int k = 0; k < nk; ++k) {
        const int s = k % kStages;
        // slice k has landed (groups complete in order; kStages - 2 newer
        // groups may still be in flight)
        asm volatile("cp.async.wait_group %0;\n" ::"n"(kStages - 2) : "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t abase = smem0 + uint32_t(s) * kStage, bbase = abase + kTcAbytes;
#pragma unroll
            for (int r = 0; r < ROWS; ++r)
#pragma unroll
                for (int t = 0; t < 9; ++t) {
                    const int ky = t / 3, kx = t % 3;
                    const uint64_t ad = tc_sdesc(abase + ((r + ky) * 2) * kTcPlane + kx * 16, kTcPlane, 128);
                    const uint64_t bd = tc_sdesc(bbase + (t * 2) * COUT * 16, COUT * 16, 128);
                    const uint32_t acc = (k > 0 || t > 0) ? 1u : 0u;
                    asm volatile(
                        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(taddr + uint32_t(r * COUT)),
                        "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                        : "memory");
                }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(mbar + s))
                         : "memory");
        }
        issued = k + 1;
        // refill: slice k + kStages - 1 goes into the stage slice k - 1 used
        const int j = k + kStages - 1;
        if (j < nk) {
            if (k >= 1 && !tc_wait(smem_u32(mbar + (k - 1) % kStages), uint32_t((k - 1) / kStages) & 1u)) {
                timed_out = true;
                atomicOr(status, MRT_STATUS_PIPE_TIMEOUT);
            }
            timed_out = __syncthreads_or(timed_out) != 0;
            if (timed_out) break;
            const uint32_t st = smem0 + uint32_t(j % kStages) * kStage;
            tc_load_slice<COUT, ROWS>(a, st, st + kTcAbytes, n, y0, x0, 16 * j, cin, ha, wa);
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    // the slices not yet waited for: the last kStages committed (bounded even
    // after a timeout, so the tensor memory is only freed once they are done)
    for (int c = issued - kStages < 0 ? 0 : issued - kStages; c < issued; ++c)
        if (!tc_wait(smem_u32(mbar + c % kStages), uint32_t(c / kStages) & 1u)) {
            timed_out = true;
            atomicOr(status, MRT_STATUS_PIPE_TIMEOUT);
        }
    timed_out = __syncthreads_or(timed_out) != 0;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!timed_out) {
        tc_epilogue<COUT, ROWS>(a, taddr, n, y0, x0, warp, lane);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(uint32_t(kCols))
                     : "memory");
}

// ---- TMA form, for layers whose inputs are not upsampled ------------------
//
// One thread streams the slices with the Tensor Memory Accelerator and issues
// the MMAs.  Per slice: two tiled tensor loads of the halo (box 8 channels x
// 130 pixels x (ROWS + 2) rows from the NHWC source; rows and pixels outside
// the image read as zeros) and one bulk copy of the slice's weights from a
// copy laid out as [slice][tap][half][cout][8] (k_tc_weights), all
// completing on the stage's `full` mbarrier (expect_tx).  In shared memory
// the two 8-channel halves of the halo are each ROWS + 2 consecutive planes,
// each half starting on a 128-byte boundary (a tensor copy's shared-memory
// destination must be 128-byte aligned), so the A operand's leading byte
// offset (between K halves) is the padded half size.  Slices k+1 .. k+STAGES-1 are in flight while the MMAs of slice k
// run; a stage is refilled once the MMAs of the slice before have retired
// (its `empty` mbarrier, signalled by tcgen05.commit).  Every wait is
// bounded; on a timeout the thread sets the status bit, waits (bounded) for
// the copies and MMAs it issued and skips the epilogue.
template <int ROWS>
__host__ __device__ constexpr uint32_t tma_half_bytes() { return (uint32_t((ROWS + 2) * kTcPlane) + 127u) & ~127u; }
template <int ROWS>
__host__ __device__ constexpr uint32_t tma_halo_bytes() { return 2u * tma_half_bytes<ROWS>(); }
template <int COUT, int ROWS>
__host__ __device__ constexpr uint32_t tma_stage_bytes() {
    return (tma_halo_bytes<ROWS>() + uint32_t(9 * 2 * COUT * 16) + 127u) & ~127u;
}

__device__ __forceinline__ void tma_load_halo(uint32_t dst, const CUtensorMap* map, int c, int x, int y, int n,
                                              uint32_t mbar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c), "r"(x), "r"(y), "r"(n), "r"(mbar)
        : "memory");
}

template <int COUT, int ROWS, int STAGES>
__global__ void __launch_bounds__(128) k_conv_tma(ConvArgs a, const __grid_constant__ CUtensorMap map_a,
                                                  const __grid_constant__ CUtensorMap map_b, const bf16* wt,
                                                  uint32_t* status) {
    constexpr int kAcc = ROWS * COUT;
    constexpr int kCols = kAcc < 32 ? 32 : kAcc;
    static_assert(kCols <= 512 && (kCols & (kCols - 1)) == 0, "tensor memory columns");
    constexpr uint32_t kHalo = tma_halo_bytes<ROWS>(), kHalf = tma_half_bytes<ROWS>();
    static_assert(kHalf % 128u == 0u && kHalo % 128u == 0u, "tensor copy destinations are 128-byte aligned");
    // bytes the two halo boxes deliver (the halves' padding is not written)
    constexpr uint32_t kHaloTx = 2u * uint32_t((ROWS + 2) * kTcPlane);
    constexpr uint32_t kWBytes = uint32_t(9 * 2 * COUT * 16);
    constexpr uint32_t kStage = tma_stage_bytes<COUT, ROWS>();
    extern __shared__ __align__(128) unsigned char tsm[];
    uint64_t* full = reinterpret_cast<uint64_t*>(tsm + STAGES * kStage);
    uint64_t* empty = full + STAGES;
    uint32_t* slot = reinterpret_cast<uint32_t*>(empty + STAGES);
    uint32_t* ok_flag = slot + 1;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tiles_x = (a.w_ + kTcPix - 1) / kTcPix, rows_per_img = (a.h + ROWS - 1) / ROWS;
    const int tx = blockIdx.x % tiles_x, rb = blockIdx.x / tiles_x;
    const int y0 = (rb % rows_per_img) * ROWS, n = rb / rows_per_img;
    const int x0 = tx * kTcPix;
    const int cin = a.ca + a.cb, nk = cin / 16;
    const uint32_t smem0 = smem_u32(tsm);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                     "r"(uint32_t(kCols))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < STAGES; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(full + s)) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(empty + s)) : "memory");
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = *slot;

    if (tid == 0) {
        // after a timeout anywhere in this launch (or an earlier one) the
        // remaining CTAs skip their work, so a stuck pipeline costs one wave
        const bool skip = (*reinterpret_cast<volatile uint32_t*>(status) & MRT_STATUS_PIPE_TIMEOUT) != 0u;
        auto load = [&](int j) -> bool {  // slice j into stage j % STAGES
            const uint32_t st = smem0 + uint32_t(j % STAGES) * kStage, mb = smem_u32(full + j % STAGES);
            const int c = 16 * j;
            const CUtensorMap* map = c < a.ca ? &map_a : &map_b;
            const int cc = c < a.ca ? c : c - a.ca;
            // the copies' alignment rules, checked before anything is issued
            if ((st & 127u) != 0u || (cc & 7) != 0) return false;
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(kHaloTx + kWBytes)
                         : "memory");
            tma_load_halo(st, map, cc, x0 - 1, y0 - 1, n, mb);
            tma_load_halo(st + kHalf, map, cc + 8, x0 - 1, y0 - 1, n, mb);
            asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                             st + kHalo),
                         "l"(wt + size_t(j) * (kWBytes / 2)), "r"(kWBytes), "r"(mb)
                         : "memory");
            return true;
        };
        constexpr uint32_t idesc = tc_idesc(kTcPix, COUT);
        bool ok = !skip;
        int loaded = 0, issued = 0;
        for (; ok && loaded < STAGES && loaded < nk; ++loaded) ok = load(loaded);
        if (!ok && !skip) --loaded;  // the refused load was not issued
        for (int k = 0; ok && k < nk; ++k) {
            const int s = k % STAGES;
            if (!tc_wait(smem_u32(full + s), uint32_t(k / STAGES) & 1u)) {
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t abase = smem0 + uint32_t(s) * kStage, bbase = abase + kHalo;
#pragma unroll
            for (int r = 0; r < ROWS; ++r)
#pragma unroll
                for (int t = 0; t < 9; ++t) {
                    const int ky = t / 3, kx = t % 3;
                    const uint64_t ad = tc_sdesc(abase + (r + ky) * kTcPlane + kx * 16, kHalf, 128);
                    const uint64_t bd = tc_sdesc(bbase + (t * 2) * COUT * 16, COUT * 16, 128);
                    const uint32_t acc = (k > 0 || t > 0) ? 1u : 0u;
                    asm volatile(
                        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(taddr + uint32_t(r * COUT)),
                        "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                        : "memory");
                }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(empty + s))
                         : "memory");
            issued = k + 1;
            // refill the stage of slice k - 1 once its MMAs have retired
            if (k >= 1 && loaded < nk) {
                if (!tc_wait(smem_u32(empty + (k - 1) % STAGES), uint32_t((k - 1) / STAGES) & 1u) ||
                    !load(loaded)) {
                    ok = false;
                    break;
                }
                ++loaded;
            }
        }
        // drain what was issued: the last commit covers every MMA; loads
        // not consumed by an MMA are waited for on their full barriers
        if (issued > 0 && !tc_wait(smem_u32(empty + (issued - 1) % STAGES), uint32_t((issued - 1) / STAGES) & 1u))
            ok = false;
        for (int j = issued; j < loaded; ++j)
            if (!tc_wait(smem_u32(full + j % STAGES), uint32_t(j / STAGES) & 1u)) ok = false;
        if (!ok || issued < nk) {
            atomicOr(status, MRT_STATUS_PIPE_TIMEOUT);
            *ok_flag = 0u;
        } else {
            *ok_flag = 1u;
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (*ok_flag) {
        tc_epilogue<COUT, ROWS>(a, taddr, n, y0, x0, warp, lane);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(uint32_t(kCols))
                     : "memory");
}

// Weights of every layer re-laid out for the TMA form: per layer,
// [slice of 16 input channels][tap][half][cout][8 channels].
struct TcLayerTable {
    int cin[16], cout[16];
    size_t off[16];
    int count;
};
__global__ void k_tc_weights(const bf16* w16, bf16* wt, TcLayerTable t) {
    for (int l = 0; l < t.count; ++l) {
        const int cin = t.cin[l], cout = t.cout[l];
        const size_t total = size_t(9) * cin * cout;
        for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < total; i += size_t(gridDim.x) * blockDim.x) {
            const int e = int(i % 8);
            size_t q = i / 8;
            const int co = int(q % cout);
            q /= cout;
            const int hf = int(q % 2);
            q /= 2;
            const int tap = int(q % 9);
            const int k = int(q / 9);
            wt[t.off[l] + i] = w16[t.off[l] + (size_t(co) * 9 + tap) * cin + 16 * k + 8 * hf + e];
        }
    }
}

// Weights of the layers with COUT <= 32 for the row-stacked persistent form:
// per layer [slice of 16 input channels][kx][half][ky = 2, 1, 0][cout][8
// channels], so one tap column's three taps are one N = 3 COUT operand.
__global__ void k_tc_weights_stack(const bf16* w16, bf16* wt, TcLayerTable t) {
    for (int l = 0; l < t.count; ++l) {
        const int cin = t.cin[l], cout = t.cout[l];
        if (cout > 32) continue;
        const size_t total = size_t(9) * cin * cout;
        for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < total; i += size_t(gridDim.x) * blockDim.x) {
            const int e = int(i % 8);
            size_t q = i / 8;
            const int row = int(q % (3 * cout));
            q /= 3 * cout;
            const int hf = int(q % 2);
            q /= 2;
            const int kx = int(q % 3);
            const int k = int(q / 3);
            const int ky = 2 - row / cout, co = row % cout;
            wt[t.off[l] + i] = w16[t.off[l] + (size_t(co) * 9 + ky * 3 + kx) * cin + 16 * k + 8 * hf + e];
        }
    }
}

// Shapes of the TMA form per COUT, from sweeps on the 1080p denoiser (ms per
// inference, upsampling layers on the cp.async kernel: cp.async everywhere
// 1.607; TMA with 2 / 4 / 8 rows at COUT 128 / 64 / <= 32 1.341; 2 rows at
// COUT >= 64 and 4 below 1.307; 2 rows everywhere 1.350; 1 row at COUT >= 64
// 1.401; three stages 1.42-1.64): rows per CTA and two stages, two CTAs per
// SM.  With one thread driving a CTA's pipeline, more and smaller CTAs keep
// more copies and MMAs in flight.
__host__ __device__ constexpr int tma_rows(int cout) { return cout >= 64 ? 2 : 4; }
__host__ __device__ constexpr int tma_stages(int) { return 2; }

// NHWC BF16 tensor map with a box of one 8-channel half x box_x pixels x
// box_rows rows; x_stride 2 loads every other pixel (box_x / 2 of them)
inline bool tma_encode_box(CUtensorMap* map, const bf16* base, int c, int w, int h, int n, int box_x, int box_rows,
                           int x_stride) {
    using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    static EncodeFn fn = nullptr;
    if (!fn) {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !f)
            return false;
        fn = reinterpret_cast<EncodeFn>(f);
    }
    const cuuint64_t dims[4] = {cuuint64_t(c), cuuint64_t(w), cuuint64_t(h), cuuint64_t(n)};
    const cuuint64_t strides[3] = {cuuint64_t(c) * 2, cuuint64_t(c) * 2 * w, cuuint64_t(c) * 2 * w * h};
    const cuuint32_t box[4] = {8u, cuuint32_t(box_x), cuuint32_t(box_rows), 1u};
    const cuuint32_t estr[4] = {1u, cuuint32_t(x_stride), 1u, 1u};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<bf16*>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// the halo box of the convolutions: 130 pixels x (rows + 2) rows
inline bool tma_encode(CUtensorMap* map, const bf16* base, int c, int w, int h, int n, int rows) {
    return tma_encode_box(map, base, c, w, h, n, kTcHalo, rows + 2, 1);
}

// cudaFuncSetAttribute(MaxDynamicSharedMemorySize) once per device for the
// kernel whose flag word this is (bit d = device d configured)
template <class K>
cudaError_t tc_configure(K kernel, size_t smem, uint64_t& configured) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const uint64_t bit = uint64_t(1) << (dev & 63);
    if (configured & bit) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e == cudaSuccess) configured |= bit;
    return e;
}

template <int COUT>
cudaError_t launch_conv_tma(const ConvArgs& ca, const bf16* wt, uint32_t* status, cudaStream_t s) {
    constexpr int kRows = tma_rows(COUT), kStages = tma_stages(COUT);
    static uint64_t configured = 0;
    const size_t smem = size_t(kStages) * tma_stage_bytes<COUT, kRows>() + 128;
    cudaError_t e = tc_configure(k_conv_tma<COUT, kRows, kStages>, smem, configured);
    if (e != cudaSuccess) return e;
    CUtensorMap ma, mb;
    if (!tma_encode(&ma, ca.a, ca.ca, ca.w_, ca.h, ca.n, kRows)) return cudaErrorInvalidValue;
    if (ca.cb > 0) {
        if (!tma_encode(&mb, ca.b, ca.cb, ca.w_, ca.h, ca.n, kRows)) return cudaErrorInvalidValue;
    } else {
        mb = ma;
    }
    const int blocks = ((ca.w_ + kTcPix - 1) / kTcPix) * ((ca.h + kRows - 1) / kRows) * ca.n;
    k_conv_tma<COUT, kRows, kStages><<<blocks, 128, smem, s>>>(ca, ma, mb, wt, status);
    return cudaGetLastError();
}

// ---- persistent, warp-specialised TMA form ---------------------------------
//
// The same implicit GEMM with each CTA resident for the whole layer: it walks
// the output tiles (ROWS rows x 128 pixels) blockIdx.x, blockIdx.x +
// gridDim.x, ..., and its six warps split the work.  Warp 4 (one thread)
// streams the (tile, 16-channel slice) pairs into a ring of STAGES
// shared-memory stages with tensor copies (halo) and bulk copies (weights),
// each completing on the stage's `full` mbarrier; warp 5 (one thread) waits
// for a stage, issues its 9 x ROWS MMAs into one of two tensor-memory
// accumulators and commits them to the stage's `empty` mbarrier (releasing it
// to the producer) and, after a tile's last slice, to the accumulator's
// `acc_full` mbarrier; warps 0-3 (TMEM lanes 0-127) wait for `acc_full`, run
// the epilogue and arrive on `acc_empty`.  So the copies of the next tiles,
// the MMAs of this tile and the epilogue of the previous one overlap, and a
// layer with one or two slices per tile no longer pays a CTA's set-up,
// tensor-memory allocation and epilogue in series per tile.  Every wait is
// bounded and also ends when another role has given up (a shared abort
// word); the CTA then sets MRT_STATUS_PIPE_TIMEOUT, waits (bounded) for the
// copies and MMAs it issued and frees its tensor memory.  Sources are read
// at the output's resolution (the decoder's upsampling layers run k_conv_up).
//
// Row-stacked form (STACK, the 16- and 32-channel layers): an MMA costs a
// fixed ~46 cycles up to N = 64, so instead of one MMA per (output row, tap)
// with N = COUT, one MMA per (halo row h, tap column kx) feeds the three
// output rows h - 2, h - 1, h at once: N = 3 COUT with the weights of taps
// (2, kx), (1, kx), (0, kx) stacked, into accumulator blocks laid out per
// output row r at columns (r + 2) COUT, r = -2 .. ROWS + 1 (the four outer
// blocks only collect the edge rows' unused products).  Per slice (ROWS + 2)
// x 3 MMAs instead of 9 ROWS.  Blocks are written by overlapping MMAs, so a
// tile's accumulator is first cleared by one MMA of zero operands (N = the
// whole accumulator) and every real MMA accumulates.
template <int COUT, int ROWS, bool STACK>
__host__ __device__ constexpr int ws_acc_cols() { return STACK ? (ROWS + 4) * COUT : ROWS * COUT; }
template <int COUT, int ROWS, bool STACK>
__host__ __device__ constexpr uint32_t ws_zero_bytes() {
    return STACK ? uint32_t(128 * 32 + ws_acc_cols<COUT, ROWS, STACK>() * 32) : 0u;  // A and B zero operands
}
template <int COUT, int ROWS, int STAGES, bool STACK = false>
__host__ __device__ constexpr size_t ws_smem_bytes() {
    return size_t(STAGES) * tma_stage_bytes<COUT, ROWS>() + ws_zero_bytes<COUT, ROWS, STACK>() +
           size_t(2 * STAGES + 5) * 8 + 32;
}

__device__ __forceinline__ bool ws_wait(uint32_t mbar, uint32_t parity, const volatile uint32_t* abort) {
    for (uint32_t spins = 0; spins < kTcSpin; ++spins) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
        if (*abort) return false;
    }
    return false;
}

// Threads of the persistent forms: four epilogue warps, a producer warp (one
// thread issuing tensor and bulk copies), an MMA warp (one thread).
constexpr int kWsThreads = 6 * 32;

template <int COUT, int ROWS, int STAGES, bool STACK = false>
__global__ void __launch_bounds__(kWsThreads) k_conv_ws(ConvArgs a, const __grid_constant__ CUtensorMap map_a,
                                                              const __grid_constant__ CUtensorMap map_b, const bf16* wt,
                                                              uint32_t* status) {
    constexpr int kAcc = ws_acc_cols<COUT, ROWS, STACK>();  // TMEM columns of one accumulator
    constexpr uint32_t kZero = ws_zero_bytes<COUT, ROWS, STACK>();
    constexpr int kCols = 2 * kAcc < 32 ? 32 : 2 * kAcc;
    static_assert(kCols <= 512 && (kCols & (kCols - 1)) == 0, "tensor memory columns");
    constexpr uint32_t kHalo = tma_halo_bytes<ROWS>(), kHalf = tma_half_bytes<ROWS>();
    constexpr uint32_t kHaloTx = 2u * uint32_t((ROWS + 2) * kTcPlane);
    constexpr uint32_t kWBytes = uint32_t(9 * 2 * COUT * 16);
    constexpr uint32_t kStage = tma_stage_bytes<COUT, ROWS>();
    constexpr int kMmaWarp = 5;
    extern __shared__ __align__(128) unsigned char tsm[];
    uint64_t* full = reinterpret_cast<uint64_t*>(tsm + STAGES * kStage + kZero);
    uint64_t* empty = full + STAGES;
    uint64_t* acc_full = empty + STAGES;    // [2]
    uint64_t* acc_empty = acc_full + 2;     // [2]
    uint64_t* fin = acc_empty + 2;          // the MMA thread's final commit
    uint32_t* slot = reinterpret_cast<uint32_t*>(fin + 1);
    volatile uint32_t* abort = slot + 1;
    uint32_t* consumed = slot + 2;          // slices the MMA thread waited for
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tiles_x = (a.w_ + kTcPix - 1) / kTcPix, rows_per_img = (a.h + ROWS - 1) / ROWS;
    const int tiles = tiles_x * rows_per_img * a.n;
    const int cin = a.ca + a.cb, nk = cin / 16;
    const uint32_t smem0 = smem_u32(tsm);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                     "r"(uint32_t(kCols))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < STAGES; ++s) {  // full: the producer's expect_tx arrival
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(full + s)) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(empty + s)) : "memory");
        }
        for (int b = 0; b < 2; ++b) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(acc_full + b)) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 4;" ::"r"(smem_u32(acc_empty + b)) : "memory");
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(fin)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        // after a timeout anywhere in this launch (or an earlier one) the
        // remaining CTAs skip their work
        *abort = (*reinterpret_cast<volatile uint32_t*>(status) & MRT_STATUS_PIPE_TIMEOUT) != 0u ? 2u : 0u;
        *consumed = 0u;
    }
    if (STACK) {  // the zero operands of the accumulator-clearing MMA
        for (uint32_t i = tid; i < kZero / 16u; i += blockDim.x)
            reinterpret_cast<uint4*>(tsm + STAGES * kStage)[i] = make_uint4(0u, 0u, 0u, 0u);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = *slot;
    auto give_up = [&]() {
        if (*abort == 0u) atomicOr(status, MRT_STATUS_PIPE_TIMEOUT);
        *abort = 1u;
    };

    int produced = 0;
    if (warp == 4) {
        // producer (one thread): (tile, slice) pairs into the stage ring
        if (lane == 0) {
            int g = 0;
            bool ok = *abort == 0u;
            for (int tile = blockIdx.x; ok && tile < tiles; tile += gridDim.x) {
                const int tx = tile % tiles_x, rb = tile / tiles_x;
                const int y0 = (rb % rows_per_img) * ROWS, n = rb / rows_per_img, x0 = tx * kTcPix;
                for (int k = 0; k < nk; ++k, ++g) {
                    const int s = g % STAGES;
                    const uint32_t u = uint32_t(g / STAGES);
                    const uint32_t st = smem0 + uint32_t(s) * kStage, mb = smem_u32(full + s);
                    const int c = 16 * k;
                    const CUtensorMap* map = c < a.ca ? &map_a : &map_b;
                    const int cc = c < a.ca ? c : c - a.ca;
                    if (!ws_wait(smem_u32(empty + s), (u & 1u) ^ 1u, abort) || (st & 127u) != 0u || (cc & 7) != 0)
                        give_up();
                    if (*abort != 0u) { ok = false; break; }
                    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb),
                                 "r"(kHaloTx + kWBytes)
                                 : "memory");
                    tma_load_halo(st, map, cc, x0 - 1, y0 - 1, n, mb);
                    tma_load_halo(st + kHalf, map, cc + 8, x0 - 1, y0 - 1, n, mb);
                    asm volatile(
                        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                            st + kHalo),
                        "l"(wt + size_t(k) * (kWBytes / 2)), "r"(kWBytes), "r"(mb)
                        : "memory");
                    produced = g + 1;
                }
            }
        }
    } else if (warp == kMmaWarp) {
        if (lane == 0 && *abort == 0u) {  // MMA issuer
            constexpr uint32_t idesc = tc_idesc(kTcPix, COUT);
            int g = 0, it = 0;
            bool ok = true, any = false;
            for (int tile = blockIdx.x; ok && tile < tiles; tile += gridDim.x, ++it) {
                const int b = it & 1;
                const uint32_t ub = uint32_t(it >> 1);
                if (!ws_wait(smem_u32(acc_empty + b), (ub & 1u) ^ 1u, abort)) { ok = false; break; }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t tacc = taddr + uint32_t(b * kAcc);
                if (STACK) {  // clear the accumulator: zero A (128 x 16) times zero B (kAcc x 16)
                    const uint32_t za = smem0 + uint32_t(STAGES) * kStage;
                    asm volatile(
                        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, 0;\n" ::"r"(tacc),
                        "l"(tc_sdesc(za, 128 * 16, 128)), "l"(tc_sdesc(za + 128 * 32, kAcc * 16, 128)),
                        "r"(tc_idesc(kTcPix, kAcc))
                        : "memory");
                }
                for (int k = 0; k < nk; ++k, ++g) {
                    const int s = g % STAGES;
                    const uint32_t u = uint32_t(g / STAGES);
                    if (!ws_wait(smem_u32(full + s), u & 1u, abort)) { ok = false; break; }
                    *consumed = uint32_t(g + 1);
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t abase = smem0 + uint32_t(s) * kStage, bbase = abase + kHalo;
                    if (STACK) {
                        // halo row h, tap column kx -> output rows h - 2 .. h
                        // (accumulator blocks h .. h + 2), weights of taps
                        // (2, kx), (1, kx), (0, kx) stacked along N
                        constexpr uint32_t idesc3 = tc_idesc(kTcPix, 3 * COUT);
#pragma unroll
                        for (int hrow = 0; hrow < ROWS + 2; ++hrow)
#pragma unroll
                            for (int kx = 0; kx < 3; ++kx) {
                                const uint64_t ad = tc_sdesc(abase + hrow * kTcPlane + kx * 16, kHalf, 128);
                                const uint64_t bd = tc_sdesc(bbase + kx * 2 * 3 * COUT * 16, 3 * COUT * 16, 128);
                                asm volatile(
                                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, 1;\n" ::"r"(
                                        tacc + uint32_t(hrow * COUT)),
                                    "l"(ad), "l"(bd), "r"(idesc3)
                                    : "memory");
                            }
                    } else {
#pragma unroll
                        for (int r = 0; r < ROWS; ++r)
#pragma unroll
                            for (int t = 0; t < 9; ++t) {
                                const int ky = t / 3, kx = t % 3;
                                const uint64_t ad = tc_sdesc(abase + (r + ky) * kTcPlane + kx * 16, kHalf, 128);
                                const uint64_t bd = tc_sdesc(bbase + (t * 2) * COUT * 16, COUT * 16, 128);
                                const uint32_t acc = (k > 0 || t > 0) ? 1u : 0u;
                                asm volatile(
                                    "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
                                        tacc + uint32_t(r * COUT)),
                                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                                    : "memory");
                            }
                    }
                    any = true;
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                     smem_u32(empty + s))
                                 : "memory");
                }
                if (!ok) break;
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 smem_u32(acc_full + b))
                             : "memory");
            }
            if (!ok) give_up();
            // every MMA this thread issued has completed once this commit has
            if (any) {
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 smem_u32(fin))
                             : "memory");
                if (!tc_wait(smem_u32(fin), 0u) && *abort == 0u) {
                    atomicOr(status, MRT_STATUS_PIPE_TIMEOUT);
                    *abort = 1u;
                }
            }
        }
    } else {  // epilogue: warps 0-3, TMEM lanes 32 warp ..
        int it = 0;
        for (int tile = blockIdx.x; tile < tiles && *abort == 0u; tile += gridDim.x, ++it) {
            const int tx = tile % tiles_x, rb = tile / tiles_x;
            const int y0 = (rb % rows_per_img) * ROWS, n = rb / rows_per_img, x0 = tx * kTcPix;
            const int b = it & 1;
            const uint32_t ub = uint32_t(it >> 1);
            const bool ok = ws_wait(smem_u32(acc_full + b), ub & 1u, abort);
            if (!__all_sync(0xFFFFFFFFu, ok)) {
                if (lane == 0) give_up();
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            // (row-stacked: output row r is accumulator block r + 2)
            tc_epilogue<COUT, ROWS>(a, taddr + uint32_t(b * kAcc + (STACK ? 2 * COUT : 0)), n, y0, x0, warp, lane);
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(acc_empty + b)) : "memory");
        }
    }
    __syncthreads();
    // after an abort: the copies issued but never consumed land before the
    // shared memory is released
    if (tid == 128) {
        for (int g = int(*consumed); g < produced; ++g)
            if (!tc_wait(smem_u32(full + g % STAGES), uint32_t(g / STAGES) & 1u)) atomicOr(status, MRT_STATUS_PIPE_TIMEOUT);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(uint32_t(kCols))
                     : "memory");
}

// Shape of the persistent form per COUT: rows per tile (two accumulators of
// ROWS x COUT columns within the 512 TMEM columns) and ring stages, from
// sweeps of the 1080p inference (ms: 2 rows at COUT 64 1.008, 4 rows
// 0.981; 8 rows below COUT 64 no change).  Five stages for the 32- and
// 64-channel layers (one CTA per SM either way) measured slower: 0.883 ->
// 0.934 ms, e1a / e1b / d1b 51 / 58 / 58 -> 66 / 77 / 76 us
__host__ __device__ constexpr int ws_rows(int cout) { return cout >= 128 ? 2 : 4; }
__host__ __device__ constexpr int ws_stages(int cout) { return cout >= 128 ? 4 : 3; }

// STACK: the row-stacked form; its weights come as
// [slice][kx][half][ky = 2, 1, 0][COUT][8] (k_tc_weights_stack).
template <int COUT, bool STACK = false>
cudaError_t launch_conv_ws(const ConvArgs& ca, const bf16* wt, uint32_t* status, int sm_count, cudaStream_t s) {
    constexpr int kRows = ws_rows(COUT), kStages = ws_stages(COUT);
    constexpr int kAccCols = 2 * ws_acc_cols<COUT, kRows, STACK>();
    constexpr int kCols = kAccCols < 32 ? 32 : kAccCols;
    constexpr int kThreads = kWsThreads;
    static uint64_t configured = 0;
    static int per_sm = 0;
    static_assert(ws_smem_bytes<COUT, kRows, kStages, STACK>() <= 227u * 1024u, "shared memory of one CTA");
    const size_t smem = ws_smem_bytes<COUT, kRows, kStages, STACK>();
    cudaError_t e = tc_configure(k_conv_ws<COUT, kRows, kStages, STACK>, smem, configured);
    if (e != cudaSuccess) return e;
    if (per_sm == 0) {
        int occ = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_conv_ws<COUT, kRows, kStages, STACK>, kThreads, smem);
        if (e != cudaSuccess) return e;
        per_sm = std::max(1, std::min(occ, 512 / kCols));
    }
    if (ca.ups) return cudaErrorInvalidValue;  // upsampled sources: k_conv_up
    CUtensorMap ma, mb;
    if (!tma_encode(&ma, ca.a, ca.ca, ca.w_, ca.h, ca.n, kRows)) return cudaErrorInvalidValue;
    if (ca.cb > 0) {
        if (!tma_encode(&mb, ca.b, ca.cb, ca.w_, ca.h, ca.n, kRows)) return cudaErrorInvalidValue;
    } else {
        mb = ma;
    }
    const int tiles = ((ca.w_ + kTcPix - 1) / kTcPix) * ((ca.h + kRows - 1) / kRows) * ca.n;
    const int blocks = std::max(1, std::min(tiles, sm_count * per_sm));
    k_conv_ws<COUT, kRows, kStages, STACK><<<blocks, kThreads, smem, s>>>(ca, ma, mb, wt, status);
    return cudaGetLastError();
}

template <int COUT>
cudaError_t launch_conv_tc(const ConvArgs& ca, uint32_t* status, cudaStream_t s) {
    constexpr int kRows = tc_rows(COUT), kStages = tc_stages(COUT);
    static uint64_t configured = 0;
    const size_t smem = tc_smem_bytes(COUT, kRows, kStages);
    cudaError_t e = tc_configure(k_conv_tc<COUT, kRows, kStages>, smem, configured);
    if (e != cudaSuccess) return e;
    const int blocks = ((ca.w_ + kTcPix - 1) / kTcPix) * ((ca.h + kRows - 1) / kRows) * ca.n;
    k_conv_tc<COUT, kRows, kStages><<<blocks, 128, smem, s>>>(ca, status);
    return cudaGetLastError();
}

// ---- phase-decomposed form of the decoder's upsampling layers -------------
//
// Layers d1a / d0a read [nearest-2x-upsampled source A ++ skip source B].
// An output pixel (2Y + py, 2X + px) sees, through the 3x3 window over the
// upsampled A, only the 2 x 2 low-resolution pixels (Y + py - 1 + ry,
// X + px - 1 + rx), ry, rx in {0, 1}, with merged weights
//   W_{py,px}[ry][rx] = sum_{ky in S(py,ry)} sum_{kx in S(px,rx)} W[ky][kx],
// S(0,0) = {0}, S(0,1) = {1,2}, S(1,0) = {0,1}, S(1,1) = {2}: four 2x2
// convolutions on the low-resolution source instead of one 3x3 on four
// copies of each of its pixels (4/9 of the MMAs for A's channels), and the
// halo of A comes with tensor copies at its own resolution instead of a
// gather.  A tile is R low-resolution rows x 126 low-resolution columns,
// i.e. 2R output rows x 252 output columns in two column phases px; an
// accumulator block holds 128 lanes = output pixels (2(X0 + i) + px) of one
// output row j (lanes 126, 127 compute beyond the tile and are not stored).
// Blocks are laid out [px][j] x COUT columns so that one MMA serves every
// output row a halo row feeds (row-stacked along N, as in k_conv_ws): low-
// resolution halo row t feeds output rows j = 2t - py - 2ry, i.e. 2t - 3
// .. 2t, and for each (column shift s = px + rx, phase px) — (0,0), (1,0),
// (1,1), (2,1) — one MMA with the merged weights of those rows stacked.  The
// blocks are written by overlapping MMAs, so a tile's accumulator is
// cleared first by one MMA of zero operands.
// The skip source B at full resolution comes by tensor copies with an
// element stride of 2 into two planes per row, even and odd pixels (entry e
// of parity q = pixel 2(X0 - 1 + e) + q; a 256-pixel box loads 128 entries,
// which cover the 126 columns' taps; lanes 126, 127 read past them into the
// next row, unused), so that a phase's tap reads consecutive entries; per
// full-resolution halo row fr and member (px, kx) the tap reads plane
// parity q = (px + kx + 1) & 1 at shift o = (px + kx - 1 - q) / 2 + 1 and
// feeds output rows fr - 2 .. fr: one MMA with the unmerged weights of
// taps ky = 2, 1, 0 stacked.  Weights per 16-channel slice come from a copy
// laid out per MMA (k_up_weights; [half][rows][8]), of which an MMA reads
// the rows of the output rows inside the tile.  Roles, waits and abort
// handling are those of k_conv_ws.
constexpr int kUpCols = 126;    // low-resolution columns of a tile
constexpr int kUpEntries = 128; // skip-source entries per plane row: one 256-pixel, stride-2 tensor box
template <int COUT>
__host__ __device__ constexpr uint32_t up_wbytes_a() { return uint32_t(16 * COUT * 32); }  // 4 x (1+2+1) x COUT rows
template <int COUT>
__host__ __device__ constexpr uint32_t up_wbytes_b() { return uint32_t(18 * COUT * 32); }  // 3 x (1+2+2+1) x COUT rows
template <int R>
__host__ __device__ constexpr uint32_t up_half_a() { return (uint32_t((R + 2) * kTcPlane) + 127u) & ~127u; }
template <int R>
__host__ __device__ constexpr uint32_t up_half_b() { return uint32_t((2 * R + 2) * 2 * kUpEntries * 16); }
template <int COUT, int R>
__host__ __device__ constexpr uint32_t up_stage_bytes() {
    const uint32_t a = 2u * up_half_a<R>() + up_wbytes_a<COUT>();
    const uint32_t b = 2u * up_half_b<R>() + 128u + up_wbytes_b<COUT>();  // 128: the garbage rows' overrun
    return ((a > b ? a : b) + 127u) & ~127u;
}
// zero operands of the accumulator-clearing MMA: A (128 x 16) and B (4 R COUT x 16)
template <int COUT, int R>
__host__ __device__ constexpr uint32_t up_zero_bytes() { return uint32_t(128 * 32 + 4 * R * COUT * 32); }
template <int COUT, int R, int STAGES>
__host__ __device__ constexpr size_t up_smem_bytes() {
    return size_t(STAGES) * up_stage_bytes<COUT, R>() + up_zero_bytes<COUT, R>() + size_t(2 * STAGES + 5) * 8 + 32;
}
// Per-slice weights of the phase-decomposed form for one layer: slice k of
// the virtual input (A's channels first) at wup + k * (up_wbytes_b / 2)
// elements.  A slice: four variants v = (shift s, phase px) = (0,0), (1,0),
// (1,1), (2,1) (rx = s - px), each [half][4 COUT rows][8] with the rows in
// output-row order of one halo row t: (py, ry) = (1,1), (0,1), (1,0), (0,0)
// feed output rows 2t - 3 .. 2t; merged over the taps of S(py, ry) x
// S(px, rx) in FP32 and rounded to BF16.  B slice: six members (px, kx) =
// (0,0) .. (1,2), each [half][3 COUT rows][8] with ky = 2, 1, 0 (output rows
// fr - 2 .. fr of full-resolution halo row fr), the unmerged taps.
__global__ void k_up_weights(const bf16* w16, bf16* wup, int ca, int cb, int cout) {
    const int cin = ca + cb, nk = cin / 16, nka = ca / 16;
    const size_t slice = size_t(18) * cout * 16;  // elements of the larger (B) slice layout
    const size_t total = size_t(nk) * slice;
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < total; i += size_t(gridDim.x) * blockDim.x) {
        const int k = int(i / slice);
        int rem = int(i % slice);
        const int c0 = 16 * k;
        if (k < nka) {
            const int vsize = 4 * cout * 16;  // elements of one variant
            if (rem >= 4 * vsize) continue;
            const int v = rem / vsize, e = rem % vsize;
            const int hf = e / (4 * cout * 8), row = (e / 8) % (4 * cout), ci = c0 + 8 * hf + (e % 8);
            const int s = v == 0 ? 0 : (v == 3 ? 2 : 1), px = v >= 2 ? 1 : 0, rx = s - px;
            const int b = row / cout, co = row % cout;
            const int py = (b == 0 || b == 2) ? 1 : 0, ry = b <= 1 ? 1 : 0;
            const int ky0 = py == 0 ? (ry == 0 ? 0 : 1) : (ry == 0 ? 0 : 2);
            const int ky1 = py == 0 ? (ry == 0 ? 0 : 2) : (ry == 0 ? 1 : 2);
            const int kx0 = px == 0 ? (rx == 0 ? 0 : 1) : (rx == 0 ? 0 : 2);
            const int kx1 = px == 0 ? (rx == 0 ? 0 : 2) : (rx == 0 ? 1 : 2);
            float acc = 0.0f;
            for (int ky = ky0; ky <= ky1; ++ky)
                for (int kx = kx0; kx <= kx1; ++kx)
                    acc += __bfloat162float(w16[(size_t(co) * 9 + ky * 3 + kx) * cin + ci]);
            wup[i] = __float2bfloat16_rn(acc);
        } else {
            const int msize = 3 * cout * 16;  // elements of one member
            const int m = rem / msize, e = rem % msize;
            const int hf = e / (3 * cout * 8), row = (e / 8) % (3 * cout), ci = c0 + 8 * hf + (e % 8);
            const int kx = m % 3, ky = 2 - row / cout, co = row % cout;
            wup[i] = w16[(size_t(co) * 9 + ky * 3 + kx) * cin + ci];
        }
    }
}

// Epilogue of the phase-decomposed form: warp w reads TMEM lanes
// 32w..32w+31 (low-resolution column X0 + i, i = 32w + lane), the 4R
// accumulator blocks [px][j] (j = output row 2Y0 + j), adds the bias,
// applies ReLU and stores output pixel (2 Y0 + j, 2(X0 + i) + px) as BF16.
template <int COUT, int R>
__device__ __forceinline__ void up_epilogue(const ConvArgs& a, uint32_t taddr, int n, int Y0, int X0, int warp,
                                            int lane) {
    const int i = 32 * warp + lane;
    // per 16-channel group: its biases read once for the tile, and the
    // accumulators of four blocks loaded before one wait (as tc_epilogue)
    constexpr int kBlocks = 4 * R, kBatch = 4;
    static_assert(kBlocks % kBatch == 0, "block batches");
#pragma unroll
    for (int jj = 0; jj < COUT / 16; ++jj) {
        float bias[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) bias[k] = a.bias[16 * jj + k];
#pragma unroll
        for (int b0 = 0; b0 < kBlocks; b0 += kBatch) {
            uint32_t v[kBatch][16];
#pragma unroll
            for (int bb = 0; bb < kBatch; ++bb) {
                const uint32_t ta = taddr + (uint32_t(32 * warp) << 16) + uint32_t((b0 + bb) * COUT + 16 * jj);
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                    "[%16];\n"
                    : "=r"(v[bb][0]), "=r"(v[bb][1]), "=r"(v[bb][2]), "=r"(v[bb][3]), "=r"(v[bb][4]), "=r"(v[bb][5]),
                      "=r"(v[bb][6]), "=r"(v[bb][7]), "=r"(v[bb][8]), "=r"(v[bb][9]), "=r"(v[bb][10]), "=r"(v[bb][11]),
                      "=r"(v[bb][12]), "=r"(v[bb][13]), "=r"(v[bb][14]), "=r"(v[bb][15])
                    : "r"(ta));
            }
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int bb = 0; bb < kBatch; ++bb) {
                const int blk = b0 + bb;
                const int px = blk / (2 * R), j = blk % (2 * R);
                const int y = 2 * Y0 + j, x = 2 * (X0 + i) + px;
                if (i < kUpCols && x < a.w_ && y < a.h) {
                    bf16* dst = a.y + ((size_t(n) * a.h + y) * a.w_ + x) * COUT;
                    uint32_t packed[8];
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        float f0 = __uint_as_float(v[bb][2 * q]) + bias[2 * q];
                        float f1 = __uint_as_float(v[bb][2 * q + 1]) + bias[2 * q + 1];
                        if (a.relu) {
                            f0 = fmaxf(f0, 0.0f);
                            f1 = fmaxf(f1, 0.0f);
                        }
                        const __nv_bfloat162 hv = __floats2bfloat162_rn(f0, f1);
                        packed[q] = *reinterpret_cast<const uint32_t*>(&hv);
                    }
                    uint4* o = reinterpret_cast<uint4*>(dst + 16 * jj);
                    o[0] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
                    o[1] = make_uint4(packed[4], packed[5], packed[6], packed[7]);
                }
            }
        }
    }
}

template <int COUT, int R, int STAGES>
__global__ void __launch_bounds__(kWsThreads) k_conv_up(ConvArgs a, const __grid_constant__ CUtensorMap map_a,
                                                              const __grid_constant__ CUtensorMap map_b, const bf16* wup,
                                                              uint32_t* status) {
    constexpr int kAcc = 4 * R * COUT;  // TMEM columns of one accumulator set
    constexpr int kCols = 2 * kAcc < 32 ? 32 : 2 * kAcc;
    static_assert(kCols <= 512 && (kCols & (kCols - 1)) == 0, "tensor memory columns");
    constexpr uint32_t kHalfA = up_half_a<R>(), kHalfB = up_half_b<R>();
    constexpr uint32_t kHaloTxA = 2u * uint32_t((R + 2) * kTcPlane);
    constexpr uint32_t kWA = up_wbytes_a<COUT>(), kWB = up_wbytes_b<COUT>();
    constexpr uint32_t kStage = up_stage_bytes<COUT, R>();
    constexpr uint32_t kPlaneB = uint32_t((2 * R + 2) * kUpEntries * 16);  // one (half, parity) plane set
    constexpr uint32_t kHaloTxB = 4u * kPlaneB;
    constexpr uint32_t kWOffB = 2u * kHalfB + 128u;
    constexpr int kMmaWarp = 5;
    constexpr uint32_t kZero = up_zero_bytes<COUT, R>();
    static_assert(kAcc <= 256, "the clearing MMA spans the accumulator with N <= 256");
    extern __shared__ __align__(128) unsigned char tsm[];
    uint64_t* full = reinterpret_cast<uint64_t*>(tsm + STAGES * kStage + kZero);
    uint64_t* empty = full + STAGES;
    uint64_t* acc_full = empty + STAGES;    // [2]
    uint64_t* acc_empty = acc_full + 2;     // [2]
    uint64_t* fin = acc_empty + 2;
    uint32_t* slot = reinterpret_cast<uint32_t*>(fin + 1);
    volatile uint32_t* abort = slot + 1;
    uint32_t* consumed = slot + 2;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int hl = a.h >> 1, wl = a.w_ >> 1;  // low resolution (source A)
    const int tiles_x = (wl + kUpCols - 1) / kUpCols, rows_per_img = (hl + R - 1) / R;
    const int tiles = tiles_x * rows_per_img * a.n;
    const int cin = a.ca + a.cb, nk = cin / 16, nka = a.ca / 16;
    const uint32_t smem0 = smem_u32(tsm);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                     "r"(uint32_t(kCols))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < STAGES; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(full + s)) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(empty + s)) : "memory");
        }
        for (int b = 0; b < 2; ++b) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(acc_full + b)) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 4;" ::"r"(smem_u32(acc_empty + b)) : "memory");
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(fin)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *abort = (*reinterpret_cast<volatile uint32_t*>(status) & MRT_STATUS_PIPE_TIMEOUT) != 0u ? 2u : 0u;
        *consumed = 0u;
    }
    for (uint32_t i = tid; i < kZero / 16u; i += blockDim.x)
        reinterpret_cast<uint4*>(tsm + STAGES * kStage)[i] = make_uint4(0u, 0u, 0u, 0u);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the zero operands, for the tensor cores
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = *slot;
    auto give_up = [&]() {
        if (*abort == 0u) atomicOr(status, MRT_STATUS_PIPE_TIMEOUT);
        *abort = 1u;
    };

    int produced = 0;
    if (warp == 4) {
        // producer (one thread): per slice, tensor copies of the upsampled
        // source's low-resolution halo (A slices) or of the skip source's
        // even and odd pixels (element stride 2: entry e of parity q =
        // pixel 2 (X0 - 1 + e) + q, rows 2 Y0 - 1 .. 2 Y0 + 2R), and a bulk
        // copy of the slice's weights, all completing on the stage's `full`
        if (lane == 0) {
            int g = 0;
            bool ok = *abort == 0u;
            for (int tile = blockIdx.x; ok && tile < tiles; tile += gridDim.x) {
                const int tx = tile % tiles_x, rb = tile / tiles_x;
                const int Y0 = (rb % rows_per_img) * R, n = rb / rows_per_img, X0 = tx * kUpCols;
                for (int k = 0; k < nk; ++k, ++g) {
                    const int s = g % STAGES;
                    const uint32_t u = uint32_t(g / STAGES);
                    const uint32_t st = smem0 + uint32_t(s) * kStage, mb = smem_u32(full + s);
                    const bool is_a = k < nka;
                    if (!ws_wait(smem_u32(empty + s), (u & 1u) ^ 1u, abort) || (st & 127u) != 0u) give_up();
                    if (*abort != 0u) { ok = false; break; }
                    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb),
                                 "r"(is_a ? kHaloTxA + kWA : kHaloTxB + kWB)
                                 : "memory");
                    if (is_a) {
                        tma_load_halo(st, &map_a, 16 * k, X0 - 1, Y0 - 1, n, mb);
                        tma_load_halo(st + kHalfA, &map_a, 16 * k + 8, X0 - 1, Y0 - 1, n, mb);
                    } else {
                        const int c = 16 * k - a.ca;
#pragma unroll
                        for (int hf = 0; hf < 2; ++hf)
#pragma unroll
                            for (int q = 0; q < 2; ++q)
                                tma_load_halo(st + uint32_t(hf) * kHalfB + uint32_t(q) * kPlaneB, &map_b, c + 8 * hf,
                                              2 * (X0 - 1) + q, 2 * Y0 - 1, n, mb);
                    }
                    asm volatile(
                        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                            st + (is_a ? 2u * kHalfA : kWOffB)),
                        "l"(wup + size_t(k) * (kWB / 2)), "r"(is_a ? kWA : kWB), "r"(mb)
                        : "memory");
                    produced = g + 1;
                }
            }
        }
    } else if (warp == kMmaWarp) {
        if (lane == 0 && *abort == 0u) {
            int g = 0, it = 0;
            bool ok = true, any = false;
            // stage-0 descriptors: A-source halo, skip planes, weight
            // blocks (leading byte offset = one K half of the whole variant /
            // member block, whose row sub-range an MMA reads)
            const uint64_t da_a = tc_sdesc(smem0, kHalfA, 128), da_b = tc_sdesc(smem0, kHalfB, 128);
            const uint64_t dw_a = tc_sdesc(smem0 + 2u * kHalfA, 4 * COUT * 16, 128);
            const uint64_t dw_b = tc_sdesc(smem0 + kWOffB, 3 * COUT * 16, 128);
            const uint32_t za = smem0 + uint32_t(STAGES) * kStage;
            for (int tile = blockIdx.x; ok && tile < tiles; tile += gridDim.x, ++it) {
                const int b = it & 1;
                const uint32_t ub = uint32_t(it >> 1);
                if (!ws_wait(smem_u32(acc_empty + b), (ub & 1u) ^ 1u, abort)) { ok = false; break; }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t tacc = taddr + uint32_t(b * kAcc);
                // the blocks are written by overlapping MMAs: clear them
                // first (zero A times zero B, N = the whole accumulator)
                asm volatile("tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, 0;\n" ::"r"(tacc),
                             "l"(tc_sdesc(za, 128 * 16, 128)), "l"(tc_sdesc(za + 128 * 32, kAcc * 16, 128)),
                             "r"(tc_idesc(kTcPix, kAcc))
                             : "memory");
                for (int k = 0; k < nk; ++k, ++g) {
                    const int s = g % STAGES;
                    const uint32_t u = uint32_t(g / STAGES);
                    if (!ws_wait(smem_u32(full + s), u & 1u, abort)) { ok = false; break; }
                    *consumed = uint32_t(g + 1);
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    // descriptors are the stage-0 bases plus (byte offset / 16):
                    // only the 14-bit start field changes (no carry: shared
                    // addresses stay below 2^18)
                    const uint64_t so = uint64_t((uint32_t(s) * kStage) >> 4);
                    auto mma = [&](int blk0, int nblk, uint64_t ad, uint64_t bd) {
                        asm volatile("tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, 1;\n" ::"r"(
                                         tacc + uint32_t(blk0 * COUT)),
                                     "l"(ad), "l"(bd), "r"(tc_idesc(kTcPix, nblk * COUT))
                                     : "memory");
                    };
                    if (k < nka) {
                        // halo row t feeds output rows 2t - 3 .. 2t (those in the
                        // tile); per variant (shift, phase) one MMA
                        const uint64_t a0 = da_a + so, w0 = dw_a + so;
#pragma unroll
                        for (int t = 0; t < R + 2; ++t) {
                            const int jlo = 2 * t - 3 < 0 ? 0 : 2 * t - 3, jhi = 2 * t < 2 * R - 1 ? 2 * t : 2 * R - 1;
                            const uint64_t row = a0 + uint64_t((t * kTcPlane) >> 4);
                            const uint64_t roff = uint64_t(((jlo - (2 * t - 3)) * COUT * 16) >> 4);
#pragma unroll
                            for (int v = 0; v < 4; ++v) {
                                const int sh = v == 0 ? 0 : (v == 3 ? 2 : 1), px = v >= 2 ? 1 : 0;
                                mma(px * 2 * R + jlo, jhi - jlo + 1, row + uint64_t(sh),
                                    w0 + uint64_t((v * 4 * COUT * 32) >> 4) + roff);
                            }
                        }
                    } else {
                        // full-resolution halo row fr feeds output rows fr - 2 .. fr;
                        // per member (phase, tap column) one MMA on its (parity,
                        // shift) plane
                        const uint64_t a0 = da_b + so, w0 = dw_b + so;
#pragma unroll
                        for (int fr = 0; fr < 2 * R + 2; ++fr) {
                            const int jlo = fr - 2 < 0 ? 0 : fr - 2, jhi = fr < 2 * R - 1 ? fr : 2 * R - 1;
                            const uint64_t roff = uint64_t(((jlo - (fr - 2)) * COUT * 16) >> 4);
#pragma unroll
                            for (int m = 0; m < 6; ++m) {
                                const int px = m / 3, kx = m % 3;
                                const int q = (px + kx + 1) & 1, o = (px + kx - 1 - q) / 2 + 1;
                                const uint64_t ad =
                                    a0 + uint64_t((uint32_t(q) * kPlaneB + uint32_t(fr * kUpEntries + o) * 16u) >> 4);
                                mma(px * 2 * R + jlo, jhi - jlo + 1, ad,
                                    w0 + uint64_t((m * 2 * 3 * COUT * 16) >> 4) + roff);
                            }
                        }
                    }
                    any = true;
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                     smem_u32(empty + s))
                                 : "memory");
                }
                if (!ok) break;
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 smem_u32(acc_full + b))
                             : "memory");
            }
            if (!ok) give_up();
            if (any) {
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 smem_u32(fin))
                             : "memory");
                if (!tc_wait(smem_u32(fin), 0u) && *abort == 0u) {
                    atomicOr(status, MRT_STATUS_PIPE_TIMEOUT);
                    *abort = 1u;
                }
            }
        }
    } else {  // epilogue: warps 0-3
        int it = 0;
        for (int tile = blockIdx.x; tile < tiles && *abort == 0u; tile += gridDim.x, ++it) {
            const int tx = tile % tiles_x, rb = tile / tiles_x;
            const int Y0 = (rb % rows_per_img) * R, n = rb / rows_per_img, X0 = tx * kUpCols;
            const int b = it & 1;
            const uint32_t ub = uint32_t(it >> 1);
            const bool ok = ws_wait(smem_u32(acc_full + b), ub & 1u, abort);
            if (!__all_sync(0xFFFFFFFFu, ok)) {
                if (lane == 0) give_up();
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            up_epilogue<COUT, R>(a, taddr + uint32_t(b * kAcc), n, Y0, X0, warp, lane);
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(acc_empty + b)) : "memory");
        }
    }
    __syncthreads();
    if (tid == 128) {
        for (int g = int(*consumed); g < produced; ++g)
            if (!tc_wait(smem_u32(full + g % STAGES), uint32_t(g / STAGES) & 1u)) atomicOr(status, MRT_STATUS_PIPE_TIMEOUT);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(uint32_t(kCols))
                     : "memory");
}

// Shape of the phase-decomposed form per COUT: low-resolution rows per tile
// (two accumulator sets of 4 R COUT columns within the 512 TMEM columns)
// and ring stages, from sweeps of the 1080p inference (ms with the above:
// 2 stages 0.981, 3 stages 0.966; one row at COUT 32 0.994)
__host__ __device__ constexpr int up_rows(int cout) { return cout >= 64 ? 1 : 2; }
__host__ __device__ constexpr int up_stages(int) { return 3; }

template <int COUT>
cudaError_t launch_conv_up(const ConvArgs& ca, const bf16* wup, uint32_t* status, int sm_count, cudaStream_t s) {
    constexpr int kR = up_rows(COUT), kStages = up_stages(COUT);
    constexpr int kCols = 2 * 4 * kR * COUT;
    constexpr int kThreads = kWsThreads;
    static uint64_t configured = 0;
    static int per_sm = 0;
    const size_t smem = up_smem_bytes<COUT, kR, kStages>();
    cudaError_t e = tc_configure(k_conv_up<COUT, kR, kStages>, smem, configured);
    if (e != cudaSuccess) return e;
    if (per_sm == 0) {
        int occ = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_conv_up<COUT, kR, kStages>, kThreads, smem);
        if (e != cudaSuccess) return e;
        per_sm = std::max(1, std::min(occ, 512 / kCols));
    }
    if (!ca.ups || ca.cb <= 0 || (ca.h & 1) || (ca.w_ & 1) || ca.ca % 16 || ca.cb % 16) return cudaErrorInvalidValue;
    CUtensorMap ma, mb;
    if (!tma_encode(&ma, ca.a, ca.ca, ca.w_ / 2, ca.h / 2, ca.n, kR) ||
        !tma_encode_box(&mb, ca.b, ca.cb, ca.w_, ca.h, ca.n, 2 * kUpEntries, 2 * kR + 2, 2))
        return cudaErrorInvalidValue;
    const int tiles = ((ca.w_ / 2 + kUpCols - 1) / kUpCols) * ((ca.h / 2 + kR - 1) / kR) * ca.n;
    const int blocks = std::max(1, std::min(tiles, sm_count * per_sm));
    k_conv_up<COUT, kR, kStages><<<blocks, kThreads, smem, s>>>(ca, ma, mb, wup, status);
    return cudaGetLastError();
}
