// Learned radiance cache: a multiresolution hash-grid encoding of position
// plus normal and view direction into a 64-wide MLP, trained online on the
// path tracer's own samples and queried at the first diffuse bounce so
// paths end there (neural radiance caching in the manner of Mueller et al.,
// "Real-time Neural Radiance Caching for Path Tracing", SIGGRAPH 2021, with
// the hash encoding of Mueller et al., "Instant Neural Graphics Primitives",
// SIGGRAPH 2022).  The reference has no learned component; all of this is
// new.
//
// Network: input 64 halves = 32 hash features (16 levels x 2) + normal (3)
// + direction (3) + zero padding; 4 hidden layers of width 64 with ReLU,
// no biases; a linear output of 3 (padded to 16 rows of weights).  FP16
// weights and activations, FP32 accumulation, on the tensor cores through
// mma.sync.m16n8k16: a warp owns 16 rows, and the FP32 accumulator tiles of
// one layer (16 x 64) are, element for element, the A fragments of the next
// layer's product after packing to half2, so activations stay in registers.
// Weight gradients are FP32 sums over rows on the CUDA cores; the grid's
// gradients are FP32 atomics; Adam keeps FP32 master weights.
#include "internal.hpp"
#include "tcgen05.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

namespace mrt {
int set_error(mrt_ctx* ctx, int code, const char* msg);
int persistent_blocks(mrt_ctx* ctx);
TraceParams make_trace_params(const mrt_trace_params* p);
FrameParams make_frame_params(const mrt_camera_consts* c, uint32_t w, uint32_t h);
}

using namespace mrt;

namespace {

constexpr int kLevels = 16, kFeat = 2, kEnc = kLevels * kFeat;  // 32 encoded features
constexpr int kWidth = 64;                                     // hidden width = padded input width
constexpr int kHidden = 4;                                     // hidden layers
constexpr int kOutRows = 16;                                   // output weight rows (3 used)
constexpr int kLayerW = kWidth * kWidth;                       // 4096 weights per hidden layer
constexpr int kWeights = kHidden * kLayerW + kOutRows * kWidth; // 17408
constexpr int kMlpWarps = 4;                                   // warps per MLP block (16 rows each)
constexpr float kGradScale = 1024.0f;  // loss scale of the FP16 backward (undone on the gradients)

struct GridSpec {
    uint32_t log2_t;           // entries per level = 2^log2_t
    float base_res, growth;    // resolution of level l = base_res * growth^l
};

__device__ __forceinline__ uint32_t pack_half2(float a, float b) {
    __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
}

__device__ __forceinline__ void mma16816(float* d, const uint32_t* a, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// ---------------------------------------------------------------- encoding

struct Corner {
    uint32_t idx[kLevels][8];
    float w[kLevels][8];
};

__device__ __forceinline__ uint32_t grid_index(uint32_t x, uint32_t y, uint32_t z, uint32_t res, bool dense,
                                               uint32_t mask) {
    if (dense) return x + res * (y + res * z);
    return ((x * 1u) ^ (y * 2654435761u) ^ (z * 805459861u)) & mask;
}

// Corner indices (table-wide) and trilinear weights of position p in [0,1]^3
// on level l.  Level l has scale s_l = base_res * growth^l cells per unit;
// dense indexing while (ceil(s_l) + 2)^3 fits the table, hashed otherwise.
__device__ __forceinline__ void level_corners(const GridSpec& g, int l, float px, float py, float pz,
                                              uint32_t idx[8], float w[8]) {
    const uint32_t T = 1u << g.log2_t, mask = T - 1u;
    const float s = g.base_res * exp2f(float(l) * log2f(g.growth));
    const uint32_t res = uint32_t(ceilf(s)) + 2u;
    const bool dense = uint64_t(res) * res * res <= T;
    const float fx = px * s, fy = py * s, fz = pz * s;
    const float x0 = floorf(fx), y0 = floorf(fy), z0 = floorf(fz);
    const float tx = fx - x0, ty = fy - y0, tz = fz - z0;
    const uint32_t ix = uint32_t(x0), iy = uint32_t(y0), iz = uint32_t(z0);
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const uint32_t cx = c & 1, cy = (c >> 1) & 1, cz = c >> 2;
        idx[c] = uint32_t(l) * T + grid_index(ix + cx, iy + cy, iz + cz, res, dense, mask);
        w[c] = (cx ? tx : 1.0f - tx) * (cy ? ty : 1.0f - ty) * (cz ? tz : 1.0f - tz);
    }
}

// Encoded features of levels [l0, l1) of one query (position p in [0,1]^3,
// clamped) into row[2l], row[2l+1].  Two levels at a time, so 16 corner
// loads are in flight per lane.
__device__ void encode_levels(const GridSpec& g, const __half2* grid, const float* q, __half* row, int l0, int l1) {
    const float px = fminf(fmaxf(q[0], 0.0f), 1.0f), py = fminf(fmaxf(q[1], 0.0f), 1.0f),
                pz = fminf(fmaxf(q[2], 0.0f), 1.0f);
#pragma unroll 2
    for (int l = l0; l < l1; ++l) {
        uint32_t idx[8];
        float w[8];
        level_corners(g, l, px, py, pz, idx, w);
        float f0 = 0.0f, f1 = 0.0f;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const float2 v = __half22float2(grid[idx[c]]);
            f0 = fmaf(w[c], v.x, f0);
            f1 = fmaf(w[c], v.y, f1);
        }
        row[2 * l] = __float2half_rn(f0);
        row[2 * l + 1] = __float2half_rn(f1);
    }
}

// Normal, direction and the zero padding of an input row.
__device__ void encode_tail(const float* q, __half* row) {
    for (int k = 0; k < 6; ++k) row[kEnc + k] = __float2half_rn(q[3 + k]);
    for (int k = kEnc + 6; k < kWidth; ++k) row[k] = __float2half_rn(0.0f);
}

// The 16 rows of a warp's tile encoded by all 32 lanes: lane i takes row
// i mod 16 and half of its levels (i < 16: levels 0-7 and the normal /
// direction / padding; i >= 16: levels 8-15), so twice as many hash-grid
// gathers are in flight as with one lane per row.  q_row(r, qq) fills the 9
// floats of tile row r (zeros past the end).
template <class QRow>
__device__ __forceinline__ void encode_tile(const GridSpec& g, const __half2* grid, __half* X, QRow q_row) {
    const int lane = int(lane_id()), r = lane & 15, half = lane >> 4;
    float qq[9];
    q_row(r, qq);
    encode_levels(g, grid, qq, X + r * kWidth, half * (kLevels / 2), (half + 1) * (kLevels / 2));
    if (!half) encode_tail(qq, X + r * kWidth);
}

// ------------------------------------------------------------ MLP on mma

// Weights in shared memory, row-major [out][in] halves per layer, followed by
// the transposes ([in][out]) for the backward pass.  B fragment of an 8-wide
// n-tile j and a 16-deep k-tile k: b0 = W[8j + g][16k + 2t .. +1],
// b1 = W[8j + g][16k + 8 + 2t .. +1].
__device__ __forceinline__ void load_b(const __half* W, int in_w, int j, int k, uint32_t& b0, uint32_t& b1) {
    const int g = lane_id() >> 2, t = lane_id() & 3;
    const __half* r = W + (8 * j + g) * in_w + 16 * k + 2 * t;
    b0 = *reinterpret_cast<const uint32_t*>(r);
    b1 = *reinterpret_cast<const uint32_t*>(r + 8);
}

// A fragments of a 16 x 64 half tile stored row-major in shared memory
__device__ __forceinline__ void load_a(const __half* X, int ld, uint32_t a[4][4]) {
    const int g = lane_id() >> 2, t = lane_id() & 3;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const __half* r0 = X + g * ld + 16 * k + 2 * t;
        const __half* r1 = X + (g + 8) * ld + 16 * k + 2 * t;
        a[k][0] = *reinterpret_cast<const uint32_t*>(r0);
        a[k][1] = *reinterpret_cast<const uint32_t*>(r1);
        a[k][2] = *reinterpret_cast<const uint32_t*>(r0 + 8);
        a[k][3] = *reinterpret_cast<const uint32_t*>(r1 + 8);
    }
}

// acc (8 n-tiles x 4) of a 16 x 64 layer output -> ReLU -> A fragments
__device__ __forceinline__ void acc_to_a(const float acc[8][4], uint32_t a[4][4], bool relu) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float* c0 = acc[2 * k];
        const float* c1 = acc[2 * k + 1];
        auto r = [&](float v) { return relu ? fmaxf(v, 0.0f) : v; };
        a[k][0] = pack_half2(r(c0[0]), r(c0[1]));
        a[k][1] = pack_half2(r(c0[2]), r(c0[3]));
        a[k][2] = pack_half2(r(c1[0]), r(c1[1]));
        a[k][3] = pack_half2(r(c1[2]), r(c1[3]));
    }
}

// out(16 x 8*ntiles) = A(16 x 64) * W^T, W row-major [out][64]
template <int kNTiles>
__device__ __forceinline__ void layer(const uint32_t a[4][4], const __half* W, float acc[kNTiles][4]) {
#pragma unroll
    for (int j = 0; j < kNTiles; ++j) {
        acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            uint32_t b0, b1;
            load_b(W, kWidth, j, k, b0, b1);
            mma16816(acc[j], a[k], b0, b1);
        }
    }
}

// Forward of 16 rows whose inputs sit row-major in shared memory; hidden
// activations optionally stored (post-ReLU, half) for training; output
// (16 x 3) written as float.
__device__ void mlp_forward_tile(const __half* sW, const __half* X, __half* act_out /* 4 x 16 x 64 or null */,
                                 size_t act_ld, float* out /* 16 x 3 */) {
    uint32_t a[4][4];
    float acc[8][4];
    load_a(X, kWidth, a);
    const int g = lane_id() >> 2, t = lane_id() & 3;
#pragma unroll 1
    for (int l = 0; l < kHidden; ++l) {
        layer<8>(a, sW + l * kLayerW, acc);
        acc_to_a(acc, a, true);
        if (act_out) {
            __half* base = act_out + size_t(l) * act_ld;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                *reinterpret_cast<uint32_t*>(base + g * kWidth + 16 * k + 2 * t) = a[k][0];
                *reinterpret_cast<uint32_t*>(base + (g + 8) * kWidth + 16 * k + 2 * t) = a[k][1];
                *reinterpret_cast<uint32_t*>(base + g * kWidth + 16 * k + 8 + 2 * t) = a[k][2];
                *reinterpret_cast<uint32_t*>(base + (g + 8) * kWidth + 16 * k + 8 + 2 * t) = a[k][3];
            }
        }
    }
    float o[1][4];
    layer<1>(a, sW + kHidden * kLayerW, o);  // first 8 output rows; rows 0..2 used
    // o: (row g, cols 2t,2t+1), (row g+8, cols 2t, 2t+1)
    const int c0 = 2 * t, c1 = 2 * t + 1;
    if (c0 < 3) { out[g * 3 + c0] = o[0][0]; out[(g + 8) * 3 + c0] = o[0][2]; }
    if (c1 < 3) { out[g * 3 + c1] = o[0][1]; out[(g + 8) * 3 + c1] = o[0][3]; }
}

__device__ void load_weights_smem(__half* sW, const __half* W, int count) {
    for (int i = threadIdx.x; i < count / 2; i += blockDim.x)
        reinterpret_cast<uint32_t*>(sW)[i] = reinterpret_cast<const uint32_t*>(W)[i];
}

} // namespace

// ---------------------------------------------------------------- kernels

namespace mrt {

struct CacheDev {
    GridSpec spec;
    const __half2* grid;  // levels * 2^log2_t entries of 2 features
    const __half* W;      // kWeights halves (hidden layers, then output rows)
    const __half* WT;     // transposes of the hidden layers + output ([in][out], 64 x 16)
    float lo[3], inv_ext[3];
};

} // namespace mrt

namespace {

// Inference: rows of 9 floats (position normalised to [0,1]^3, normal,
// direction) -> 3 floats.  One block = kMlpWarps warps x 16 rows.
__global__ void __launch_bounds__(kMlpWarps * 32)
k_cache_infer(CacheDev c, const float* q, uint32_t n_max, const uint32_t* n_dev, float* out) {
    extern __shared__ __align__(16) unsigned char smem[];
    __half* sW = reinterpret_cast<__half*>(smem);
    __half* sX = sW + kWeights;  // kMlpWarps x 16 x 64
    float* sO = reinterpret_cast<float*>(sX + kMlpWarps * 16 * kWidth);  // kMlpWarps x 16 x 3
    const uint32_t n = n_dev ? min(*n_dev, n_max) : n_max;
    load_weights_smem(sW, c.W, kWeights);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = lane_id();
    __half* X = sX + warp * 16 * kWidth;
    float* O = sO + warp * 16 * 3;
    for (uint32_t base = (blockIdx.x * kMlpWarps + warp) * 16u; base < n; base += gridDim.x * kMlpWarps * 16u) {
        encode_tile(c.spec, c.grid, X, [&](int rr, float* qq) {
            const uint32_t r = base + uint32_t(rr);
            for (int k = 0; k < 9; ++k) qq[k] = r < n ? q[size_t(r) * 9 + k] : 0.0f;
        });
        __syncwarp();
        mlp_forward_tile(sW, X, nullptr, 0, O);
        __syncwarp();
        if (lane < 16 && base + lane < n)
            for (int k = 0; k < 3; ++k) out[size_t(base + lane) * 3 + k] = O[lane * 3 + k];
        __syncwarp();
    }
}

// ---------------------------------------------------------- MLP on tcgen05
//
// Inference on the 5th-generation tensor cores.  A CTA of 256 threads owns
// a tile of 128 queries at a time (persistent over the tiles): the encoded
// input rows are written into shared memory in the canonical K-major layout
// (eight 2 KB planes, plane k holding elements 8k..8k+7 of each of the 128
// rows), then each layer is one 128 x 64 x 64 product issued by one thread
// as four tcgen05.mma kind::f16 (K = 16 each: FP16 A and B, FP32 accumulator
// in 64 tensor-memory columns) and committed to an mbarrier; all 8 warps
// read the accumulators back (warp w: lanes 32 (w mod 4) .., columns
// 32 (w / 4) ..), apply ReLU, round to FP16 and write them over the tile as
// the next layer's A operand.  The output layer is N = 16 (3 used).  The
// weights sit in shared memory in the same layout for the whole launch
// (4 x 8 KB + 2 KB).  Every wait is bounded: on a timeout the CTA sets
// MRT_STATUS_PIPE_TIMEOUT, stops, waits (bounded) for its last commit and
// frees its tensor memory.

constexpr int kTcRows = 128;                               // queries per tile (MMA M)
constexpr int kTcPlaneA = kTcRows * 16;                    // bytes of one 8-element K plane of the tile
constexpr int kTcLayerB = kWidth * 16 * (kWidth / 8);      // 8 KB: one hidden layer's weights
constexpr int kTcOutB = kOutRows * 16 * (kWidth / 8);      // 2 KB: the output layer's weights
constexpr int kTcWBytes = kHidden * kTcLayerB + kTcOutB;   // 34 KB
constexpr int kTcSmem = kTcWBytes + (kWidth / 8) * kTcPlaneA + 64;
constexpr int kTcThreads = 256;

// instruction descriptor of kind::f16 with FP16 A and B, FP32 accumulator,
// both operands K-major
__host__ __device__ constexpr uint32_t mlp_idesc(int m, int n) {
    return (1u << 4) | (uint32_t(n >> 3) << 17) | (uint32_t(m >> 4) << 24);
}

// The weights (row-major [out][64] halves, hidden layers then the output
// rows) into the K-plane layout: hidden layer l at l * 8 KB, plane kc of it
// holding element 8 kc .. 8 kc + 7 of its 64 rows; the output layer after
// them with planes of 16 rows.
__device__ void tc_load_weights(const __half* W, unsigned char* sW) {
    for (int i = threadIdx.x; i < (kHidden * kWidth + kOutRows) * (kWidth / 8); i += blockDim.x) {
        const int kc = i % (kWidth / 8), row = i / (kWidth / 8);  // row over all layers' output rows
        const int l = row / kWidth, n = row % kWidth;
        const uint4 v = *reinterpret_cast<const uint4*>(W + size_t(row) * kWidth + kc * 8);
        const int off = l < kHidden ? l * kTcLayerB + kc * (kWidth * 16) + n * 16
                                    : kHidden * kTcLayerB + kc * (kOutRows * 16) + (row - kHidden * kWidth) * 16;
        *reinterpret_cast<uint4*>(sW + off) = v;
    }
}

__device__ __forceinline__ void tc_tmem_ld16(uint32_t taddr, uint32_t v[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr));
}

__global__ void __launch_bounds__(kTcThreads)
k_cache_infer_tc(CacheDev c, const float* q, uint32_t n_max, const uint32_t* n_dev, float* out, uint32_t* status) {
    extern __shared__ __align__(128) unsigned char tsm[];
    unsigned char* sW = tsm;
    unsigned char* sA = tsm + kTcWBytes;
    uint64_t* mbar = reinterpret_cast<uint64_t*>(sA + (kWidth / 8) * kTcPlaneA);
    uint32_t* slot = reinterpret_cast<uint32_t*>(mbar + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t n = n_dev ? min(*n_dev, n_max) : n_max;
    const uint32_t tiles = (n + kTcRows - 1) / kTcRows;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                     "r"(uint32_t(kWidth))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tc_load_weights(c.W, sW);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = *slot;
    const uint32_t a0 = smem_u32(sA), w0 = smem_u32(sW), mb = smem_u32(mbar);
    uint32_t phase = 0u;
    bool timed_out = false;
    bool pending = false;  // a commit not yet seen complete

    const int r = tid & (kTcRows - 1), half = tid >> 7;  // encoding: row, half of the levels
    const int quad = warp & 3, ch = warp >> 2;           // epilogue: TMEM lane quadrant, column half
    const int er = 32 * quad + lane;                     // epilogue row
    for (uint32_t tile = blockIdx.x; tile < tiles && !timed_out; tile += gridDim.x) {
        const uint32_t row = tile * kTcRows + uint32_t(r);
        // encode row r: levels 8 half .. 8 half + 7 (and the tail in half 0)
        float qq[9];
        for (int k = 0; k < 9; ++k) qq[k] = row < n ? q[size_t(row) * 9 + k] : 0.0f;
        {
            const float px = fminf(fmaxf(qq[0], 0.0f), 1.0f), py = fminf(fmaxf(qq[1], 0.0f), 1.0f),
                        pz = fminf(fmaxf(qq[2], 0.0f), 1.0f);
            // 8 levels = 16 features: element 2l of the row is in plane l / 4,
            // 4 (l mod 4) bytes into the row's 16
#pragma unroll 2
            for (int j = 0; j < 8; ++j) {
                const int l = 8 * half + j;
                uint32_t idx[8];
                float w[8];
                level_corners(c.spec, l, px, py, pz, idx, w);
                float f0 = 0.0f, f1 = 0.0f;
#pragma unroll
                for (int cc = 0; cc < 8; ++cc) {
                    const float2 v = __half22float2(c.grid[idx[cc]]);
                    f0 = fmaf(w[cc], v.x, f0);
                    f1 = fmaf(w[cc], v.y, f1);
                }
                *reinterpret_cast<uint32_t*>(sA + (l >> 2) * kTcPlaneA + r * 16 + (l & 3) * 4) = pack_half2(f0, f1);
            }
            if (half == 0) {  // normal and direction: elements 32..37 (plane 4), 38..39 zero
                *reinterpret_cast<uint4*>(sA + 4 * kTcPlaneA + r * 16) =
                    make_uint4(pack_half2(qq[3], qq[4]), pack_half2(qq[5], qq[6]), pack_half2(qq[7], qq[8]), 0u);
            } else {          // zero padding: planes 5..7
#pragma unroll
                for (int pl = 5; pl < 8; ++pl)
                    *reinterpret_cast<uint4*>(sA + pl * kTcPlaneA + r * 16) = make_uint4(0u, 0u, 0u, 0u);
            }
        }
        for (int L = 0; L <= kHidden; ++L) {
            const int nn = L < kHidden ? kWidth : kOutRows;
            // the tile's A operand is in shared memory: hand it to the tensor cores
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncthreads();
            if (tid == 0) {
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t wb = w0 + uint32_t(L * kTcLayerB);
                const uint32_t idesc = L < kHidden ? mlp_idesc(kTcRows, kWidth) : mlp_idesc(kTcRows, kOutRows);
#pragma unroll
                for (int k = 0; k < kWidth / 16; ++k) {
                    const uint64_t ad = tc_sdesc(a0 + uint32_t(2 * k * kTcPlaneA), kTcPlaneA, 128);
                    const uint64_t bd = tc_sdesc(wb + uint32_t(2 * k * nn * 16), uint32_t(nn * 16), 128);
                    asm volatile(
                        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(taddr),
                        "l"(ad), "l"(bd), "r"(idesc), "r"(uint32_t(k > 0))
                        : "memory");
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mb)
                             : "memory");
            }
            pending = true;
            const bool ok = tc_wait(mb, phase);
            if (ok) {
                phase ^= 1u;
                pending = false;
            }
            if (__syncthreads_or(!ok)) {
                timed_out = true;
                if (tid == 0) atomicOr(status, MRT_STATUS_PIPE_TIMEOUT);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            if (L < kHidden) {
                // warp w: rows 32 quad .., columns 32 ch .. 32 ch + 31 -> planes 4 ch .. 4 ch + 3
                uint32_t v[32];
                const uint32_t ta = taddr + (uint32_t(32 * quad) << 16) + uint32_t(32 * ch);
                tc_tmem_ld16(ta, v);
                tc_tmem_ld16(ta + 16u, v + 16);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int pl = 0; pl < 4; ++pl) {
                    uint32_t h[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e)
                        h[e] = pack_half2(fmaxf(__uint_as_float(v[8 * pl + 2 * e]), 0.0f),
                                          fmaxf(__uint_as_float(v[8 * pl + 2 * e + 1]), 0.0f));
                    *reinterpret_cast<uint4*>(sA + (4 * ch + pl) * kTcPlaneA + er * 16) =
                        make_uint4(h[0], h[1], h[2], h[3]);
                }
            } else if (ch == 0) {
                uint32_t v[16];
                tc_tmem_ld16(taddr + (uint32_t(32 * quad) << 16), v);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                const uint32_t orow = tile * kTcRows + uint32_t(er);
                if (orow < n)
                    for (int k = 0; k < 3; ++k) out[size_t(orow) * 3 + k] = __uint_as_float(v[k]);
            }
        }
    }
    // a commit still outstanding after a timeout: wait for it (bounded)
    // before the tensor memory is freed
    if (pending && !tc_wait(mb, phase)) atomicOr(status, MRT_STATUS_PIPE_TIMEOUT);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(uint32_t(kWidth))
                     : "memory");
}

// Training forward: stores the input rows and hidden activations, the
// output, and dL/dout of the relative L2 loss
//   L = mean_r sum_k (y_rk - t_rk)^2 / (sg(y_rk)^2 + 0.01)
// (sg = stop-gradient), plus the loss sum into loss_acc.
__global__ void __launch_bounds__(kMlpWarps * 32)
k_cache_train_fwd(CacheDev c, const float* q, const float* target, uint32_t n, __half* inputs, __half* acts,
                  float* dout, float* loss_acc) {
    extern __shared__ __align__(16) unsigned char smem[];
    __half* sW = reinterpret_cast<__half*>(smem);
    __half* sX = sW + kWeights;
    float* sO = reinterpret_cast<float*>(sX + kMlpWarps * 16 * kWidth);
    load_weights_smem(sW, c.W, kWeights);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = lane_id();
    __half* X = sX + warp * 16 * kWidth;
    float* O = sO + warp * 16 * 3;
    const size_t act_ld = size_t(n) * kWidth;  // layer stride in `acts`
    float loss = 0.0f;
    for (uint32_t base = (blockIdx.x * kMlpWarps + warp) * 16u; base + 16u <= n;
         base += gridDim.x * kMlpWarps * 16u) {
        encode_tile(c.spec, c.grid, X, [&](int rr, float* qq) {
            for (int k = 0; k < 9; ++k) qq[k] = q[size_t(base + uint32_t(rr)) * 9 + k];
        });
        __syncwarp();
        // the tile's input rows, kept for the backward (16 x 64 halves)
        for (int i = lane; i < 16 * kWidth / 2; i += 32)
            reinterpret_cast<uint32_t*>(inputs + size_t(base) * kWidth)[i] = reinterpret_cast<const uint32_t*>(X)[i];
        __syncwarp();
        mlp_forward_tile(sW, X, acts + size_t(base) * kWidth, act_ld, O);
        __syncwarp();
        if (lane < 16) {
            const uint32_t r = base + lane;
            for (int k = 0; k < 3; ++k) {
                const float y = O[lane * 3 + k], t = target[size_t(r) * 3 + k];
                const float den = y * y + 0.01f;
                loss += (y - t) * (y - t) / den;
                // scaled by kGradScale so the FP16 MMA operands of the
                // backward stay out of the subnormal range
                dout[size_t(r) * 3 + k] = 2.0f * (y - t) / den / float(n) * kGradScale;
            }
        }
        __syncwarp();
    }
    for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xFFFFFFFFu, loss, o);
    if (lane == 0) atomicAdd(loss_acc, loss);
}

// Training backward for 16-row tiles: activation gradients on the tensor
// cores (dh_{l-1} = dz_l * W_l with the stored transposes), ReLU masks from
// the stored activations, weight gradients dW_l = dz_l^T h_{l-1} summed in
// FP32 per warp and added to gW, and dL/d(input) written for the grid.
__global__ void __launch_bounds__(kMlpWarps * 32)
k_cache_train_bwd(CacheDev c, uint32_t n, const __half* inputs, const __half* acts, const float* dout, float* gW,
                  float* d_in) {
    extern __shared__ __align__(16) unsigned char smem[];
    __half* sWT = reinterpret_cast<__half*>(smem);                 // kWeights halves of transposes
    float* sD = reinterpret_cast<float*>(sWT + kWeights);           // kMlpWarps x 16 x 64 dz tile
    __half* sH = reinterpret_cast<__half*>(sD + kMlpWarps * 16 * kWidth);  // kMlpWarps x 16 x 64 h tile
    float* sG = reinterpret_cast<float*>(sH + kMlpWarps * 16 * kWidth);    // block gradient accumulator
    load_weights_smem(sWT, c.WT, kWeights);
    for (int i = threadIdx.x; i < kWeights; i += blockDim.x) sG[i] = 0.0f;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = lane_id(), g = lane >> 2, t = lane & 3;
    float* D = sD + warp * 16 * kWidth;
    __half* H = sH + warp * 16 * kWidth;
    const size_t act_ld = size_t(n) * kWidth;
    for (uint32_t base = (blockIdx.x * kMlpWarps + warp) * 16u; base + 16u <= n;
         base += gridDim.x * kMlpWarps * 16u) {
        // dz of the output layer: 16 x 16 (3 used)
        for (int i = lane; i < 16 * kWidth; i += 32) D[i] = 0.0f;
        __syncwarp();
        if (lane < 16)
            for (int k = 0; k < 3; ++k) D[lane * kWidth + k] = dout[size_t(base + lane) * 3 + k];
        __syncwarp();
        // layers from the output down: layer index L = kHidden (output) .. 0
#pragma unroll 1
        for (int L = kHidden; L >= 0; --L) {
            const int out_w = L == kHidden ? kOutRows : kWidth;
            // h_{L-1}: input of layer L (stored activation or the input row)
            const __half* hsrc = L == 0 ? inputs + size_t(base) * kWidth
                                        : acts + size_t(L - 1) * act_ld + size_t(base) * kWidth;
            for (int i = lane; i < 16 * kWidth / 2; i += 32)
                reinterpret_cast<uint32_t*>(H)[i] = reinterpret_cast<const uint32_t*>(hsrc)[i];
            __syncwarp();
            // weight gradient gW_L[o][i] += sum_r D[r][o] * H[r][i] on the
            // tensor cores: A = D^T (out_w x 16 rows), B = H (16 rows x 64)
            float* G = sG + L * kLayerW;
            for (int mt = 0; mt < out_w / 16; ++mt) {
                const int o0 = 16 * mt + g, o1 = o0 + 8;
                uint32_t a[4];
                a[0] = pack_half2(D[(2 * t) * kWidth + o0], D[(2 * t + 1) * kWidth + o0]);
                a[1] = pack_half2(D[(2 * t) * kWidth + o1], D[(2 * t + 1) * kWidth + o1]);
                a[2] = pack_half2(D[(2 * t + 8) * kWidth + o0], D[(2 * t + 9) * kWidth + o0]);
                a[3] = pack_half2(D[(2 * t + 8) * kWidth + o1], D[(2 * t + 9) * kWidth + o1]);
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const int nn = 8 * j + g;
                    const uint32_t b0 = uint32_t(__half_as_ushort(H[(2 * t) * kWidth + nn])) |
                                        (uint32_t(__half_as_ushort(H[(2 * t + 1) * kWidth + nn])) << 16);
                    const uint32_t b1 = uint32_t(__half_as_ushort(H[(2 * t + 8) * kWidth + nn])) |
                                        (uint32_t(__half_as_ushort(H[(2 * t + 9) * kWidth + nn])) << 16);
                    float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
                    mma16816(c, a, b0, b1);
                    const int i0 = 8 * j + 2 * t;
                    atomicAdd(&G[o0 * kWidth + i0], c[0]);
                    atomicAdd(&G[o0 * kWidth + i0 + 1], c[1]);
                    atomicAdd(&G[o1 * kWidth + i0], c[2]);
                    atomicAdd(&G[o1 * kWidth + i0 + 1], c[3]);
                }
            }
            // dh_{L-1} = D * W_L: A = D (16 x out_w as half), B from W_L^T [in][out]
            float acc[8][4];
            const __half* WT = sWT + L * kLayerW;  // [64 in][out_w]
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
            const int ktiles = out_w / 16;
            for (int k = 0; k < ktiles; ++k) {
                uint32_t a[4];
                const float* r0 = D + g * kWidth + 16 * k + 2 * t;
                const float* r1 = D + (g + 8) * kWidth + 16 * k + 2 * t;
                a[0] = pack_half2(r0[0], r0[1]);
                a[1] = pack_half2(r1[0], r1[1]);
                a[2] = pack_half2(r0[8], r0[9]);
                a[3] = pack_half2(r1[8], r1[9]);
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const __half* wr = WT + (8 * j + g) * out_w + 16 * k + 2 * t;
                    mma16816(acc[j], a, *reinterpret_cast<const uint32_t*>(wr),
                             *reinterpret_cast<const uint32_t*>(wr + 8));
                }
            }
            __syncwarp();
            // D <- dh_{L-1} masked by ReLU'(h_{L-1}) (layer input > 0), or d_in
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int col = 8 * j + 2 * t;
                const float v[4] = {acc[j][0], acc[j][1], acc[j][2], acc[j][3]};
                const int rows[2] = {g, g + 8};
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    for (int e = 0; e < 2; ++e) {
                        const int r = rows[h], cc = col + e;
                        float dv = v[2 * h + e];
                        if (L > 0 && !(__half2float(H[r * kWidth + cc]) > 0.0f)) dv = 0.0f;
                        D[r * kWidth + cc] = dv;
                    }
                }
            }
            __syncwarp();
        }
        // D holds dL/d(input row) x kGradScale; keep the 32 encoded features
        for (int i = lane; i < 16 * kEnc; i += 32) {
            const int r = i / kEnc, k = i % kEnc;
            d_in[size_t(base + r) * kEnc + k] = D[r * kWidth + k] * (1.0f / kGradScale);
        }
        __syncwarp();
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kWeights; i += blockDim.x)
        if (sG[i] != 0.0f) atomicAdd(&gW[i], sG[i] * (1.0f / kGradScale));
}

// Hash-grid gradient: scatter dL/d(features) to the 8 corners per level.
__global__ void k_grid_bwd(CacheDev c, const float* q, const float* d_in, uint32_t n, float* g_grid) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const float px = fminf(fmaxf(q[size_t(r) * 9 + 0], 0.0f), 1.0f);
    const float py = fminf(fmaxf(q[size_t(r) * 9 + 1], 0.0f), 1.0f);
    const float pz = fminf(fmaxf(q[size_t(r) * 9 + 2], 0.0f), 1.0f);
    for (int l = 0; l < kLevels; ++l) {
        const float d0 = d_in[size_t(r) * kEnc + 2 * l], d1 = d_in[size_t(r) * kEnc + 2 * l + 1];
        if (d0 == 0.0f && d1 == 0.0f) continue;
        uint32_t idx[8];
        float w[8];
        level_corners(c.spec, l, px, py, pz, idx, w);
        for (int k = 0; k < 8; ++k) {
            atomicAdd(&g_grid[2 * size_t(idx[k])], w[k] * d0);
            atomicAdd(&g_grid[2 * size_t(idx[k]) + 1], w[k] * d1);
        }
    }
}

// Adam on FP32 masters, writing the FP16 copies (and the transposed MLP
// layout when `wt` is set).  Gradients are cleared after use.
__global__ void k_adam(float* p, float* m, float* v, float* grad, __half* p16, __half* wt, uint32_t n, float lr,
                       float b1, float b2, float eps, float bc1, float bc2) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gr = grad[i];
    grad[i] = 0.0f;
    const float mi = b1 * m[i] + (1.0f - b1) * gr;
    const float vi = b2 * v[i] + (1.0f - b2) * gr * gr;
    m[i] = mi;
    v[i] = vi;
    const float pi = p[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    p[i] = pi;
    const __half h = __float2half_rn(pi);
    p16[i] = h;
    if (wt) {
        // hidden layers: [L][o][i] -> [L][i][o]; output rows: [o][i] -> [i][o] (64 x 16)
        const uint32_t L = i / kLayerW, e = i % kLayerW;
        if (L < uint32_t(kHidden)) {
            const uint32_t o = e / kWidth, in = e % kWidth;
            wt[L * kLayerW + in * kWidth + o] = h;
        } else {
            const uint32_t o = e / kWidth, in = e % kWidth;
            wt[L * kLayerW + in * kOutRows + o] = h;
        }
    }
}

// Adam on the grid features, four at a time, lazily: a group whose four
// gradients are all zero (no training sample touched those corners this
// step) keeps its parameters and moments, so a step reads the whole
// gradient array but only the touched part of the rest.
__global__ void k_adam_grid4(float4* p, float4* m, float4* v, float4* grad, __half2* p16, uint32_t n4, float lr,
                             float b1, float b2, float eps, float bc1, float bc2) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n4) return;
    const float4 g = grad[i];
    if (g.x == 0.0f && g.y == 0.0f && g.z == 0.0f && g.w == 0.0f) return;
    grad[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float4 mi = m[i], vi = v[i], pi = p[i];
    const float gs[4] = {g.x, g.y, g.z, g.w};
    float* ms = &mi.x;
    float* vs = &vi.x;
    float* ps = &pi.x;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        ms[k] = b1 * ms[k] + (1.0f - b1) * gs[k];
        vs[k] = b2 * vs[k] + (1.0f - b2) * gs[k] * gs[k];
        ps[k] = ps[k] - lr * (ms[k] / bc1) / (sqrtf(vs[k] / bc2) + eps);
    }
    m[i] = mi;
    v[i] = vi;
    p[i] = pi;
    p16[2 * i] = __floats2half2_rn(pi.x, pi.y);
    p16[2 * i + 1] = __floats2half2_rn(pi.z, pi.w);
}

} // namespace

// ============================================================ host object

struct mrt_cache {
    mrt_cache_config cfg{};
    CacheDev dev{};
    uint32_t grid_entries = 0;        // levels * 2^log2_t
    // MLP: fp32 master, adam state, grads, fp16 + transposed fp16
    float *w = nullptr, *wm = nullptr, *wv = nullptr, *wg = nullptr;
    __half *w16 = nullptr, *wt16 = nullptr;
    // grid
    float *gp = nullptr, *gm = nullptr, *gv = nullptr, *gg = nullptr;
    __half2* g16 = nullptr;
    // training buffers (capacity in samples)
    uint32_t cap = 0;
    float *tq = nullptr, *tt = nullptr, *tdout = nullptr, *tdin = nullptr, *loss = nullptr;
    __half *tin = nullptr, *tact = nullptr;
    uint32_t* tcount = nullptr;
    uint32_t step = 0;
    float last_loss = 0.0f;
    float* h_loss = nullptr;
    uint32_t* h_count = nullptr;
    uint32_t frame = 0;
    // per-frame sample buffer (training paths) and query buffers (render)
    uint32_t scap = 0;
    float *sq = nullptr, *st = nullptr;
    size_t qcap = 0;
    float *qq = nullptr, *qpred = nullptr;
    float4* qpb = nullptr;
    // inference on tcgen05 (k_cache_infer_tc, default) or mma.sync (k_cache_infer)
    bool tcgen05 = true;
    int sm_count = 0;
};

namespace {

int ensure_train(mrt_ctx* ctx, mrt_cache* c, uint32_t n) {
    if (c->cap >= n) return MRT_OK;
    cudaFree(c->tq); cudaFree(c->tt); cudaFree(c->tdout); cudaFree(c->tdin); cudaFree(c->tin); cudaFree(c->tact);
    c->cap = 0;
    bool ok = cudaMalloc(&c->tq, size_t(n) * 9 * 4) == cudaSuccess && cudaMalloc(&c->tt, size_t(n) * 3 * 4) == cudaSuccess &&
              cudaMalloc(&c->tdout, size_t(n) * 3 * 4) == cudaSuccess &&
              cudaMalloc(&c->tdin, size_t(n) * kEnc * 4) == cudaSuccess &&
              cudaMalloc(&c->tin, size_t(n) * kWidth * 2) == cudaSuccess &&
              cudaMalloc(&c->tact, size_t(n) * kWidth * 2 * kHidden) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        return set_error(ctx, MRT_ENOMEM, "radiance cache: training buffers");
    }
    c->cap = n;
    return MRT_OK;
}

size_t smem_infer() { return kWeights * 2 + kMlpWarps * 16 * kWidth * 2 + kMlpWarps * 16 * 3 * 4; }
size_t smem_bwd() { return kWeights * 2 + kMlpWarps * 16 * kWidth * 4 + kMlpWarps * 16 * kWidth * 2 + kWeights * 4; }

uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

} // namespace

namespace mrt {
uint32_t cache_query_vertex(const mrt_cache* c) { return c->cfg.query_vertex; }

// Inference over device rows of 9 floats; with n_dev the row count is read
// on the device (at most n).
cudaError_t cache_infer(const mrt_cache* c, const float* q, uint32_t n, const uint32_t* n_dev, float* out,
                        uint32_t* status, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    if (c->tcgen05) {  // persistent: up to 4 CTAs (51 KB of shared memory, 64 TMEM columns each) per SM
        const uint32_t tiles = (n + kTcRows - 1) / kTcRows;
        const uint32_t blocks = std::min<uint32_t>(tiles, uint32_t(c->sm_count) * 4u);
        k_cache_infer_tc<<<blocks, kTcThreads, kTcSmem, s>>>(c->dev, q, n, n_dev, out, status);
        return cudaGetLastError();
    }
    const uint32_t tiles = (n + 15u) / 16u;
    const uint32_t blocks = std::min<uint32_t>((tiles + kMlpWarps - 1) / kMlpWarps, 4096u);
    k_cache_infer<<<blocks, kMlpWarps * 32, smem_infer(), s>>>(c->dev, q, n, n_dev, out);
    return cudaGetLastError();
}

// Query buffers of the cache-terminated shade for `n` rays.
int cache_frame_buffers(mrt_ctx* ctx, mrt_cache* c, size_t n, float** q, float4** pb, float** pred) {
    if (c->qcap < n) {
        cudaFree(c->qq); cudaFree(c->qpred); cudaFree(c->qpb);
        c->qq = c->qpred = nullptr;
        c->qpb = nullptr;
        c->qcap = 0;
        if (cudaMalloc(&c->qq, n * 9 * 4) != cudaSuccess || cudaMalloc(&c->qpred, n * 3 * 4) != cudaSuccess ||
            cudaMalloc(&c->qpb, n * sizeof(float4)) != cudaSuccess) {
            cudaGetLastError();
            return set_error(ctx, MRT_ENOMEM, "radiance cache: query buffers");
        }
        c->qcap = n;
    }
    *q = c->qq;
    *pb = c->qpb;
    *pred = c->qpred;
    return MRT_OK;
}

// Trains the cache on this frame: cfg.train_paths fresh paths from the
// camera (plain estimator up to cfg.train_bounces), every vertex's suffix
// radiance a sample, then cfg.train_steps Adam steps on equal slices.
int cache_train_frame(mrt_ctx* ctx, mrt_cache* c, const DevScene& sc, const FrameParams& fp, const TraceParams& tp,
                      uint32_t* status, cudaStream_t s) {
    const uint32_t paths = c->cfg.train_paths ? c->cfg.train_paths : 65536u;
    const uint32_t cap = paths * 4u;
    if (c->scap < cap) {
        cudaFree(c->sq); cudaFree(c->st);
        c->sq = c->st = nullptr;
        c->scap = 0;
        if (cudaMalloc(&c->sq, size_t(cap) * 9 * 4) != cudaSuccess || cudaMalloc(&c->st, size_t(cap) * 3 * 4) != cudaSuccess) {
            cudaGetLastError();
            return set_error(ctx, MRT_ENOMEM, "radiance cache: sample buffers");
        }
        c->scap = cap;
    }
    if (!c->tcount) {
        if (cudaMalloc(&c->tcount, 4) != cudaSuccess || cudaMallocHost(&c->h_count, 4) != cudaSuccess)
            return set_error(ctx, MRT_ENOMEM, "radiance cache: counter");
    }
    if (cudaMemsetAsync(c->tcount, 0, 4, s) != cudaSuccess) return set_error(ctx, MRT_ECUDA, "cache: memset");
    if (launch_cache_train_paths(sc, fp, tp, c->cfg.train_bounces ? c->cfg.train_bounces : 8u, paths, c->frame++,
                                 c->sq, c->st, c->tcount, cap, status, s) != cudaSuccess)
        return set_error(ctx, MRT_ECUDA, "cache: training paths launch");
    ctx->launches++;
    if (cudaMemcpyAsync(c->h_count, c->tcount, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return set_error(ctx, MRT_ECUDA, "cache: sample count read-back");
    const uint32_t total = std::min(*c->h_count, cap);
    const uint32_t steps = c->cfg.train_steps ? c->cfg.train_steps : 4u;
    const uint32_t per = (total / steps) & ~15u;
    if (per < 16u) return MRT_OK;  // nothing hit this frame
    for (uint32_t k = 0; k < steps; ++k) {
        int rc = mrt_cuda_cache_train_step(ctx, c, c->sq + size_t(k) * per * 9, c->st + size_t(k) * per * 3, per, 1,
                                           nullptr, s);
        if (rc) return rc;
    }
    return MRT_OK;
}
} // namespace mrt

extern "C" {

int mrt_cuda_cache_create(mrt_ctx* ctx, const mrt_cache_config* cfg, mrt_cache** out) {
    if (!ctx || !cfg || !out) return set_error(ctx, MRT_EINVAL, "cache_create: null argument");
    if (cfg->log2_table < 10 || cfg->log2_table > 24 || !(cfg->base_res >= 2.0f) || !(cfg->max_res >= cfg->base_res))
        return set_error(ctx, MRT_EINVAL, "cache_create: bad grid configuration");
    if (cfg->query_vertex > 1u) return set_error(ctx, MRT_EINVAL, "cache_create: query_vertex must be 0 or 1");
    cudaSetDevice(ctx->device);
    mrt_cache* c = new (std::nothrow) mrt_cache;
    if (!c) return MRT_ENOMEM;
    c->cfg = *cfg;
    c->dev.spec.log2_t = cfg->log2_table;
    c->dev.spec.base_res = cfg->base_res;
    c->dev.spec.growth = std::exp((std::log(cfg->max_res) - std::log(cfg->base_res)) / float(kLevels - 1));
    c->grid_entries = uint32_t(kLevels) << cfg->log2_table;
    const size_t gn = size_t(c->grid_entries) * 2;  // floats
    bool ok = cudaMalloc(&c->w, kWeights * 4) == cudaSuccess && cudaMalloc(&c->wm, kWeights * 4) == cudaSuccess &&
              cudaMalloc(&c->wv, kWeights * 4) == cudaSuccess && cudaMalloc(&c->wg, kWeights * 4) == cudaSuccess &&
              cudaMalloc(&c->w16, kWeights * 2) == cudaSuccess && cudaMalloc(&c->wt16, kWeights * 2) == cudaSuccess &&
              cudaMalloc(&c->gp, gn * 4) == cudaSuccess && cudaMalloc(&c->gm, gn * 4) == cudaSuccess &&
              cudaMalloc(&c->gv, gn * 4) == cudaSuccess && cudaMalloc(&c->gg, gn * 4) == cudaSuccess &&
              cudaMalloc(&c->g16, gn * 2) == cudaSuccess && cudaMalloc(&c->loss, 4) == cudaSuccess &&
              cudaMallocHost(&c->h_loss, 4) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        mrt_cuda_cache_destroy(ctx, c);
        return set_error(ctx, MRT_ENOMEM, "cache_create: out of device memory");
    }
    // initialisation: MLP weights uniform(+-sqrt(6 / fan_in)) (He-uniform),
    // grid features uniform(+-1e-4), seeded
    std::vector<float> w(kWeights, 0.0f), g(gn);
    uint64_t s = 0x5EEDull + cfg->seed;
    for (int L = 0; L <= kHidden; ++L) {
        const int rows = L == kHidden ? kOutRows : kWidth;
        const int fan_in = L == 0 ? kEnc + 6 : kWidth;
        const float a = std::sqrt(6.0f / float(fan_in)) * (L == kHidden ? 0.5f : 1.0f);
        for (int o = 0; o < rows; ++o)
            for (int i = 0; i < kWidth; ++i) {
                const float u = float(splitmix(s) >> 11) * (1.0f / 9007199254740992.0f);
                const bool used = (L == kHidden ? o < 3 : true) && (L == 0 ? i < kEnc + 6 : true);
                w[size_t(L) * kLayerW + size_t(o) * kWidth + i] = used ? (2.0f * u - 1.0f) * a : 0.0f;
            }
    }
    for (auto& x : g) x = (float(splitmix(s) >> 11) * (1.0f / 9007199254740992.0f) * 2.0f - 1.0f) * 1e-4f;
    {
        std::vector<__half> w16(kWeights), wt16(kWeights);
        for (int i = 0; i < kWeights; ++i) w16[i] = __float2half_rn(w[i]);
        for (int L = 0; L <= kHidden; ++L) {
            const int rows = L == kHidden ? kOutRows : kWidth;
            for (int o = 0; o < rows; ++o)
                for (int i = 0; i < kWidth; ++i)
                    wt16[size_t(L) * kLayerW + size_t(i) * rows + o] = w16[size_t(L) * kLayerW + size_t(o) * kWidth + i];
        }
        std::vector<__half> g16(gn);
        for (size_t i = 0; i < gn; ++i) g16[i] = __float2half_rn(g[i]);
        ok = cudaMemcpy(c->w, w.data(), kWeights * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
             cudaMemcpy(c->w16, w16.data(), kWeights * 2, cudaMemcpyHostToDevice) == cudaSuccess &&
             cudaMemcpy(c->wt16, wt16.data(), kWeights * 2, cudaMemcpyHostToDevice) == cudaSuccess &&
             cudaMemcpy(c->gp, g.data(), gn * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
             cudaMemcpy(c->g16, g16.data(), gn * 2, cudaMemcpyHostToDevice) == cudaSuccess &&
             cudaMemset(c->wm, 0, kWeights * 4) == cudaSuccess && cudaMemset(c->wv, 0, kWeights * 4) == cudaSuccess &&
             cudaMemset(c->wg, 0, kWeights * 4) == cudaSuccess && cudaMemset(c->gm, 0, gn * 4) == cudaSuccess &&
             cudaMemset(c->gv, 0, gn * 4) == cudaSuccess && cudaMemset(c->gg, 0, gn * 4) == cudaSuccess;
    }
    if (!ok ||
        cudaFuncSetAttribute(k_cache_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem_infer())) != cudaSuccess ||
        cudaFuncSetAttribute(k_cache_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem) != cudaSuccess ||
        cudaFuncSetAttribute(k_cache_train_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem_infer())) != cudaSuccess ||
        cudaFuncSetAttribute(k_cache_train_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem_bwd())) != cudaSuccess) {
        cudaGetLastError();
        mrt_cuda_cache_destroy(ctx, c);
        return set_error(ctx, MRT_ECUDA, "cache_create: initialisation failed");
    }
    c->dev.grid = c->g16;
    c->dev.W = c->w16;
    c->dev.WT = c->wt16;
    c->sm_count = ctx->sm_count;
    *out = c;
    return MRT_OK;
}

int mrt_cuda_cache_set_tcgen05(mrt_cache* c, int enable) {
    if (!c) return MRT_EINVAL;
    c->tcgen05 = enable != 0;
    return MRT_OK;
}

int mrt_cuda_cache_destroy(mrt_ctx* ctx, mrt_cache* c) {
    if (!ctx || !c) return MRT_EINVAL;
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();
    void* ps[] = {c->w, c->wm, c->wv, c->wg, c->w16, c->wt16, c->gp, c->gm, c->gv, c->gg, c->g16, c->loss,
                  c->tq, c->tt, c->tdout, c->tdin, c->tin, c->tact, c->tcount, c->sq, c->st, c->qq, c->qpred, c->qpb};
    for (void* p : ps) cudaFree(p);
    if (c->h_loss) cudaFreeHost(c->h_loss);
    if (c->h_count) cudaFreeHost(c->h_count);
    delete c;
    return MRT_OK;
}

int mrt_cuda_cache_set_bounds(mrt_ctx* ctx, mrt_cache* c, const float lo[3], const float hi[3]) {
    if (!ctx || !c || !lo || !hi) return set_error(ctx, MRT_EINVAL, "cache_set_bounds: null argument");
    for (int a = 0; a < 3; ++a) {
        c->dev.lo[a] = lo[a];
        c->dev.inv_ext[a] = hi[a] > lo[a] ? 1.0f / (hi[a] - lo[a]) : 0.0f;
    }
    return MRT_OK;
}

int mrt_cuda_cache_infer(mrt_ctx* ctx, mrt_cache* c, const float* queries, uint32_t n, float* out, void* stream) {
    if (!ctx || !c || (n && (!queries || !out))) return set_error(ctx, MRT_EINVAL, "cache_infer: bad arguments");
    cudaSetDevice(ctx->device);
    if (cache_infer(c, queries, n, nullptr, out, ctx->d_status, static_cast<cudaStream_t>(stream)) != cudaSuccess)
        return set_error(ctx, MRT_ECUDA, "cache_infer: launch failed");
    ctx->launches++;
    return MRT_OK;
}

int mrt_cuda_cache_train_step(mrt_ctx* ctx, mrt_cache* c, const float* queries, const float* targets, uint32_t n,
                              int apply_update, float* loss_out, void* stream) {
    if (!ctx || !c || !queries || !targets) return set_error(ctx, MRT_EINVAL, "cache_train_step: bad arguments");
    n &= ~15u;  // whole 16-row tiles
    if (n == 0) return set_error(ctx, MRT_EINVAL, "cache_train_step: fewer than 16 samples");
    cudaSetDevice(ctx->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int rc = ensure_train(ctx, c, n);
    if (rc) return rc;
    const uint32_t tiles = n / 16u;
    const uint32_t blocks = std::min<uint32_t>((tiles + kMlpWarps - 1) / kMlpWarps, 2048u);
    if (cudaMemsetAsync(c->loss, 0, 4, s) != cudaSuccess) return set_error(ctx, MRT_ECUDA, "train: memset");
    k_cache_train_fwd<<<blocks, kMlpWarps * 32, smem_infer(), s>>>(c->dev, queries, targets, n, c->tin, c->tact,
                                                                   c->tdout, c->loss);
    k_cache_train_bwd<<<blocks, kMlpWarps * 32, smem_bwd(), s>>>(c->dev, n, c->tin, c->tact, c->tdout, c->wg,
                                                                 c->tdin);
    k_grid_bwd<<<(n + 127) / 128, 128, 0, s>>>(c->dev, queries, c->tdin, n, c->gg);
    ctx->launches += 3;
    if (apply_update) {
        c->step++;
        const float b1 = 0.9f, b2 = 0.99f, eps = 1e-10f;
        const float bc1 = 1.0f - std::pow(b1, float(c->step)), bc2 = 1.0f - std::pow(b2, float(c->step));
        k_adam<<<(kWeights + 255) / 256, 256, 0, s>>>(c->w, c->wm, c->wv, c->wg, c->w16, c->wt16, kWeights,
                                                      c->cfg.lr_mlp, b1, b2, eps, bc1, bc2);
        const uint32_t gn4 = c->grid_entries / 2u;  // 2 features per entry, 4 floats per group
        k_adam_grid4<<<(gn4 + 255) / 256, 256, 0, s>>>(
            reinterpret_cast<float4*>(c->gp), reinterpret_cast<float4*>(c->gm), reinterpret_cast<float4*>(c->gv),
            reinterpret_cast<float4*>(c->gg), c->g16, gn4, c->cfg.lr_grid, b1, b2, eps, bc1, bc2);
        ctx->launches += 2;
    }
    if (cudaGetLastError() != cudaSuccess) return set_error(ctx, MRT_ECUDA, "train: launch failed");
    if (loss_out) {
        if (cudaMemcpyAsync(c->h_loss, c->loss, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return set_error(ctx, MRT_ECUDA, "train: loss read-back");
        *loss_out = *c->h_loss / float(n);
    }
    return MRT_OK;
}

// Parameter access for checks: which = 0 MLP weights (fp32 master,
// kWeights), 1 MLP weight gradients, 2 grid params (fp32 master), 3 grid
// gradients.  get copies device -> host; set copies host -> device (and
// refreshes the fp16 copies for 0 and 2).
int mrt_cuda_cache_params(mrt_ctx* ctx, mrt_cache* c, int which, float* host, size_t count, int set) {
    if (!ctx || !c || !host || which < 0 || which > 3) return set_error(ctx, MRT_EINVAL, "cache_params: bad arguments");
    cudaSetDevice(ctx->device);
    const size_t gn = size_t(c->grid_entries) * 2;
    float* dptr = which == 0 ? c->w : which == 1 ? c->wg : which == 2 ? c->gp : c->gg;
    const size_t total = which < 2 ? size_t(kWeights) : gn;
    if (count != total) return set_error(ctx, MRT_EINVAL, "cache_params: count mismatch");
    cudaDeviceSynchronize();
    if (!set) {
        if (cudaMemcpy(host, dptr, total * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
            return set_error(ctx, MRT_ECUDA, "cache_params: copy");
        return MRT_OK;
    }
    if (cudaMemcpy(dptr, host, total * 4, cudaMemcpyHostToDevice) != cudaSuccess)
        return set_error(ctx, MRT_ECUDA, "cache_params: copy");
    if (which == 0) {
        std::vector<__half> w16(kWeights), wt16(kWeights);
        for (int i = 0; i < kWeights; ++i) w16[i] = __float2half_rn(host[i]);
        for (int L = 0; L <= kHidden; ++L) {
            const int rows = L == kHidden ? kOutRows : kWidth;
            for (int o = 0; o < rows; ++o)
                for (int i = 0; i < kWidth; ++i)
                    wt16[size_t(L) * kLayerW + size_t(i) * rows + o] = w16[size_t(L) * kLayerW + size_t(o) * kWidth + i];
        }
        cudaMemcpy(c->w16, w16.data(), kWeights * 2, cudaMemcpyHostToDevice);
        cudaMemcpy(c->wt16, wt16.data(), kWeights * 2, cudaMemcpyHostToDevice);
    } else if (which == 2) {
        std::vector<__half> g16(gn);
        for (size_t i = 0; i < gn; ++i) g16[i] = __float2half_rn(host[i]);
        cudaMemcpy(c->g16, g16.data(), gn * 2, cudaMemcpyHostToDevice);
    }
    return MRT_OK;
}

} // extern "C"
