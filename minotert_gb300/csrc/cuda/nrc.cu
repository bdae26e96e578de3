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
// weights and activations, FP32 accumulation.  By default inference, the
// training forward and the backward run on the 5th-generation tensor cores
// (tcgen05: 128-row tiles, accumulators and the weight-gradient sums in
// tensor memory; k_cache_fwd_tc, k_cache_bwd_tc).  The earlier mma.sync
// kernels stay selectable for comparison: there a warp owns 16 rows, and
// the FP32 accumulator tiles of one layer (16 x 64) are, element for
// element, the A fragments of the next layer's product after packing to
// half2.  The grid's gradients are FP32 atomics; Adam keeps FP32 master
// weights.
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
    const __half* Wimg;   // the weights in the tcgen05 kernels' shared-memory layout (wimg_off)
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
    if (blockIdx.x * kMlpWarps * 16u >= n) return;  // no rows for this block
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

// Byte offset of weight (layer L, output row o, input i) in the K-plane
// layout the tcgen05 kernels keep in shared memory: hidden layer L at
// L * 8 KB, plane i / 8 of it holding inputs 8 (i / 8) .. + 7 of its 64 rows
// (16 bytes a row); the output layer after them with planes of 16 rows.
// Adam writes this image beside the FP16 weights, so a CTA fetches it with
// one bulk copy.
__host__ __device__ constexpr uint32_t wimg_off(int L, int o, int i) {
    return L < kHidden ? uint32_t(L * kTcLayerB + (i / 8) * (kWidth * 16) + o * 16 + (i % 8) * 2)
                       : uint32_t(kHidden * kTcLayerB + (i / 8) * (kOutRows * 16) + o * 16 + (i % 8) * 2);
}

__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t mb) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(mb)
                 : "memory");
}

__device__ __forceinline__ void tc_tmem_ld16(uint32_t taddr, uint32_t v[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr));
}

// Training outputs of the tcgen05 forward: per 128-row tile, the five
// 16 KB shared-memory images of the layers' A operands (the encoded input
// rows, then the hidden activations after ReLU, in the K-plane layout
// above) and the 4 KB image of dL/dy (16 FP16 columns, 3 used, scaled by
// kGradScale), which are what the tcgen05 backward reads; plus the loss.
constexpr int kImg = kTcRows * kWidth * 2;       // 16 KB: one tile's 64 FP16 columns
constexpr int kDyImg = kTcRows * kOutRows * 2;   // 4 KB: one tile's dL/dy
constexpr int kImgs = kHidden + 1;               // images per tile: input rows, 4 hidden layers
struct TrainTc {
    const float* target;  // rows x 3
    uint4* img;           // tiles x kImgs x kImg bytes
    uint4* dy;            // tiles x kDyImg bytes
    float* loss_acc;
};

// Rows of a training step: the whole buffer (slice == null: rows
// [0, n_max)) or the device-side slice {first row, count} that a frame's
// training step takes from the samples its paths produced.
struct Rows {
    uint32_t off, n;
};
__device__ __forceinline__ Rows rows_of(const uint32_t* slice, uint32_t n_max) {
    return slice ? Rows{slice[0], min(slice[1], n_max)} : Rows{0u, n_max};
}

// Inference (kTrain = false: n_dev, when set, holds the query count) and
// the training forward (kTrain = true: n_dev, when set, is a training
// slice {first row, count}; the tile images and dL/dy are written instead
// of the outputs).
template <bool kTrain>
__global__ void __launch_bounds__(kTcThreads)
k_cache_fwd_tc(CacheDev c, const float* q, uint32_t n_max, const uint32_t* n_dev, float* out, uint32_t* status,
               TrainTc tr) {
    extern __shared__ __align__(128) unsigned char tsm[];
    unsigned char* sW = tsm;
    unsigned char* sA = tsm + kTcWBytes;
    uint64_t* mbar = reinterpret_cast<uint64_t*>(sA + (kWidth / 8) * kTcPlaneA);
    uint32_t* slot = reinterpret_cast<uint32_t*>(mbar + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    uint32_t n;
    if (kTrain) {
        const Rows rs = rows_of(n_dev, n_max);
        n = rs.n;
        q += size_t(rs.off) * 9;
        tr.target += size_t(rs.off) * 3;
    } else {
        n = n_dev ? min(*n_dev, n_max) : n_max;
    }
    const uint32_t tiles = (n + kTcRows - 1) / kTcRows;
    // grids are sized by the capacity; with a device-side count the CTAs
    // past the last tile leave before loading weights or taking tensor
    // memory (uniform over the CTA)
    if (blockIdx.x >= tiles) return;
    const float dy_scale = kTrain ? kGradScale / float(max(n, 1u)) : 0.0f;
    float loss = 0.0f;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                     "r"(uint32_t(kWidth))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    uint64_t* wbar = mbar + 2;  // the weights' bulk copy
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar)) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(wbar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        // the weights come in while the first tile is encoded
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(wbar)),
                     "r"(uint32_t(kTcWBytes))
                     : "memory");
        bulk_load(smem_u32(sW), c.Wimg, kTcWBytes, smem_u32(wbar));
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = *slot;
    const uint32_t a0 = smem_u32(sA), w0 = smem_u32(sW), mb = smem_u32(mbar);
    uint32_t phase = 0u;
    bool timed_out = false;
    bool pending = false;   // a commit not yet seen complete
    bool w_wait = true;     // the weights' copy not yet seen complete

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
            if (w_wait) {  // first product of the launch: the weights must have landed
                const bool wok = tid != 0 || tc_wait(smem_u32(wbar), 0u);
                if (__syncthreads_or(!wok)) {
                    timed_out = true;
                    if (tid == 0) atomicOr(status, MRT_STATUS_PIPE_TIMEOUT);
                    break;
                }
                w_wait = false;
            } else {
                __syncthreads();
            }
            if (kTrain) {  // the operand image goes out for the backward (read while the MMAs read it too)
                uint4* dst = tr.img + (size_t(tile) * kImgs + size_t(L)) * (kImg / 16);
                const uint4* src = reinterpret_cast<const uint4*>(sA);
#pragma unroll
                for (int i = 0; i < kImg / 16 / kTcThreads; ++i) dst[tid + i * kTcThreads] = src[tid + i * kTcThreads];
            }
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
                if (!kTrain) {
                    if (orow < n)
                        for (int k = 0; k < 3; ++k) out[size_t(orow) * 3 + k] = __uint_as_float(v[k]);
                } else {
                    // relative L2 loss L = mean_r sum_k (y - t)^2 / (sg(y)^2 + 0.01) and
                    // dL/dy (scaled by kGradScale so the FP16 operands of the
                    // backward stay out of the subnormal range); zero past n
                    float dy[3] = {0.0f, 0.0f, 0.0f};
                    if (orow < n) {
                        for (int k = 0; k < 3; ++k) {
                            const float y = __uint_as_float(v[k]), t = tr.target[size_t(orow) * 3 + k];
                            const float den = y * y + 0.01f;
                            loss += (y - t) * (y - t) / den;
                            dy[k] = 2.0f * (y - t) / den * dy_scale;
                        }
                    }
                    uint4* d = tr.dy + size_t(tile) * (kDyImg / 16);
                    d[er] = make_uint4(pack_half2(dy[0], dy[1]), pack_half2(dy[2], 0.0f), 0u, 0u);
                    d[kTcRows + er] = make_uint4(0u, 0u, 0u, 0u);
                }
            }
        }
    }
    if (kTrain) {
        for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xFFFFFFFFu, loss, o);
        if (lane == 0 && loss != 0.0f) atomicAdd(tr.loss_acc, loss);
    }
    // a commit or the weights' copy still outstanding after a timeout: wait
    // for it (bounded) before the tensor memory and shared memory are freed
    if (pending && !tc_wait(mb, phase)) atomicOr(status, MRT_STATUS_PIPE_TIMEOUT);
    if (w_wait && tid == 0 && !tc_wait(smem_u32(wbar), 0u)) atomicOr(status, MRT_STATUS_PIPE_TIMEOUT);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(uint32_t(kWidth))
                     : "memory");
}

// Training state of one hash-grid entry, one 32-byte sector: FP32 master
// features, Adam moments and the gradient, so that the grid's Adam step
// reads and writes one sector per entry it updates (the FP16 features the
// encodings gather stay in their own compact table).
struct __align__(32) GridEntry {
    float2 p, m, v, g;
};
static_assert(sizeof(GridEntry) == 32, "one sector per grid entry");

// Adds (a0, a1) to grid entry e's gradient and marks the entry in the
// touched bitmap (bit e) for the grid's Adam step (k_adam_grid).
__device__ __forceinline__ void grid_grad_add(GridEntry* gs, uint32_t* touched, uint32_t e, float a0, float a1) {
    if (a0 == 0.0f && a1 == 0.0f) return;
    atomicAdd(&gs[e].g, make_float2(a0, a1));
    atomicOr(touched + (e >> 5), 1u << (e & 31u));
}

// ------------------------------------------- training backward on tcgen05
//
// One CTA of 256 threads (one per SM) per run of 128-row tiles.  A tile
// takes five phases from the output layer down; phase p works on the layer
// whose output gradient dZ (FP16, scaled by kGradScale) sits in shared
// memory as a K-plane image:
//   dW += dZ^T H  M = 128 over the layer's outputs, N = 64 inputs, K = the
//                 tile's 128 rows: 8 MMAs, both operands MN-major (the
//                 K-plane images read along their rows);
//   dH  = dZ W    M = 128 rows, N = 64, K = the layer's outputs: 4 MMAs (1
//                 for the output layer), W read MN-major from the layout
//                 the forward reads K-major;
// then the epilogue writes the next dZ = dH where the layer's input H > 0
// (ReLU), or, below the first layer, scatters dL/d(encoded features) into
// the hash grid's gradients.  The five layer inputs H (the forward's
// images) and dL/dy come by bulk copies when the tile starts — the next
// tile's as soon as this tile's last MMAs are done — so the phases run back
// to back, the epilogue reading its ReLU mask from the same images.  The
// weight gradients of all the CTA's tiles accumulate in tensor memory and
// are added to the FP32 gradients once.  Tensor memory, 256 columns:
// [0, 64) dH; [64, 128) dW of hidden layer 3 (lanes 0-63) and 2 (lanes
// 64-127); [128, 192) dW of layers 1 and 0; [192, 256) dW of the output
// layer (lanes 0-15).  Two layers share columns by lanes: the 128 A rows of
// the dW product are [dZ ; zeros] for the lower layer and [zeros ; dZ] for
// the upper one, so each adds exactly zero to the other's lanes.  Shared
// memory holds dZ1 | 16 KB of zeros | dZ2, and the phases alternate
// between dZ1 (lower) and dZ2 (upper).
constexpr int kBwThreads = 256;
constexpr uint32_t kBwCols = 256;
constexpr int kBwDy = 0;                      // dL/dy image; the weights follow it
constexpr int kBwW = kBwDy + kDyImg;
constexpr int kBwD1 = kBwW + kTcWBytes;       // dZ of phases 1 and 3 (lower lanes)
constexpr int kBwZ = kBwD1 + kImg;            // zeros
constexpr int kBwD2 = kBwZ + kImg;            // dZ of phases 2 and 4 (upper lanes)
constexpr int kBwH = kBwD2 + kImg;            // the layer inputs: image i = input of layer i
constexpr int kBwBar = kBwH + kImgs * kImg;
constexpr int kBwSmem = kBwBar + 64;
// The output layer's dW product reads 128 A rows of which the first 16 are
// dL/dy: the other 14 row groups (2 KB apart) fall on the weights.
static_assert(kBwDy + 16 * kTcPlaneA <= kBwD1, "the output layer's dW rows stay inside the weights");
static_assert(kBwSmem <= 227 * 1024, "one CTA per SM");

// dL/dy and the five layer-input images of `tile` (and, once, the weights)
// onto mbarrier mb
__device__ __forceinline__ void bw_load(uint32_t s0, uint32_t mb, const uint4* img, const uint4* dyimg, uint32_t tile,
                                        const __half* wimg) {
    const uint32_t bytes = uint32_t(kImgs * kImg + kDyImg) + (wimg ? uint32_t(kTcWBytes) : 0u);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(bytes) : "memory");
    if (wimg) bulk_load(s0 + uint32_t(kBwW), wimg, kTcWBytes, mb);
    bulk_load(s0 + uint32_t(kBwDy), dyimg + size_t(tile) * (kDyImg / 16), kDyImg, mb);
    bulk_load(s0 + uint32_t(kBwH), img + size_t(tile) * kImgs * (kImg / 16), kImgs * kImg, mb);
}

__device__ __forceinline__ void bw_mma(uint32_t d, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
        "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
        : "memory");
}

__global__ void __launch_bounds__(kBwThreads)
k_cache_bwd_tc(CacheDev c, const float* q, uint32_t n_max, const uint32_t* slice, const uint4* img,
               const uint4* dyimg, float* gW, GridEntry* gs, uint32_t* touched, uint32_t* status) {
    extern __shared__ __align__(128) unsigned char bsm[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(bsm + kBwBar);  // [0] bulk loads, [1] MMAs
    uint32_t* slot = reinterpret_cast<uint32_t*>(bar + 2);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const Rows rs = rows_of(slice, n_max);
    const uint32_t n = rs.n;
    q += size_t(rs.off) * 9;
    const uint32_t tiles = (n + kTcRows - 1) / kTcRows;
    if (blockIdx.x >= tiles) return;  // uniform over the CTA, before any allocation

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                     "r"(kBwCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    const uint32_t s0 = smem_u32(bsm), mb_ld = smem_u32(bar), mb_mma = smem_u32(bar + 1);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb_ld) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb_mma) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        bw_load(s0, mb_ld, img, dyimg, blockIdx.x, c.Wimg);  // the weights come with the first tile
    }
    for (int i = tid; i < kImg / 16; i += kBwThreads) reinterpret_cast<uint4*>(bsm + kBwZ)[i] = make_uint4(0, 0, 0, 0);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = *slot;
    uint32_t ld_phase = 0u, mma_phase = 0u;
    bool ld_pending = true, mma_pending = false, failed = false, first = true;
    const int quad = warp & 3, ch = warp >> 2, er = 32 * quad + lane;
    constexpr uint32_t idesc_w = mlp_idesc(kTcRows, kWidth) | (1u << 15) | (1u << 16);  // A, B MN-major
    constexpr uint32_t idesc_x = mlp_idesc(kTcRows, kWidth) | (1u << 16);               // B MN-major
    for (uint32_t tile = blockIdx.x; tile < tiles && !failed; tile += gridDim.x) {
        const uint32_t row = tile * kTcRows + uint32_t(er);
        const bool valid = row < n;
        float px = 0.0f, py = 0.0f, pz = 0.0f;
        if (valid) {
            px = fminf(fmaxf(q[size_t(row) * 9 + 0], 0.0f), 1.0f);
            py = fminf(fmaxf(q[size_t(row) * 9 + 1], 0.0f), 1.0f);
            pz = fminf(fmaxf(q[size_t(row) * 9 + 2], 0.0f), 1.0f);
        }
        // the tile's images (every thread waits: they read the masks)
        {
            const bool ok = tc_wait(mb_ld, ld_phase);
            if (__syncthreads_or(!ok)) {
                failed = true;
                break;
            }
            ld_phase ^= 1u;
            ld_pending = false;
        }
        for (int p = 0; p <= kHidden; ++p) {
            const uint32_t h = s0 + uint32_t(kBwH + (kHidden - p) * kImg);  // this phase's layer input
            if (tid == 0) {
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                // phase p's dZ: dL/dy, then dZ1 / dZ2 alternately
                const bool upper = p == 2 || p == 4;
                const uint32_t dz = p == 0 ? s0 + kBwDy : (p & 1) ? s0 + kBwD1 : s0 + kBwD2;
                const uint32_t a_dw = upper ? s0 + kBwZ : dz;
                const uint32_t col = p == 0 ? 192u : p <= 2 ? 64u : 128u;
                const bool clears = first && !upper;  // the column range's first product this launch
#pragma unroll
                for (int k = 0; k < kTcRows / 16; ++k)
                    bw_mma(taddr + col, tc_sdesc(a_dw + 256u * k, 128, kTcPlaneA), tc_sdesc(h + 256u * k, 128, kTcPlaneA),
                           idesc_w, uint32_t(k > 0 || !clears));
                if (p == 0) {
                    bw_mma(taddr, tc_sdesc(dz, kTcPlaneA, 128),
                           tc_sdesc(s0 + kBwW + kHidden * kTcLayerB, 128, kOutRows * 16), idesc_x, 0u);
                } else {
                    const uint32_t wl = s0 + kBwW + uint32_t(kHidden - p) * kTcLayerB;
#pragma unroll
                    for (int k = 0; k < kWidth / 16; ++k)
                        bw_mma(taddr, tc_sdesc(dz + 2u * k * kTcPlaneA, kTcPlaneA, 128),
                               tc_sdesc(wl + 256u * k, 128, kWidth * 16), idesc_x, uint32_t(k > 0));
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 mb_mma)
                             : "memory");
            }
            // this thread's ReLU mask while the MMAs run: row er, columns
            // 32 ch .. 32 ch + 31 of the layer input
            uint4 hm[4];
            if (p < kHidden) {
#pragma unroll
                for (int pl = 0; pl < 4; ++pl)
                    hm[pl] = *reinterpret_cast<const uint4*>(bsm + kBwH + (kHidden - p) * kImg + (4 * ch + pl) * kTcPlaneA +
                                                             er * 16);
            }
            mma_pending = true;
            const bool ok2 = tc_wait(mb_mma, mma_phase);
            if (ok2) {
                mma_phase ^= 1u;
                mma_pending = false;
            }
            if (__syncthreads_or(!ok2)) {
                failed = true;
                break;
            }
            // after the last phase's MMAs every buffer is free: the next tile's images come in
            if (p == kHidden && tid == 0 && tile + gridDim.x < tiles) {
                bw_load(s0, mb_ld, img, dyimg, tile + gridDim.x, nullptr);
                ld_pending = true;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            if (p < kHidden) {
                uint32_t v[32];
                const uint32_t ta = taddr + (uint32_t(32 * quad) << 16) + uint32_t(32 * ch);
                tc_tmem_ld16(ta, v);
                tc_tmem_ld16(ta + 16u, v + 16);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                unsigned char* dst = bsm + ((p & 1) ? kBwD2 : kBwD1);
#pragma unroll
                for (int pl = 0; pl < 4; ++pl) {
                    const uint32_t hw[4] = {hm[pl].x, hm[pl].y, hm[pl].z, hm[pl].w};
                    uint32_t hh[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const float h0 = __half2float(__ushort_as_half(uint16_t(hw[e] & 0xFFFFu))),
                                    h1 = __half2float(__ushort_as_half(uint16_t(hw[e] >> 16)));
                        hh[e] = pack_half2(h0 > 0.0f ? __uint_as_float(v[8 * pl + 2 * e]) : 0.0f,
                                           h1 > 0.0f ? __uint_as_float(v[8 * pl + 2 * e + 1]) : 0.0f);
                    }
                    *reinterpret_cast<uint4*>(dst + (4 * ch + pl) * kTcPlaneA + er * 16) =
                        make_uint4(hh[0], hh[1], hh[2], hh[3]);
                }
            } else {
                // dL/d(encoded features) of row er: columns 16 ch .. 16 ch + 15,
                // i.e. levels 8 ch .. 8 ch + 7, to the 8 corners of each
                uint32_t v[16];
                tc_tmem_ld16(taddr + (uint32_t(32 * quad) << 16) + uint32_t(16 * ch), v);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if (valid) {
#pragma unroll
                    for (int j = 0; j < kLevels / 2; ++j) {
                        const float d0 = __uint_as_float(v[2 * j]) * (1.0f / kGradScale),
                                    d1 = __uint_as_float(v[2 * j + 1]) * (1.0f / kGradScale);
                        if (d0 == 0.0f && d1 == 0.0f) continue;
                        uint32_t idx[8];
                        float w[8];
                        level_corners(c.spec, 8 * ch + j, px, py, pz, idx, w);
#pragma unroll
                        for (int k = 0; k < 8; ++k) grid_grad_add(gs, touched, idx[k], w[k] * d0, w[k] * d1);
                    }
                }
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncthreads();
        }
        first = false;
    }
    // anything still in flight after a timeout: bounded waits before the
    // buffers and the tensor memory are released
    if (ld_pending && !tc_wait(mb_ld, ld_phase) && tid == 0) atomicOr(status, MRT_STATUS_PIPE_TIMEOUT);
    if (mma_pending && !tc_wait(mb_mma, mma_phase) && tid == 0) atomicOr(status, MRT_STATUS_PIPE_TIMEOUT);
    if (failed) {
        if (tid == 0) atomicOr(status, MRT_STATUS_PIPE_TIMEOUT);
    } else {
        // the CTA's weight gradients (unscaled) into the FP32 sums
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const float inv = 1.0f / kGradScale;
#pragma unroll 1
        for (int R = 0; R < 2; ++R) {
            uint32_t v[32];
            const uint32_t ta = taddr + (uint32_t(32 * quad) << 16) + uint32_t(64 + 64 * R + 32 * ch);
            tc_tmem_ld16(ta, v);
            tc_tmem_ld16(ta + 16u, v + 16);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            const int layer = R == 0 ? (quad < 2 ? 3 : 2) : (quad < 2 ? 1 : 0);
            float4* g = reinterpret_cast<float4*>(gW + layer * kLayerW + (er & 63) * kWidth + 32 * ch);
#pragma unroll
            for (int j = 0; j < 8; ++j)
                atomicAdd(g + j, make_float4(__uint_as_float(v[4 * j]) * inv, __uint_as_float(v[4 * j + 1]) * inv,
                                             __uint_as_float(v[4 * j + 2]) * inv,
                                             __uint_as_float(v[4 * j + 3]) * inv));
        }
        if (quad == 0) {  // output layer: rows 0-2 (the padding rows' gradients are zero)
            uint32_t v[32];
            const uint32_t ta = taddr + uint32_t(192 + 32 * ch);
            tc_tmem_ld16(ta, v);
            tc_tmem_ld16(ta + 16u, v + 16);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (lane < 3) {
                float4* g = reinterpret_cast<float4*>(gW + kHidden * kLayerW + lane * kWidth + 32 * ch);
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    atomicAdd(g + j, make_float4(__uint_as_float(v[4 * j]) * inv, __uint_as_float(v[4 * j + 1]) * inv,
                                                 __uint_as_float(v[4 * j + 2]) * inv,
                                                 __uint_as_float(v[4 * j + 3]) * inv));
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(kBwCols) : "memory");
}

// Training forward: stores the input rows and hidden activations, the
// output, and dL/dout of the relative L2 loss
//   L = mean_r sum_k (y_rk - t_rk)^2 / (sg(y_rk)^2 + 0.01)
// (sg = stop-gradient), plus the loss sum into loss_acc.
__global__ void __launch_bounds__(kMlpWarps * 32)
k_cache_train_fwd(CacheDev c, const float* q, const float* target, uint32_t n_max, const uint32_t* slice,
                  __half* inputs, __half* acts, float* dout, float* loss_acc) {
    extern __shared__ __align__(16) unsigned char smem[];
    const Rows rs = rows_of(slice, n_max);
    const uint32_t n = rs.n;
    q += size_t(rs.off) * 9;
    target += size_t(rs.off) * 3;
    if (blockIdx.x * kMlpWarps * 16u + 16u > n) return;  // no whole tile for this block
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
k_cache_train_bwd(CacheDev c, uint32_t n_max, const uint32_t* slice, const __half* inputs, const __half* acts,
                  const float* dout, float* gW, float* d_in) {
    extern __shared__ __align__(16) unsigned char smem[];
    const uint32_t n = rows_of(slice, n_max).n;
    if (blockIdx.x * kMlpWarps * 16u + 16u > n) return;  // no whole tile for this block
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

// Hash-grid gradient: scatter dL/d(features) to the 8 corners per level
// (flagging the entries for the grid's Adam step).
__global__ void k_grid_bwd(CacheDev c, const float* q, const float* d_in, uint32_t n_max, const uint32_t* slice,
                           GridEntry* gs, uint32_t* touched) {
    const Rows rs = rows_of(slice, n_max);
    q += size_t(rs.off) * 9;
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rs.n) return;
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
            grid_grad_add(gs, touched, idx[k], w[k] * d0, w[k] * d1);
        }
    }
}

// Adam on FP32 masters, writing the FP16 copies (and the transposed MLP
// layout when `wt` is set, the tcgen05 image when `wimg` is).  Gradients are cleared after use.  A training
// slice that came out empty (a frame whose paths left fewer than 16
// samples per step) updates nothing.
__global__ void k_adam(float* p, float* m, float* v, float* grad, __half* p16, __half* wt, __half* wimg, uint32_t n,
                       float lr, float b1, float b2, float eps, float bc1, float bc2, const uint32_t* slice) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || (slice && slice[1] == 0u)) return;
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
    if (wimg) wimg[wimg_off(int(i / kLayerW), int((i % kLayerW) / kWidth), int(i % kWidth)) / 2] = h;
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

// Adam on the grid features, lazily and per entry (its 2 features): the
// gradient scatter marks every entry it adds a nonzero amount to in a
// bitmap, and only marked entries whose gradient is nonzero are updated;
// the rest keep their parameters and moments.  A warp takes a bitmap word
// (32 consecutive entries, 1 KB of training state): each lane whose bit is
// set reads its entry's sector, updates it with the gradient cleared, and
// writes its FP16 features; the word is cleared.  kAdamWords words in
// flight per warp.
constexpr int kAdamWords = 4;

__global__ void k_adam_grid(GridEntry* gs, __half2* p16, uint32_t* touched, uint32_t nwords, float lr, float b1,
                            float b2, float eps, float bc1, float bc2) {
    const uint32_t lane = lane_id();
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t w0 = warp; w0 < nwords; w0 += warps * kAdamWords) {
        uint32_t word[kAdamWords];
#pragma unroll
        for (int j = 0; j < kAdamWords; ++j) {
            const uint32_t w = w0 + uint32_t(j) * warps;
            const uint32_t x = (lane == 0u && w < nwords) ? touched[w] : 0u;
            word[j] = __shfl_sync(0xFFFFFFFFu, x, 0);
        }
        GridEntry en[kAdamWords];
#pragma unroll
        for (int j = 0; j < kAdamWords; ++j)
            if ((word[j] >> lane) & 1u) en[j] = gs[32u * (w0 + uint32_t(j) * warps) + lane];
#pragma unroll
        for (int j = 0; j < kAdamWords; ++j) {
            if (lane == 0u && word[j] != 0u) touched[w0 + uint32_t(j) * warps] = 0u;
            if (!((word[j] >> lane) & 1u)) continue;
            GridEntry x = en[j];
            const float2 g = x.g;
            if (g.x == 0.0f && g.y == 0.0f) continue;
            x.m.x = b1 * x.m.x + (1.0f - b1) * g.x;
            x.m.y = b1 * x.m.y + (1.0f - b1) * g.y;
            x.v.x = b2 * x.v.x + (1.0f - b2) * g.x * g.x;
            x.v.y = b2 * x.v.y + (1.0f - b2) * g.y * g.y;
            x.p.x = x.p.x - lr * (x.m.x / bc1) / (sqrtf(x.v.x / bc2) + eps);
            x.p.y = x.p.y - lr * (x.m.y / bc1) / (sqrtf(x.v.y / bc2) + eps);
            x.g = make_float2(0.0f, 0.0f);
            const uint32_t e = 32u * (w0 + uint32_t(j) * warps) + lane;
            gs[e] = x;
            p16[e] = __floats2half2_rn(x.p.x, x.p.y);
        }
    }
}

// Copies one float2 field (at float offset `field`: 0 features, 6
// gradient) of every grid entry from (to_state = 0) or into the training
// state, for parameter access and initialisation.
__global__ void k_grid_field(GridEntry* gs, float2* flat, uint32_t n, int field, int to_state) {
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    float2* f = reinterpret_cast<float2*>(reinterpret_cast<float*>(gs + e) + field);
    if (to_state) *f = flat[e];
    else flat[e] = *f;
}

// A frame's training slices from the sample count its paths left on the
// device (at most cap): `steps` consecutive runs of equal length, a
// multiple of 16 rows, all empty below 16 rows per step.  Slice k is
// {first row, rows} at slices[2k].
__global__ void k_cache_slices(const uint32_t* count, uint32_t cap, uint32_t steps, uint32_t* slices) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= steps) return;
    const uint32_t per = (min(*count, cap) / steps) & ~15u;
    slices[2 * k] = k * per;
    slices[2 * k + 1] = per;
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
    GridEntry* gs = nullptr;     // per entry: FP32 features, Adam moments, gradient
    __half2* g16 = nullptr;      // FP16 features (what the encodings gather)
    uint32_t* touched = nullptr; // bitmap: entries with a gradient since the last Adam step
    __half* wimg = nullptr;      // the MLP weights in the tcgen05 kernels' shared-memory layout
    // training buffers (capacity in samples)
    uint32_t cap = 0;
    float *tq = nullptr, *tt = nullptr, *tdout = nullptr, *tdin = nullptr, *loss = nullptr;
    __half *tin = nullptr, *tact = nullptr;
    uint32_t* tcount = nullptr;
    uint32_t step = 0;
    float last_loss = 0.0f;
    float* h_loss = nullptr;
    uint32_t frame = 0;
    // per-frame sample buffer (training paths) and query buffers (render)
    uint32_t scap = 0;
    float *sq = nullptr, *st = nullptr;
    size_t qcap = 0;
    float *qq = nullptr, *qpred = nullptr;
    float4* qpb = nullptr;
    // tcgen05 training images (k_cache_fwd_tc<true> -> k_cache_bwd_tc), capacity in tiles
    uint32_t tile_cap = 0;
    uint4 *timg = nullptr, *tdy = nullptr;
    // a frame's training slices (device), capacity in steps
    uint32_t* slices = nullptr;
    uint32_t slice_cap = 0;
    // inference and training on tcgen05 (k_cache_fwd_tc, k_cache_bwd_tc;
    // default) or on mma.sync (k_cache_infer, k_cache_train_fwd / _bwd)
    bool tcgen05 = true;
    // a cache frame trains on the context's side stream while its rays are
    // traced (joined before the cache is queried)
    bool overlap_training = true;
    int sm_count = 0;
};

namespace {

int ensure_train(mrt_ctx* ctx, mrt_cache* c, uint32_t n) {
    const uint32_t tiles = (n + kTcRows - 1) / kTcRows;
    if (c->tile_cap < tiles) {
        cudaFree(c->timg); cudaFree(c->tdy);
        c->timg = c->tdy = nullptr;
        c->tile_cap = 0;
        if (cudaMalloc(&c->timg, size_t(tiles) * kImgs * kImg) != cudaSuccess ||
            cudaMalloc(&c->tdy, size_t(tiles) * kDyImg) != cudaSuccess) {
            cudaGetLastError();
            return set_error(ctx, MRT_ENOMEM, "radiance cache: training images");
        }
        c->tile_cap = tiles;
    }
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

// The tcgen05 kernels' image (wimg_off) of FP16 weights [layer][out][in].
std::vector<__half> weight_image(const std::vector<__half>& w16) {
    std::vector<__half> img(kTcWBytes / 2, __float2half_rn(0.0f));
    for (int L = 0; L <= kHidden; ++L)
        for (int o = 0; o < (L < kHidden ? kWidth : kOutRows); ++o)
            for (int i = 0; i < kWidth; ++i)
                img[wimg_off(L, o, i) / 2] = w16[size_t(L) * kLayerW + size_t(o) * kWidth + i];
    return img;
}

uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// One training step on rows [0, n) of q / t, or on the device-side slice
// {first row, rows <= n} of them: forward, loss, backward (on tcgen05 or
// mma.sync), and with `apply` an Adam step.  Launches only: nothing is
// read back.
int train_step_launch(mrt_ctx* ctx, mrt_cache* c, const float* q, const float* t, uint32_t n, const uint32_t* slice,
                      int apply, cudaStream_t s) {
    int rc = ensure_train(ctx, c, n);
    if (rc) return rc;
    if (cudaMemsetAsync(c->loss, 0, 4, s) != cudaSuccess) return set_error(ctx, MRT_ECUDA, "train: memset");
    if (c->tcgen05) {
        // forward: one 128-row tile per CTA (up to 4 per SM); backward: one
        // CTA per SM, each accumulating the weight gradients of its tiles
        const uint32_t tiles = (n + kTcRows - 1) / kTcRows;
        const TrainTc tr{t, c->timg, c->tdy, c->loss};
        k_cache_fwd_tc<true><<<std::min<uint32_t>(tiles, uint32_t(c->sm_count) * 4u), kTcThreads, kTcSmem, s>>>(
            c->dev, q, n, slice, nullptr, ctx->d_status, tr);
        k_cache_bwd_tc<<<std::min<uint32_t>(tiles, uint32_t(c->sm_count)), kBwThreads, kBwSmem, s>>>(
            c->dev, q, n, slice, c->timg, c->tdy, c->wg, c->gs, c->touched, ctx->d_status);
        ctx->launches += 2;
    } else {
        const uint32_t tiles = n / 16u;
        const uint32_t blocks = std::min<uint32_t>((tiles + kMlpWarps - 1) / kMlpWarps, 2048u);
        k_cache_train_fwd<<<blocks, kMlpWarps * 32, smem_infer(), s>>>(c->dev, q, t, n, slice, c->tin, c->tact,
                                                                       c->tdout, c->loss);
        k_cache_train_bwd<<<blocks, kMlpWarps * 32, smem_bwd(), s>>>(c->dev, n, slice, c->tin, c->tact, c->tdout,
                                                                     c->wg, c->tdin);
        k_grid_bwd<<<(n + 127) / 128, 128, 0, s>>>(c->dev, q, c->tdin, n, slice, c->gs, c->touched);
        ctx->launches += 3;
    }
    if (apply) {
        c->step++;
        const float b1 = 0.9f, b2 = 0.99f, eps = 1e-10f;
        const float bc1 = 1.0f - std::pow(b1, float(c->step)), bc2 = 1.0f - std::pow(b2, float(c->step));
        k_adam<<<(kWeights + 255) / 256, 256, 0, s>>>(c->w, c->wm, c->wv, c->wg, c->w16, c->wt16, c->wimg,
                                                      kWeights, c->cfg.lr_mlp, b1, b2, eps, bc1, bc2, slice);
        const uint32_t nwords = c->grid_entries / 32u;  // bitmap words, one warp each
        k_adam_grid<<<std::min<uint32_t>((nwords + 7) / 8, uint32_t(c->sm_count) * 8u), 256, 0, s>>>(
            c->gs, c->g16, c->touched, nwords, c->cfg.lr_grid, b1, b2, eps, bc1, bc2);
        ctx->launches += 2;
    }
    if (cudaGetLastError() != cudaSuccess) return set_error(ctx, MRT_ECUDA, "train: launch failed");
    return MRT_OK;
}

// One float2 field of every grid entry's training state to or from host
// memory (2 floats an entry), through a staging buffer on the device.
cudaError_t grid_field(mrt_cache* c, float* host, int field, bool to_state) {
    const size_t bytes = size_t(c->grid_entries) * sizeof(float2);
    float2* flat = nullptr;
    cudaError_t e = cudaMalloc(&flat, bytes);
    if (e != cudaSuccess) return e;
    const uint32_t blocks = (c->grid_entries + 255u) / 256u;
    if (to_state) {
        e = cudaMemcpy(flat, host, bytes, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) k_grid_field<<<blocks, 256>>>(c->gs, flat, c->grid_entries, field, 1);
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
    } else {
        k_grid_field<<<blocks, 256>>>(c->gs, flat, c->grid_entries, field, 0);
        e = cudaDeviceSynchronize();
        if (e == cudaSuccess) e = cudaMemcpy(host, flat, bytes, cudaMemcpyDeviceToHost);
    }
    cudaFree(flat);
    return e;
}

} // namespace

namespace mrt {
uint32_t cache_query_vertex(const mrt_cache* c) { return c->cfg.query_vertex; }
bool cache_overlap_training(const mrt_cache* c) { return c->overlap_training; }

// Inference over device rows of 9 floats; with n_dev the row count is read
// on the device (at most n).
cudaError_t cache_infer(const mrt_cache* c, const float* q, uint32_t n, const uint32_t* n_dev, float* out,
                        uint32_t* status, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    if (c->tcgen05) {  // persistent: up to 4 CTAs (51 KB of shared memory, 64 TMEM columns each) per SM
        const uint32_t tiles = (n + kTcRows - 1) / kTcRows;
        const uint32_t blocks = std::min<uint32_t>(tiles, uint32_t(c->sm_count) * 4u);
        k_cache_fwd_tc<false><<<blocks, kTcThreads, kTcSmem, s>>>(c->dev, q, n, n_dev, out, status, TrainTc{});
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
// radiance a sample, then cfg.train_steps Adam steps on equal slices of the
// samples.  The slices are cut on the device from the sample count, so
// nothing is read back and the frame stays one stream of launches (the
// Adam step counter, and with it the bias correction, advances even for a
// frame whose paths left no samples, whose steps then change nothing).
int cache_train_frame(mrt_ctx* ctx, mrt_cache* c, const DevScene& sc, const FrameParams& fp, const TraceParams& tp,
                      uint32_t* status, cudaStream_t s) {
    const uint32_t paths = c->cfg.train_paths ? c->cfg.train_paths : 65536u;
    const uint32_t cap = paths * 4u;
    const uint32_t steps = c->cfg.train_steps ? c->cfg.train_steps : 4u;
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
        if (cudaMalloc(&c->tcount, 4) != cudaSuccess) return set_error(ctx, MRT_ENOMEM, "radiance cache: counter");
    }
    if (c->slice_cap < steps) {
        cudaFree(c->slices);
        c->slices = nullptr;
        c->slice_cap = 0;
        if (cudaMalloc(&c->slices, size_t(steps) * 2 * 4) != cudaSuccess)
            return set_error(ctx, MRT_ENOMEM, "radiance cache: training slices");
        c->slice_cap = steps;
    }
    const uint32_t per_max = (cap / steps) & ~15u;  // the most rows a slice can hold
    if (per_max < 16u) return MRT_OK;  // a step could never hold a whole 16-row tile: nothing to train
    if (cudaMemsetAsync(c->tcount, 0, 4, s) != cudaSuccess) return set_error(ctx, MRT_ECUDA, "cache: memset");
    if (launch_cache_train_paths(sc, fp, tp, c->cfg.train_bounces ? c->cfg.train_bounces : 8u, paths, c->frame++,
                                 c->sq, c->st, c->tcount, cap, status, s) != cudaSuccess)
        return set_error(ctx, MRT_ECUDA, "cache: training paths launch");
    k_cache_slices<<<(steps + 63) / 64, 64, 0, s>>>(c->tcount, cap, steps, c->slices);
    ctx->launches += 2;
    for (uint32_t k = 0; k < steps; ++k) {
        int rc = train_step_launch(ctx, c, c->sq, c->st, per_max, c->slices + 2 * k, 1, s);
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
              cudaMalloc(&c->gs, size_t(c->grid_entries) * sizeof(GridEntry)) == cudaSuccess &&
              cudaMalloc(&c->g16, gn * 2) == cudaSuccess && cudaMalloc(&c->loss, 4) == cudaSuccess &&
              cudaMalloc(&c->touched, c->grid_entries / 8) == cudaSuccess &&
              cudaMalloc(&c->wimg, kTcWBytes) == cudaSuccess && cudaMallocHost(&c->h_loss, 4) == cudaSuccess;
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
        const std::vector<__half> img = weight_image(w16);
        ok = cudaMemcpy(c->w, w.data(), kWeights * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
             cudaMemcpy(c->w16, w16.data(), kWeights * 2, cudaMemcpyHostToDevice) == cudaSuccess &&
             cudaMemcpy(c->wimg, img.data(), kTcWBytes, cudaMemcpyHostToDevice) == cudaSuccess &&
             cudaMemset(c->touched, 0, c->grid_entries / 8) == cudaSuccess &&
             cudaMemset(c->gs, 0, size_t(c->grid_entries) * sizeof(GridEntry)) == cudaSuccess &&
             grid_field(c, g.data(), 0, true) == cudaSuccess &&
             cudaMemcpy(c->wt16, wt16.data(), kWeights * 2, cudaMemcpyHostToDevice) == cudaSuccess &&
             cudaMemcpy(c->g16, g16.data(), gn * 2, cudaMemcpyHostToDevice) == cudaSuccess &&
             cudaMemset(c->wm, 0, kWeights * 4) == cudaSuccess && cudaMemset(c->wv, 0, kWeights * 4) == cudaSuccess &&
             cudaMemset(c->wg, 0, kWeights * 4) == cudaSuccess;
    }
    if (!ok ||
        cudaFuncSetAttribute(k_cache_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem_infer())) != cudaSuccess ||
        cudaFuncSetAttribute(k_cache_fwd_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem) != cudaSuccess ||
        cudaFuncSetAttribute(k_cache_fwd_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem) != cudaSuccess ||
        cudaFuncSetAttribute(k_cache_bwd_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kBwSmem) != cudaSuccess ||
        cudaFuncSetAttribute(k_cache_train_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem_infer())) != cudaSuccess ||
        cudaFuncSetAttribute(k_cache_train_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem_bwd())) != cudaSuccess) {
        cudaGetLastError();
        mrt_cuda_cache_destroy(ctx, c);
        return set_error(ctx, MRT_ECUDA, "cache_create: initialisation failed");
    }
    c->dev.grid = c->g16;
    c->dev.W = c->w16;
    c->dev.Wimg = c->wimg;
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

int mrt_cuda_cache_set_overlap(mrt_cache* c, int enable) {
    if (!c) return MRT_EINVAL;
    c->overlap_training = enable != 0;
    return MRT_OK;
}

int mrt_cuda_cache_destroy(mrt_ctx* ctx, mrt_cache* c) {
    if (!ctx || !c) return MRT_EINVAL;
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();
    void* ps[] = {c->w, c->wm, c->wv, c->wg, c->w16, c->wt16, c->gs, c->g16, c->loss, c->touched, c->wimg,
                  c->tq, c->tt, c->tdout, c->tdin, c->tin, c->tact, c->tcount, c->sq, c->st, c->qq, c->qpred, c->qpb,
                  c->timg, c->tdy, c->slices};
    for (void* p : ps) cudaFree(p);
    if (c->h_loss) cudaFreeHost(c->h_loss);
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
    int rc = train_step_launch(ctx, c, queries, targets, n, nullptr, apply_update, s);
    if (rc) return rc;
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
    const size_t total = which < 2 ? size_t(kWeights) : gn;
    if (count != total) return set_error(ctx, MRT_EINVAL, "cache_params: count mismatch");
    cudaDeviceSynchronize();
    if (which >= 2) {  // a field of the grid's training state: 0 features, 6 gradient
        const int field = which == 2 ? 0 : 6;
        if (grid_field(c, host, field, set != 0) != cudaSuccess) return set_error(ctx, MRT_ECUDA, "cache_params: copy");
        if (!set) return MRT_OK;
        if (which == 2) {
            std::vector<__half> g16(gn);
            for (size_t i = 0; i < gn; ++i) g16[i] = __float2half_rn(host[i]);
            cudaMemcpy(c->g16, g16.data(), gn * 2, cudaMemcpyHostToDevice);
        } else {  // gradients set by hand: mark their entries for the grid's next Adam step
            std::vector<uint32_t> bits(c->grid_entries / 32, 0u);
            for (size_t e = 0; e < c->grid_entries; ++e)
                if (host[2 * e] != 0.0f || host[2 * e + 1] != 0.0f) bits[e >> 5] |= 1u << (e & 31u);
            cudaMemcpy(c->touched, bits.data(), bits.size() * 4, cudaMemcpyHostToDevice);
        }
        return MRT_OK;
    }
    float* dptr = which == 0 ? c->w : c->wg;
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
        const std::vector<__half> img = weight_image(w16);
        cudaMemcpy(c->w16, w16.data(), kWeights * 2, cudaMemcpyHostToDevice);
        cudaMemcpy(c->wt16, wt16.data(), kWeights * 2, cudaMemcpyHostToDevice);
        cudaMemcpy(c->wimg, img.data(), kTcWBytes, cudaMemcpyHostToDevice);
    }
    return MRT_OK;
}

} // extern "C"
