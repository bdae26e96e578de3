// Learned denoiser: a 3-level encoder-decoder CNN (U-Net) over the 1-spp
// radiance and its feature buffers (albedo, normal, depth), trained on
// pairs the path tracer renders itself.  The reference's denoiser is a
// hand-set joint bilateral filter (src/gpu/denoise/bilateral.comp); this
// learned one is new.
//
// Tensors are NHWC BF16 with channel counts padded to multiples of 16.
// Topology (C = channels, s = 1/scale):
//   in(16) -> e0a(32) -> e0b(32)=S0 -> pool -> e1a(64) -> e1b(64)=S1 -> pool
//   -> e2a(128) -> e2b(128) -> [up ++ S1](192) -> d1a(64) -> d1b(64)
//   -> [up ++ S0](96) -> d0a(32) -> d0b(32) -> out(16, 3 used)
// 3x3 convolutions with bias, ReLU except the output layer.  Radiance is
// demodulated by the surface albedo (the noise-free texture need not be
// learned) and the network predicts a correction to the input's
// log(1 + radiance / albedo) (a residual: an untrained network passes the
// noisy image through); the loss is L1 in that space.  The output layer
// starts at a tenth of the He scale.
//
// Forward: implicit-GEMM convolution on the tcgen05 tensor cores with the
// accumulators in tensor memory (conv_tc.cuh, the default), or on mma.sync
// m16n8k16 (k_conv_fwd: a warp computes 16 consecutive pixels of a row x
// all output channels); both fold the decoder's 2x upsampling and skip
// concatenation into their operand loads.
// Backward (tcgen05 mode, the default): BF16 gradients at each layer's
// pre-activation; the data gradient of a layer is a forward convolution of
// its output gradient with the mirrored, transposed weights (the same
// persistent tensor-core kernel, whose epilogue applies the source's ReLU
// derivative), the gradient through an upsampling or a pooling is an
// elementwise pass, and the weight and bias gradients are tcgen05 GEMMs that
// reduce over the pixels (wgrad_tc.cuh).  The other modes keep FP32 kernels
// on the CUDA cores for the data, weight and bias gradients, reading the
// stored BF16 activations.
#include "internal.hpp"
#include "tcgen05.cuh"

#include <cuda.h>  // CUtensorMap (the encoder is fetched through the runtime)
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

namespace mrt {
int set_error(mrt_ctx* ctx, int code, const char* msg);
}
using namespace mrt;

namespace {

typedef __nv_bfloat16 bf16;

struct ConvDesc {
    int ca, cb, cout;   // input channels from source A, from source B (skip), outputs
    int ups;            // source A is half resolution, nearest-upsampled
    int relu;
    int scale;          // resolution level of the output (0 full, 1 half, 2 quarter)
    size_t w_off, b_off;
};

constexpr int kLayers = 11;
// ca, cb, cout, ups, relu, scale
const int kTopo[kLayers][6] = {
    {16, 0, 32, 0, 1, 0},   // e0a
    {32, 0, 32, 0, 1, 0},   // e0b -> S0
    {32, 0, 64, 0, 1, 1},   // e1a (input pooled S0)
    {64, 0, 64, 0, 1, 1},   // e1b -> S1
    {64, 0, 128, 0, 1, 2},  // e2a (input pooled S1)
    {128, 0, 128, 0, 1, 2}, // e2b
    {128, 64, 64, 1, 1, 1}, // d1a: up(e2b) ++ S1
    {64, 0, 64, 0, 1, 1},   // d1b
    {64, 32, 32, 1, 1, 0},  // d0a: up(d1b) ++ S0
    {32, 0, 32, 0, 1, 0},   // d0b
    {32, 0, 16, 0, 0, 0},   // out (3 channels used)
};

__device__ __forceinline__ void mma_bf16(float* d, const uint32_t* a, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

struct ConvArgs {
    const bf16* a;   // source A: N x Ha x Wa x ca
    const bf16* b;   // source B: N x H x W x cb (or null)
    const bf16* w;   // cout x 9 x (ca + cb)
    const float* bias;
    bf16* y;         // N x H x W x cout
    int n, h, w_, ca, cb, cout, ups, relu;
    // tensor-core epilogue only: when set, an output is kept where this
    // N x H x W x cout tensor is positive and zeroed elsewhere (the ReLU
    // derivative of a data-gradient convolution)
    const bf16* gate = nullptr;
};

// channel pair (c, c+1) of the virtual concatenated input at (n, y, x)
__device__ __forceinline__ uint32_t in_pair(const ConvArgs& a, int n, int y, int x, int c) {
    if (y < 0 || y >= a.h || x < 0 || x >= a.w_) return 0u;
    if (c < a.ca) {
        const int ha = a.ups ? a.h >> 1 : a.h, wa = a.ups ? a.w_ >> 1 : a.w_;
        const int ya = a.ups ? y >> 1 : y, xa = a.ups ? x >> 1 : x;
        return *reinterpret_cast<const uint32_t*>(a.a + ((size_t(n) * ha + ya) * wa + xa) * a.ca + c);
    }
    return *reinterpret_cast<const uint32_t*>(a.b + ((size_t(n) * a.h + y) * a.w_ + x) * a.cb + (c - a.ca));
}

// One warp: 16 pixels (x0 .. x0+15) of row y of image n, all 8*NT outputs.
template <int NT>
__global__ void __launch_bounds__(128) k_conv_fwd(ConvArgs a) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, g = lane >> 2, t = lane & 3;
    const int tiles_x = (a.w_ + 63) / 64;
    int bid = blockIdx.x;
    const int tx = bid % tiles_x;
    bid /= tiles_x;
    const int y = bid % a.h, n = bid / a.h;
    const int x0 = tx * 64 + warp * 16;
    if (x0 >= a.w_) return;
    const int cin = a.ca + a.cb;
    float acc[NT][4];
#pragma unroll
    for (int j = 0; j < NT; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
    for (int tap = 0; tap < 9; ++tap) {
        const int dy = tap / 3 - 1, dx = tap % 3 - 1;
        for (int kc = 0; kc < cin; kc += 16) {
            uint32_t af[4];
            af[0] = in_pair(a, n, y + dy, x0 + g + dx, kc + 2 * t);
            af[1] = in_pair(a, n, y + dy, x0 + g + 8 + dx, kc + 2 * t);
            af[2] = in_pair(a, n, y + dy, x0 + g + dx, kc + 8 + 2 * t);
            af[3] = in_pair(a, n, y + dy, x0 + g + 8 + dx, kc + 8 + 2 * t);
#pragma unroll
            for (int j = 0; j < NT; ++j) {
                const bf16* wr = a.w + (size_t(8 * j + g) * 9 + tap) * cin + kc + 2 * t;
                mma_bf16(acc[j], af, __ldg(reinterpret_cast<const unsigned int*>(wr)),
                         __ldg(reinterpret_cast<const unsigned int*>(wr + 8)));
            }
        }
    }
#pragma unroll
    for (int j = 0; j < NT; ++j) {
        const int c = 8 * j + 2 * t;
        const float b0 = a.bias[c], b1 = a.bias[c + 1];
        float v[4] = {acc[j][0] + b0, acc[j][1] + b1, acc[j][2] + b0, acc[j][3] + b1};
        if (a.relu)
            for (int k = 0; k < 4; ++k) v[k] = fmaxf(v[k], 0.0f);
        const int xr0 = x0 + g, xr1 = x0 + g + 8;
        if (xr0 < a.w_)
            *reinterpret_cast<__nv_bfloat162*>(a.y + ((size_t(n) * a.h + y) * a.w_ + xr0) * a.cout + c) =
                __floats2bfloat162_rn(v[0], v[1]);
        if (xr1 < a.w_)
            *reinterpret_cast<__nv_bfloat162*>(a.y + ((size_t(n) * a.h + y) * a.w_ + xr1) * a.cout + c) =
                __floats2bfloat162_rn(v[2], v[3]);
    }
}

#include "conv_tc.cuh"
#include "wgrad_tc.cuh"

// 2x2 average pool, NHWC
__global__ void k_pool(const bf16* x, bf16* y, int n, int h, int w, int c) {
    // one thread per 8 channels of an output pixel: four 16-byte loads, the
    // sum taken in the same order as the scalar form (bit-identical)
    const int c8 = c / 8;
    const size_t total = size_t(n) * (h / 2) * (w / 2) * c8;
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < total; i += size_t(gridDim.x) * blockDim.x) {
        const int cg = int(i % c8);
        size_t p = i / c8;
        const int xo = int(p % (w / 2));
        p /= (w / 2);
        const int yo = int(p % (h / 2));
        const int nn = int(p / (h / 2));
        float s[8] = {};
        for (int k = 0; k < 4; ++k) {
            const uint4 v = *reinterpret_cast<const uint4*>(
                x + ((size_t(nn) * h + 2 * yo + (k >> 1)) * w + 2 * xo + (k & 1)) * c + 8 * cg);
            const __nv_bfloat162* b = reinterpret_cast<const __nv_bfloat162*>(&v);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float2 f = __bfloat1622float2(b[q]);
                s[2 * q] += f.x;
                s[2 * q + 1] += f.y;
            }
        }
        uint4 o;
        __nv_bfloat162* ob = reinterpret_cast<__nv_bfloat162*>(&o);
#pragma unroll
        for (int q = 0; q < 4; ++q) ob[q] = __floats2bfloat162_rn(0.25f * s[2 * q], 0.25f * s[2 * q + 1]);
        *reinterpret_cast<uint4*>(y + (i / c8) * c + 8 * cg) = o;
    }
}

// ---- backward (FP32) ----------------------------------------------------

// dz = dy * relu'(y) in place (y: stored bf16 output)
__global__ void k_relu_bwd(float* dy, const bf16* y, size_t count) {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < count; i += size_t(gridDim.x) * blockDim.x)
        if (!(__bfloat162float(y[i]) > 0.0f)) dy[i] = 0.0f;
}

// data gradient: for each input element of the virtual concatenated input
// at output resolution, sum over taps and outputs; written (accumulated) to
// the source gradient buffers (upsampled source: atomics into its parent)
__global__ void k_conv_bwd_data(const float* dz, const bf16* w, int n, int h, int wd, int ca, int cb, int cout, int ups,
                                float* ga, float* gb) {
    const int cin = ca + cb;
    const size_t total = size_t(n) * h * wd * cin;
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < total; i += size_t(gridDim.x) * blockDim.x) {
        const int ci = int(i % cin);
        size_t p = i / cin;
        const int x = int(p % wd);
        p /= wd;
        const int y = int(p % h);
        const int nn = int(p / h);
        float s = 0.0f;
        for (int tap = 0; tap < 9; ++tap) {
            const int dy = tap / 3 - 1, dx = tap % 3 - 1;
            const int yo = y - dy, xo = x - dx;  // output pixel that read (y, x) through this tap
            if (yo < 0 || yo >= h || xo < 0 || xo >= wd) continue;
            const float* dzr = dz + ((size_t(nn) * h + yo) * wd + xo) * cout;
            const bf16* wr = w + size_t(tap) * cin + ci;
            for (int co = 0; co < cout; ++co) s = fmaf(dzr[co], __bfloat162float(wr[size_t(co) * 9 * cin]), s);
        }
        if (ci < ca) {
            if (ups) atomicAdd(&ga[((size_t(nn) * (h / 2) + y / 2) * (wd / 2) + x / 2) * ca + ci], s);
            else ga[((size_t(nn) * h + y) * wd + x) * ca + ci] += s;
        } else {
            gb[((size_t(nn) * h + y) * wd + x) * cb + (ci - ca)] += s;
        }
    }
}

// weight + bias gradients: block (co-tile of 16, ci-tile of 16, tap) over a
// slice of pixels, partial sums atomically added
__global__ void __launch_bounds__(256)
k_conv_bwd_weight(const float* dz, const bf16* xa, const bf16* xb, int n, int h, int wd, int ca, int cb, int cout,
                  int ups, int pix_per_block, float* gw, float* gbias) {
    const int cin = ca + cb;
    const int co_tiles = (cout + 15) / 16, ci_tiles = cin / 16;
    int bid = blockIdx.x;
    const int tap = bid % 9;
    bid /= 9;
    const int cit = bid % ci_tiles;
    bid /= ci_tiles;
    const int cot = bid % co_tiles;
    const int slice = bid / co_tiles;
    const int dy = tap / 3 - 1, dx = tap % 3 - 1;
    const int co = cot * 16 + (threadIdx.x >> 4), ci = cit * 16 + (threadIdx.x & 15);
    const size_t total = size_t(n) * h * wd;
    const size_t p0 = size_t(slice) * pix_per_block, p1 = std::min(total, p0 + size_t(pix_per_block));
    float s = 0.0f, sb = 0.0f;
    const int ha = ups ? h / 2 : h, wa = ups ? wd / 2 : wd;
    for (size_t p = p0; p < p1; ++p) {
        const int x = int(p % wd);
        const int y = int((p / wd) % h);
        const int nn = int(p / (size_t(wd) * h));
        const float d = co < cout ? dz[p * cout + co] : 0.0f;
        sb += d;
        const int yi = y + dy, xi = x + dx;
        if (yi < 0 || yi >= h || xi < 0 || xi >= wd) continue;
        float xv;
        if (ci < ca) {
            const int yy = ups ? yi >> 1 : yi, xx = ups ? xi >> 1 : xi;
            xv = __bfloat162float(xa[((size_t(nn) * ha + yy) * wa + xx) * ca + ci]);
        } else {
            xv = __bfloat162float(xb[((size_t(nn) * h + yi) * wd + xi) * cb + (ci - ca)]);
        }
        s = fmaf(d, xv, s);
    }
    if (co < cout) {
        atomicAdd(&gw[(size_t(co) * 9 + tap) * cin + ci], s);
        if (tap == 4 && cit == 0 && (threadIdx.x & 15) == 0) atomicAdd(&gbias[co], sb);
    }
}

// pool backward: g_in[2y+i][2x+j] += g_out[y][x] / 4
__global__ void k_pool_bwd(const float* gout, float* gin, int n, int h, int w, int c) {
    const size_t total = size_t(n) * h * w * c;
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < total; i += size_t(gridDim.x) * blockDim.x) {
        const int ch = int(i % c);
        size_t p = i / c;
        const int x = int(p % w);
        p /= w;
        const int y = int(p % h);
        const int nn = int(p / h);
        gin[i] += 0.25f * gout[((size_t(nn) * (h / 2) + y / 2) * (w / 2) + x / 2) * c + ch];
    }
}

// Albedo a pixel's radiance is divided by before denoising (features 3..5
// as stored, BF16); sky pixels and black surfaces (albedo 0) use 1.
__device__ __forceinline__ float demod_albedo(const bf16* feat, size_t p, int k) {
    const float a = __bfloat162float(feat[p * 16 + 3 + k]);
    return a > 0.0f ? a : 1.0f;
}

// L1 loss in log(1 + irradiance) space on channels 0..2 (irradiance =
// radiance / albedo): the network predicts a correction added to the
// input's own log(1 + irradiance) (features 0..2)
// (gradient written as FP32 to dy, or as BF16 to dy16 when that is set)
__global__ void k_l1_loss(const bf16* y, const bf16* feat, const float* target, size_t pixels, float* dy,
                          bf16* dy16, float* loss) {
    float l = 0.0f;
    const float inv = 1.0f / float(pixels * 3);
    for (size_t p = blockIdx.x * size_t(blockDim.x) + threadIdx.x; p < pixels; p += size_t(gridDim.x) * blockDim.x) {
        float g[16] = {};
        for (int k = 0; k < 3; ++k) {
            const float pred = __bfloat162float(y[p * 16 + k]) + __bfloat162float(feat[p * 16 + k]);
            const float d = pred - log1pf(fmaxf(target[p * 3 + k], 0.0f) / demod_albedo(feat, p, k));
            l += fabsf(d);
            g[k] = (d > 0.0f ? 1.0f : (d < 0.0f ? -1.0f : 0.0f)) * inv;
        }
        if (dy16) {
            for (int k = 0; k < 16; k += 2)
                *reinterpret_cast<__nv_bfloat162*>(dy16 + p * 16 + k) = __floats2bfloat162_rn(g[k], g[k + 1]);
        } else {
            for (int k = 0; k < 16; ++k) dy[p * 16 + k] = g[k];
        }
    }
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xFFFFFFFFu, l, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, l * inv);
}

// ---- backward (BF16, tensor-core mode) ------------------------------------

// Weights of the data-gradient convolutions in the TMA form's layout.  The
// data gradient of a 3x3 convolution is a 3x3 convolution of its output
// gradient with the taps mirrored and inputs and outputs swapped:
// W'[ci][tap][co] = W[co][8 - tap][ci].  Per layer and source part (a: input
// channels [0, ca), b: [ca, ca + cb)) the part's W' is stored as
// [slice of 16 co][tap][half][ci][8 co] at dst_off.
struct BwdTable {
    int parts;
    int cp[2 * kLayers], cout[2 * kLayers], ci0[2 * kLayers], cin[2 * kLayers];
    size_t src_off[2 * kLayers], dst_off[2 * kLayers];
};
__global__ void k_bwd_weights(const bf16* w16, bf16* wt, BwdTable t) {
    for (int e = 0; e < t.parts; ++e) {
        const int cp = t.cp[e], cin = t.cin[e], ci0 = t.ci0[e];
        const size_t total = size_t(9) * cp * t.cout[e];
        for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < total; i += size_t(gridDim.x) * blockDim.x) {
            const int e8 = int(i % 8);
            size_t q = i / 8;
            const int ci = int(q % cp);
            q /= cp;
            const int hf = int(q % 2);
            q /= 2;
            const int tap = int(q % 9);
            const int k = int(q / 9);
            const int co = 16 * k + 8 * hf + e8;
            wt[t.dst_off[e] + i] = w16[t.src_off[e] + (size_t(co) * 9 + (8 - tap)) * cin + ci0 + ci];
        }
    }
}

// Gradient of a source read through the nearest 2x upsampling: the sum of
// the 2x2 children of t (2h x 2w, full-resolution data gradient), kept where
// the source's stored activation is positive (its ReLU), into dz (h x w).
// One thread per 8 channels of a pixel.
__global__ void k_bwd_unup(const bf16* t, const bf16* act, bf16* dz, int n, int h, int w, int c) {
    const int c8 = c / 8;
    const size_t total = size_t(n) * h * w * c8;
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < total; i += size_t(gridDim.x) * blockDim.x) {
        const int cg = int(i % c8);
        const size_t p = i / c8;
        const int x = int(p % w), y = int((p / w) % h), nn = int(p / (size_t(w) * h));
        float s[8] = {};
        for (int k = 0; k < 4; ++k) {
            const uint4 v = *reinterpret_cast<const uint4*>(
                t + ((size_t(nn) * 2 * h + 2 * y + (k >> 1)) * 2 * w + 2 * x + (k & 1)) * c + 8 * cg);
            const __nv_bfloat162* b = reinterpret_cast<const __nv_bfloat162*>(&v);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float2 f = __bfloat1622float2(b[q]);
                s[2 * q] += f.x;
                s[2 * q + 1] += f.y;
            }
        }
        const uint4 gv = *reinterpret_cast<const uint4*>(act + p * c + 8 * cg);
        const __nv_bfloat162* g = reinterpret_cast<const __nv_bfloat162*>(&gv);
        uint4 o;
        __nv_bfloat162* ob = reinterpret_cast<__nv_bfloat162*>(&o);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float2 gf = __bfloat1622float2(g[q]);
            ob[q] = __floats2bfloat162_rn(gf.x > 0.0f ? s[2 * q] : 0.0f, gf.y > 0.0f ? s[2 * q + 1] : 0.0f);
        }
        *reinterpret_cast<uint4*>(dz + p * c + 8 * cg) = o;
    }
}

// Gradient of a skip source that is also pooled: its data gradient through
// the skip concatenation plus a quarter of the pooled input's gradient
// (h/2 x w/2), kept where the source's activation is positive, into dz.
__global__ void k_bwd_unpool(const bf16* skip, const bf16* gp, const bf16* act, bf16* dz, int n, int h, int w,
                             int c) {
    const int c8 = c / 8;
    const size_t total = size_t(n) * h * w * c8;
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < total; i += size_t(gridDim.x) * blockDim.x) {
        const int cg = int(i % c8);
        const size_t p = i / c8;
        const int x = int(p % w), y = int((p / w) % h), nn = int(p / (size_t(w) * h));
        const uint4 sv = *reinterpret_cast<const uint4*>(skip + p * c + 8 * cg);
        const uint4 pv = *reinterpret_cast<const uint4*>(
            gp + ((size_t(nn) * (h / 2) + y / 2) * (w / 2) + x / 2) * c + 8 * cg);
        const uint4 gv = *reinterpret_cast<const uint4*>(act + p * c + 8 * cg);
        const __nv_bfloat162* sb = reinterpret_cast<const __nv_bfloat162*>(&sv);
        const __nv_bfloat162* pb = reinterpret_cast<const __nv_bfloat162*>(&pv);
        const __nv_bfloat162* gb = reinterpret_cast<const __nv_bfloat162*>(&gv);
        uint4 o;
        __nv_bfloat162* ob = reinterpret_cast<__nv_bfloat162*>(&o);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float2 a = __bfloat1622float2(sb[q]), b = __bfloat1622float2(pb[q]), g = __bfloat1622float2(gb[q]);
            ob[q] = __floats2bfloat162_rn(g.x > 0.0f ? a.x + 0.25f * b.x : 0.0f, g.y > 0.0f ? a.y + 0.25f * b.y : 0.0f);
        }
        *reinterpret_cast<uint4*>(dz + p * c + 8 * cg) = o;
    }
}

__global__ void k_adam_bf16(float* p, float* m, float* v, float* g, bf16* p16, size_t n, float lr, float b1, float b2,
                            float eps, float bc1, float bc2) {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
        const float gr = g[i];
        g[i] = 0.0f;
        const float mi = b1 * m[i] + (1.0f - b1) * gr, vi = b2 * v[i] + (1.0f - b2) * gr * gr;
        m[i] = mi;
        v[i] = vi;
        const float pi = p[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
        p[i] = pi;
        if (p16) p16[i] = __float2bfloat16_rn(pi);
    }
}

// Input features of one frame: log(1 + radiance / albedo) (3), albedo (3),
// normal (3), hit distance / scene diagonal (1), zeros to 16 channels.  The
// albedo divides out as stored in BF16, so decoding multiplies by exactly
// the same value.
__global__ void k_features(DevScene sc, const float* color, const uint32_t* vis, const float* hit_t, int w, int h,
                           float inv_diag, bf16* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w * h) return;
    float f[16];
    for (int k = 0; k < 16; ++k) f[k] = 0.0f;
    float a[3] = {1.0f, 1.0f, 1.0f};
    const uint32_t prim = vis[i];
    if (prim != kMiss && prim < sc.mat_count) {
        const mrt_material m = sc.mats[prim];
        for (int k = 0; k < 3; ++k) {
            f[3 + k] = __bfloat162float(__float2bfloat16_rn(float((m.albedo_rgba8 >> (8 * k)) & 0xFFu) / 255.0f));
            if (f[3 + k] > 0.0f) a[k] = f[3 + k];
        }
        f[6] = m.normal[0]; f[7] = m.normal[1]; f[8] = m.normal[2];
        f[9] = fminf(hit_t[i] * inv_diag, 4.0f);
    } else {
        f[9] = 4.0f;
    }
    for (int k = 0; k < 3; ++k) f[k] = log1pf(fmaxf(color[size_t(i) * 3 + k], 0.0f) / a[k]);
    for (int k = 0; k < 16; k += 2)
        *reinterpret_cast<__nv_bfloat162*>(out + size_t(i) * 16 + k) = __floats2bfloat162_rn(f[k], f[k + 1]);
}

// radiance = albedo x (exp(input log(1 + irradiance) + correction) - 1)
__global__ void k_decode(const bf16* y, const bf16* feat, size_t pixels, float* out) {
    for (size_t p = blockIdx.x * size_t(blockDim.x) + threadIdx.x; p < pixels; p += size_t(gridDim.x) * blockDim.x)
        for (int k = 0; k < 3; ++k) {
            const float v = __bfloat162float(y[p * 16 + k]) + __bfloat162float(feat[p * 16 + k]);
            out[p * 3 + k] = expm1f(fmaxf(v, 0.0f)) * demod_albedo(feat, p, k);
        }
}

int grid_for(size_t n) { return int(std::min<size_t>((n + 255) / 256, 65535)); }

} // namespace

struct mrt_denoiser {
    ConvDesc layers[kLayers];
    size_t n_w = 0, n_b = 0;
    float *w = nullptr, *wm = nullptr, *wv = nullptr, *wg = nullptr;  // weights + biases, FP32
    bf16* w16 = nullptr;
    bf16* wtc = nullptr;          // w16 re-laid out per 16-channel slice for the TMA convolution
    bf16* wst = nullptr;          // the 16/32-channel layers' weights for the row-stacked form
    bf16* wup = nullptr;          // per-slice weights of the phase-decomposed upsampling layers
    size_t up_off[kLayers] = {};  // their offsets in wup (upsampling layers only)
    // tc_mode the re-laid-out weights (wtc, wst, wup) were made for; -1
    // when the BF16 weights changed since (an Adam step, a parameter write)
    mutable int relayout_mode = -1;
    // activation tensors (bf16) and their gradients (fp32), sized for n*h*w
    size_t cap_pix = 0, grad_pix = 0;
    bf16* act[kLayers] = {};
    bf16 *pool0 = nullptr, *pool1 = nullptr;
    float* grad[kLayers] = {};
    float *gpool0 = nullptr, *gpool1 = nullptr, *gin = nullptr;
    // tensor-core backward: BF16 gradients at each layer's pre-activation
    // (gz), the data gradients of the decoder's upsampled sources at the
    // consumer's resolution (up8: d0a's, 64 channels at full resolution; up6:
    // d1a's, 128 at half), of the skip sources (skip8: S0 from d0a, skip6: S1
    // from d1a) and of the pooled inputs (gp0, gp1); the mirrored, transposed
    // weights of the data-gradient convolutions (wbt) and zero biases
    size_t gz_pix = 0;
    bf16* gz[kLayers] = {};
    bf16 *up8 = nullptr, *up6 = nullptr, *skip8 = nullptr, *skip6 = nullptr, *gp0 = nullptr, *gp1 = nullptr;
    bf16* wbt = nullptr;
    float* zeros = nullptr;
    float* loss = nullptr;
    float* h_loss = nullptr;
    uint32_t step = 0;
    // forward convolutions: 0 mma.sync, 1 tcgen05 with one CTA per tile
    // (k_conv_tma / k_conv_tc), 2 tcgen05 with persistent warp-specialised
    // CTAs for the layers without upsampling (k_conv_ws; default)
    int tc_mode = 2;
    int sm_count = 0;
    uint32_t* status = nullptr;   // the context's device status word
};

namespace {

size_t layer_pixels(size_t full, int scale) { return full >> (2 * scale); }

// activations for n*h*w pixels; gradient buffers only when training
int ensure_acts(mrt_ctx* ctx, mrt_denoiser* d, size_t pix, bool grads) {
    if (d->cap_pix < pix) {
        for (int l = 0; l < kLayers; ++l) { cudaFree(d->act[l]); d->act[l] = nullptr; }
        cudaFree(d->pool0); cudaFree(d->pool1);
        d->pool0 = d->pool1 = nullptr;
        d->cap_pix = 0;
        bool ok = true;
        for (int l = 0; l < kLayers && ok; ++l)
            ok = cudaMalloc(&d->act[l], layer_pixels(pix, d->layers[l].scale) * d->layers[l].cout * 2) == cudaSuccess;
        ok = ok && cudaMalloc(&d->pool0, layer_pixels(pix, 1) * 32 * 2) == cudaSuccess &&
             cudaMalloc(&d->pool1, layer_pixels(pix, 2) * 64 * 2) == cudaSuccess;
        if (!ok) {
            cudaGetLastError();
            return set_error(ctx, MRT_ENOMEM, "denoiser: activation buffers");
        }
        d->cap_pix = pix;
    }
    if (grads && d->tc_mode == 2 && d->gz_pix < pix) {
        for (int l = 0; l < kLayers; ++l) { cudaFree(d->gz[l]); d->gz[l] = nullptr; }
        bf16** tmp[] = {&d->up8, &d->up6, &d->skip8, &d->skip6, &d->gp0, &d->gp1};
        for (bf16** t : tmp) { cudaFree(*t); *t = nullptr; }
        d->gz_pix = 0;
        bool ok = true;
        for (int l = 0; l < kLayers && ok; ++l)
            ok = cudaMalloc(&d->gz[l], layer_pixels(pix, d->layers[l].scale) * d->layers[l].cout * 2) == cudaSuccess;
        ok = ok && cudaMalloc(&d->up8, pix * 64 * 2) == cudaSuccess &&
             cudaMalloc(&d->up6, layer_pixels(pix, 1) * 128 * 2) == cudaSuccess &&
             cudaMalloc(&d->skip8, pix * 32 * 2) == cudaSuccess &&
             cudaMalloc(&d->skip6, layer_pixels(pix, 1) * 64 * 2) == cudaSuccess &&
             cudaMalloc(&d->gp0, layer_pixels(pix, 1) * 32 * 2) == cudaSuccess &&
             cudaMalloc(&d->gp1, layer_pixels(pix, 2) * 64 * 2) == cudaSuccess;
        if (!ok) {
            cudaGetLastError();
            return set_error(ctx, MRT_ENOMEM, "denoiser: gradient buffers");
        }
        d->gz_pix = pix;
    }
    if (grads && d->tc_mode != 2 && d->grad_pix < pix) {
        for (int l = 0; l < kLayers; ++l) { cudaFree(d->grad[l]); d->grad[l] = nullptr; }
        cudaFree(d->gpool0); cudaFree(d->gpool1); cudaFree(d->gin);
        d->gpool0 = d->gpool1 = d->gin = nullptr;
        d->grad_pix = 0;
        bool ok = true;
        for (int l = 0; l < kLayers && ok; ++l)
            ok = cudaMalloc(&d->grad[l], layer_pixels(pix, d->layers[l].scale) * d->layers[l].cout * 4) == cudaSuccess;
        ok = ok && cudaMalloc(&d->gpool0, layer_pixels(pix, 1) * 32 * 4) == cudaSuccess &&
             cudaMalloc(&d->gpool1, layer_pixels(pix, 2) * 64 * 4) == cudaSuccess &&
             cudaMalloc(&d->gin, pix * 16 * 4) == cudaSuccess;
        if (!ok) {
            cudaGetLastError();
            return set_error(ctx, MRT_ENOMEM, "denoiser: gradient buffers");
        }
        d->grad_pix = pix;
    }
    return MRT_OK;
}

cudaError_t conv(const mrt_denoiser* d, int l, const bf16* a, const bf16* b, int n, int h, int w, cudaStream_t s) {
    const ConvDesc& L = d->layers[l];
    ConvArgs ca{a, b, d->w16 + L.w_off, d->w + L.b_off, d->act[l], n, h, w, L.ca, L.cb, L.cout, L.ups, L.relu};
    if (d->tc_mode == 2) {
        const bf16* wt = d->wtc + L.w_off;
        if (L.ups) {  // the decoder's two upsampling layers: phase-decomposed
            const bf16* wu = d->wup + d->up_off[l];
            if (L.cout == 32) return launch_conv_up<32>(ca, wu, d->status, d->sm_count, s);
            if (L.cout == 64) return launch_conv_up<64>(ca, wu, d->status, d->sm_count, s);
        } else {
            switch (L.cout) {  // 16 and 32 channels: row-stacked
            case 16: return launch_conv_ws<16, true>(ca, d->wst + L.w_off, d->status, d->sm_count, s);
            case 32: return launch_conv_ws<32, true>(ca, d->wst + L.w_off, d->status, d->sm_count, s);
            case 64: return launch_conv_ws<64>(ca, wt, d->status, d->sm_count, s);
            default: return launch_conv_ws<128>(ca, wt, d->status, d->sm_count, s);
            }
        }
    }
    if (d->tc_mode == 1 && !L.ups) {
        const bf16* wt = d->wtc + L.w_off;
        switch (L.cout) {
        case 16: return launch_conv_tma<16>(ca, wt, d->status, s);
        case 32: return launch_conv_tma<32>(ca, wt, d->status, s);
        case 64: return launch_conv_tma<64>(ca, wt, d->status, s);
        default: return launch_conv_tma<128>(ca, wt, d->status, s);
        }
    }
    if (d->tc_mode != 0) {
        switch (L.cout) {
        case 16: return launch_conv_tc<16>(ca, d->status, s);
        case 32: return launch_conv_tc<32>(ca, d->status, s);
        case 64: return launch_conv_tc<64>(ca, d->status, s);
        default: return launch_conv_tc<128>(ca, d->status, s);
        }
    }
    const int blocks = ((w + 63) / 64) * h * n;
    switch (L.cout) {
    case 16: k_conv_fwd<2><<<blocks, 128, 0, s>>>(ca); break;
    case 32: k_conv_fwd<4><<<blocks, 128, 0, s>>>(ca); break;
    case 64: k_conv_fwd<8><<<blocks, 128, 0, s>>>(ca); break;
    default: k_conv_fwd<16><<<blocks, 128, 0, s>>>(ca); break;
    }
    return cudaGetLastError();
}

// whether forward() re-lays out the weights for the tensor-core kernels
// (only after they changed: inference with fixed weights does it once)
bool needs_relayout(const mrt_denoiser* d) { return d->tc_mode != 0 && d->relayout_mode != d->tc_mode; }

// kernels the next forward() launches
int forward_launches(const mrt_denoiser* d) {
    return 13 + (needs_relayout(d) ? 1 + (d->tc_mode == 2 ? 3 : 0) : 0);  // 11 convolutions, 2 pools
}

// forward of the whole network over n images of h x w (h, w multiples of 4)
cudaError_t forward(const mrt_denoiser* d, const bf16* in, int n, int h, int w, cudaStream_t s) {
    cudaError_t e;
    if (needs_relayout(d)) {  // the TMA convolutions read the weights per slice
        d->relayout_mode = d->tc_mode;
        TcLayerTable t{};
        t.count = kLayers;
        for (int l = 0; l < kLayers; ++l) {
            t.cin[l] = d->layers[l].ca + d->layers[l].cb;
            t.cout[l] = d->layers[l].cout;
            t.off[l] = d->layers[l].w_off;
        }
        k_tc_weights<<<304, 256, 0, s>>>(d->w16, d->wtc, t);
        if (d->tc_mode == 2) k_tc_weights_stack<<<304, 256, 0, s>>>(d->w16, d->wst, t);
        if (d->tc_mode == 2)
            for (int l = 0; l < kLayers; ++l)
                if (d->layers[l].ups)
                    k_up_weights<<<152, 256, 0, s>>>(d->w16 + d->layers[l].w_off, d->wup + d->up_off[l],
                                                     d->layers[l].ca, d->layers[l].cb, d->layers[l].cout);
    }
    if ((e = conv(d, 0, in, nullptr, n, h, w, s))) return e;
    if ((e = conv(d, 1, d->act[0], nullptr, n, h, w, s))) return e;
    k_pool<<<grid_for(size_t(n) * h * w * 4 / 4), 256, 0, s>>>(d->act[1], d->pool0, n, h, w, 32);
    if ((e = conv(d, 2, d->pool0, nullptr, n, h / 2, w / 2, s))) return e;
    if ((e = conv(d, 3, d->act[2], nullptr, n, h / 2, w / 2, s))) return e;
    k_pool<<<grid_for(size_t(n) * h * w * 8 / 16), 256, 0, s>>>(d->act[3], d->pool1, n, h / 2, w / 2, 64);
    if ((e = conv(d, 4, d->pool1, nullptr, n, h / 4, w / 4, s))) return e;
    if ((e = conv(d, 5, d->act[4], nullptr, n, h / 4, w / 4, s))) return e;
    if ((e = conv(d, 6, d->act[5], d->act[3], n, h / 2, w / 2, s))) return e;
    if ((e = conv(d, 7, d->act[6], nullptr, n, h / 2, w / 2, s))) return e;
    if ((e = conv(d, 8, d->act[7], d->act[1], n, h, w, s))) return e;
    if ((e = conv(d, 9, d->act[8], nullptr, n, h, w, s))) return e;
    return conv(d, 10, d->act[9], nullptr, n, h, w, s);
}

// backward of layer l: grad[l] holds dL/d(output); accumulates into the
// gradient buffers of its sources and into the weight/bias gradients
void bwd_layer(mrt_denoiser* d, int l, const bf16* xa, const bf16* xb, float* ga, float* gb, int n, int h, int w,
               cudaStream_t s) {
    const ConvDesc& L = d->layers[l];
    const size_t pix = size_t(n) * h * w;
    if (L.relu) k_relu_bwd<<<grid_for(pix * L.cout), 256, 0, s>>>(d->grad[l], d->act[l], pix * L.cout);
    const int ppb = 1024;
    const int slices = int((pix + ppb - 1) / ppb);
    const int blocks = slices * ((L.cout + 15) / 16) * ((L.ca + L.cb) / 16) * 9;
    k_conv_bwd_weight<<<blocks, 256, 0, s>>>(d->grad[l], xa, xb, n, h, w, L.ca, L.cb, L.cout, L.ups, ppb,
                                             d->wg + L.w_off, d->wg + L.b_off);
    if (ga)
        k_conv_bwd_data<<<grid_for(pix * (L.ca + L.cb)), 256, 0, s>>>(d->grad[l], d->w16 + L.w_off, n, h, w, L.ca,
                                                                      L.cb, L.cout, L.ups, ga, gb);
}

// data-gradient convolution of layer l for source part `part` (0: a, 1: b):
// from the layer's pre-activation gradient dz (cout channels) to the part's
// channels at the layer's resolution, zeroed where `gate` (the source's
// activation) is not positive when that is set
cudaError_t dgrad(const mrt_denoiser* d, int l, int part, const bf16* dz, bf16* out, const bf16* gate, int n, int h,
                  int w, cudaStream_t s) {
    const ConvDesc& L = d->layers[l];
    const int cp = part ? L.cb : L.ca;
    ConvArgs ca{dz, nullptr, d->w16, d->zeros, out, n, h, w, L.cout, 0, cp, 0, 0};
    ca.gate = gate;
    const bf16* wt = d->wbt + L.w_off + (part ? size_t(9) * L.cout * L.ca : 0);
    switch (cp) {
    case 32: return launch_conv_ws<32>(ca, wt, d->status, d->sm_count, s);
    case 64: return launch_conv_ws<64>(ca, wt, d->status, d->sm_count, s);
    case 128: return launch_conv_ws<128>(ca, wt, d->status, d->sm_count, s);
    default: return cudaErrorInvalidValue;
    }
}

// weight and bias gradients of layer l from its pre-activation gradient dz
// and its sources
cudaError_t wgrad(const mrt_denoiser* d, int l, const bf16* dz, const bf16* xa, const bf16* xb, int n, int h, int w,
                  cudaStream_t s) {
    const ConvDesc& L = d->layers[l];
    const WgArgs wa{dz, xa, xb, d->wg + L.w_off, d->wg + L.b_off, n, h, w, L.ca, L.cb, L.cout, L.ups};
    if (L.ca + L.cb == 16) return L.cout == 32 ? launch_conv_wgrad<32, 16>(wa, d->status, d->sm_count, s)
                                               : cudaErrorInvalidValue;
    switch (L.cout) {
    case 16: return launch_conv_wgrad<16, 32>(wa, d->status, d->sm_count, s);
    case 32: return launch_conv_wgrad<32, 32>(wa, d->status, d->sm_count, s);
    case 64: return launch_conv_wgrad<64, 32>(wa, d->status, d->sm_count, s);
    case 128: return launch_conv_wgrad<128, 32>(wa, d->status, d->sm_count, s);
    default: return cudaErrorInvalidValue;
    }
}

// Backward of the whole network on the tensor cores, from the loss gradient
// in gz[10]; accumulates the weight and bias gradients into wg.  Returns the
// number of kernels launched through *launches.
cudaError_t backward_tc(mrt_denoiser* d, const bf16* in, int n, int h, int w, cudaStream_t s, int* launches) {
    BwdTable t{};
    for (int l = 1; l < kLayers; ++l) {
        const ConvDesc& L = d->layers[l];
        for (int part = 0; part < (L.cb ? 2 : 1); ++part) {
            const int e = t.parts++;
            t.cp[e] = part ? L.cb : L.ca;
            t.cout[e] = L.cout;
            t.ci0[e] = part ? L.ca : 0;
            t.cin[e] = L.ca + L.cb;
            t.src_off[e] = L.w_off;
            t.dst_off[e] = L.w_off + (part ? size_t(9) * L.cout * L.ca : 0);
        }
    }
    k_bwd_weights<<<304, 256, 0, s>>>(d->w16, d->wbt, t);
    bf16* const* z = d->gz;
    bf16* const* x = d->act;
    const int h1 = h / 2, w1 = w / 2, h2 = h / 4, w2 = w / 4;
    cudaError_t e;
    int k = 1;
#define MRT_TRY(call) do { if ((e = (call)) != cudaSuccess) return e; ++k; } while (0)
    // out (no ReLU: its pre-activation gradient is the loss gradient), d0b
    MRT_TRY(wgrad(d, 10, z[10], x[9], nullptr, n, h, w, s));
    MRT_TRY(dgrad(d, 10, 0, z[10], z[9], x[9], n, h, w, s));
    MRT_TRY(wgrad(d, 9, z[9], x[8], nullptr, n, h, w, s));
    MRT_TRY(dgrad(d, 9, 0, z[9], z[8], x[8], n, h, w, s));
    // d0a: up(d1b) ++ S0
    MRT_TRY(wgrad(d, 8, z[8], x[7], x[1], n, h, w, s));
    MRT_TRY(dgrad(d, 8, 0, z[8], d->up8, nullptr, n, h, w, s));
    k_bwd_unup<<<grid_for(size_t(n) * h1 * w1 * 8), 256, 0, s>>>(d->up8, x[7], z[7], n, h1, w1, 64);
    ++k;
    MRT_TRY(dgrad(d, 8, 1, z[8], d->skip8, nullptr, n, h, w, s));
    // d1b; d1a: up(e2b) ++ S1
    MRT_TRY(wgrad(d, 7, z[7], x[6], nullptr, n, h1, w1, s));
    MRT_TRY(dgrad(d, 7, 0, z[7], z[6], x[6], n, h1, w1, s));
    MRT_TRY(wgrad(d, 6, z[6], x[5], x[3], n, h1, w1, s));
    MRT_TRY(dgrad(d, 6, 0, z[6], d->up6, nullptr, n, h1, w1, s));
    k_bwd_unup<<<grid_for(size_t(n) * h2 * w2 * 16), 256, 0, s>>>(d->up6, x[5], z[5], n, h2, w2, 128);
    ++k;
    MRT_TRY(dgrad(d, 6, 1, z[6], d->skip6, nullptr, n, h1, w1, s));
    // e2b; e2a (input: pooled S1)
    MRT_TRY(wgrad(d, 5, z[5], x[4], nullptr, n, h2, w2, s));
    MRT_TRY(dgrad(d, 5, 0, z[5], z[4], x[4], n, h2, w2, s));
    MRT_TRY(wgrad(d, 4, z[4], d->pool1, nullptr, n, h2, w2, s));
    MRT_TRY(dgrad(d, 4, 0, z[4], d->gp1, nullptr, n, h2, w2, s));
    k_bwd_unpool<<<grid_for(size_t(n) * h1 * w1 * 8), 256, 0, s>>>(d->skip6, d->gp1, x[3], z[3], n, h1, w1, 64);
    ++k;
    // e1b; e1a (input: pooled S0)
    MRT_TRY(wgrad(d, 3, z[3], x[2], nullptr, n, h1, w1, s));
    MRT_TRY(dgrad(d, 3, 0, z[3], z[2], x[2], n, h1, w1, s));
    MRT_TRY(wgrad(d, 2, z[2], d->pool0, nullptr, n, h1, w1, s));
    MRT_TRY(dgrad(d, 2, 0, z[2], d->gp0, nullptr, n, h1, w1, s));
    k_bwd_unpool<<<grid_for(size_t(n) * h * w * 4), 256, 0, s>>>(d->skip8, d->gp0, x[1], z[1], n, h, w, 32);
    ++k;
    // e0b; e0a (input: the features)
    MRT_TRY(wgrad(d, 1, z[1], x[0], nullptr, n, h, w, s));
    MRT_TRY(dgrad(d, 1, 0, z[1], z[0], x[0], n, h, w, s));
    MRT_TRY(wgrad(d, 0, z[0], in, nullptr, n, h, w, s));
#undef MRT_TRY
    *launches = k;
    return cudaGetLastError();
}

} // namespace

extern "C" {

int mrt_cuda_denoiser_create(mrt_ctx* ctx, uint32_t seed, mrt_denoiser** out) {
    if (!ctx || !out) return set_error(ctx, MRT_EINVAL, "denoiser_create: null argument");
    cudaSetDevice(ctx->device);
    mrt_denoiser* d = new (std::nothrow) mrt_denoiser;
    if (!d) return MRT_ENOMEM;
    d->status = ctx->d_status;
    d->sm_count = ctx->sm_count;
    size_t wo = 0;
    for (int l = 0; l < kLayers; ++l) {
        ConvDesc& L = d->layers[l];
        L.ca = kTopo[l][0]; L.cb = kTopo[l][1]; L.cout = kTopo[l][2];
        L.ups = kTopo[l][3]; L.relu = kTopo[l][4]; L.scale = kTopo[l][5];
        L.w_off = wo;
        wo += size_t(L.cout) * 9 * (L.ca + L.cb);
    }
    d->n_w = wo;
    for (int l = 0; l < kLayers; ++l) {
        d->layers[l].b_off = wo;
        wo += d->layers[l].cout;
    }
    d->n_b = wo - d->n_w;
    const size_t total = wo;
    size_t n_up = 0;
    for (int l = 0; l < kLayers; ++l)
        if (d->layers[l].ups) {
            d->up_off[l] = n_up;
            n_up += size_t((d->layers[l].ca + d->layers[l].cb) / 16) * 18 * d->layers[l].cout * 16;
        }
    bool ok = cudaMalloc(&d->w, total * 4) == cudaSuccess && cudaMalloc(&d->wm, total * 4) == cudaSuccess &&
              cudaMalloc(&d->wv, total * 4) == cudaSuccess && cudaMalloc(&d->wg, total * 4) == cudaSuccess &&
              cudaMalloc(&d->w16, d->n_w * 2) == cudaSuccess && cudaMalloc(&d->wtc, d->n_w * 2) == cudaSuccess &&
              cudaMalloc(&d->wbt, d->n_w * 2) == cudaSuccess && cudaMalloc(&d->zeros, 128 * 4) == cudaSuccess &&
              cudaMalloc(&d->wup, std::max<size_t>(n_up, 1) * 2) == cudaSuccess &&
              cudaMalloc(&d->wst, d->n_w * 2) == cudaSuccess &&
              cudaMalloc(&d->loss, 4) == cudaSuccess &&
              cudaMallocHost(&d->h_loss, 4) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        delete d;
        return set_error(ctx, MRT_ENOMEM, "denoiser_create: out of memory");
    }
    // He-uniform initialisation over the fan-in (9 x inputs), zero biases;
    // the output layer's unused channels stay zero
    std::vector<float> w(total, 0.0f);
    uint64_t st = 0xD3A0ull + seed;
    auto next = [&]() {
        uint64_t z = (st += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return double((z ^ (z >> 31)) >> 11) * (1.0 / 9007199254740992.0);
    };
    for (int l = 0; l < kLayers; ++l) {
        const ConvDesc& L = d->layers[l];
        const int cin = L.ca + L.cb;
        const int real_in = l == 0 ? 10 : cin;
        const float a = std::sqrt(6.0f / float(9 * real_in)) * (l == kLayers - 1 ? 0.1f : 1.0f);
        for (int co = 0; co < L.cout; ++co)
            for (int tap = 0; tap < 9; ++tap)
                for (int ci = 0; ci < cin; ++ci) {
                    const bool used = (l != kLayers - 1 || co < 3) && (l != 0 || ci < 10);
                    w[L.w_off + (size_t(co) * 9 + tap) * cin + ci] = used ? float((2.0 * next() - 1.0) * a) : 0.0f;
                }
    }
    std::vector<bf16> w16(d->n_w);
    for (size_t i = 0; i < d->n_w; ++i) w16[i] = __float2bfloat16_rn(w[i]);
    ok = cudaMemcpy(d->w, w.data(), total * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(d->w16, w16.data(), d->n_w * 2, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemset(d->wm, 0, total * 4) == cudaSuccess && cudaMemset(d->wv, 0, total * 4) == cudaSuccess &&
         cudaMemset(d->wg, 0, total * 4) == cudaSuccess && cudaMemset(d->zeros, 0, 128 * 4) == cudaSuccess;
    if (!ok) {
        mrt_cuda_denoiser_destroy(ctx, d);
        return set_error(ctx, MRT_ECUDA, "denoiser_create: upload failed");
    }
    *out = d;
    return MRT_OK;
}

int mrt_cuda_denoiser_destroy(mrt_ctx* ctx, mrt_denoiser* d) {
    if (!ctx || !d) return MRT_EINVAL;
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();
    for (int l = 0; l < kLayers; ++l) { cudaFree(d->act[l]); cudaFree(d->grad[l]); cudaFree(d->gz[l]); }
    void* ps[] = {d->w, d->wm, d->wv, d->wg, d->w16, d->wtc, d->pool0, d->pool1, d->gpool0, d->gpool1, d->gin,
                  d->loss, d->wbt, d->zeros, d->up8, d->up6, d->skip8, d->skip6, d->gp0, d->gp1, d->wup, d->wst};
    for (void* p : ps) cudaFree(p);
    if (d->h_loss) cudaFreeHost(d->h_loss);
    delete d;
    return MRT_OK;
}

int mrt_cuda_denoiser_set_tcgen05(mrt_denoiser* d, int enable) {
    if (!d) return MRT_EINVAL;
    if (enable < 0 || enable > 2) return MRT_EINVAL;
    d->tc_mode = enable;
    return MRT_OK;
}

int mrt_cuda_denoiser_param_count(mrt_denoiser* d, size_t* weights, size_t* biases) {
    if (!d || !weights || !biases) return MRT_EINVAL;
    *weights = d->n_w;
    *biases = d->n_b;
    return MRT_OK;
}

int mrt_cuda_denoiser_features(mrt_ctx* ctx, const mrt_scene* scene, const mrt_gbuffer* gbuffer, const float* color,
                               float scene_diagonal, uint16_t* features, void* stream) {
    if (!ctx || !scene || !gbuffer || !color || !features || !gbuffer->hit_t || scene->kind != 0)
        return set_error(ctx, MRT_EINVAL, "denoiser_features: bad arguments");
    cudaSetDevice(ctx->device);
    const int n = int(gbuffer->width * gbuffer->height);
    k_features<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        scene->dev, color, gbuffer->visibility, gbuffer->hit_t, int(gbuffer->width), int(gbuffer->height),
        scene_diagonal > 0.0f ? 1.0f / scene_diagonal : 1.0f, reinterpret_cast<bf16*>(features));
    if (cudaGetLastError() != cudaSuccess) return set_error(ctx, MRT_ECUDA, "denoiser_features: launch");
    ctx->launches++;
    return MRT_OK;
}

int mrt_cuda_denoiser_infer(mrt_ctx* ctx, mrt_denoiser* d, const uint16_t* features, uint32_t batch, uint32_t width,
                            uint32_t height, float* out, void* stream) {
    if (!ctx || !d || !features || !out || batch == 0) return set_error(ctx, MRT_EINVAL, "denoiser_infer: bad arguments");
    if (width % 4 || height % 4) return set_error(ctx, MRT_EINVAL, "denoiser_infer: width and height must be multiples of 4");
    cudaSetDevice(ctx->device);
    const size_t pix = size_t(batch) * width * height;
    int rc = ensure_acts(ctx, d, pix, false);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int fl = forward_launches(d);
    if (forward(d, reinterpret_cast<const bf16*>(features), int(batch), int(height), int(width), s) != cudaSuccess)
        return set_error(ctx, MRT_ECUDA, "denoiser_infer: launch");
    k_decode<<<grid_for(pix), 256, 0, s>>>(d->act[kLayers - 1], reinterpret_cast<const bf16*>(features), pix, out);
    ctx->launches += fl + 1;  // + decode
    return MRT_OK;
}

int mrt_cuda_denoiser_train_step(mrt_ctx* ctx, mrt_denoiser* d, const uint16_t* features, const float* targets,
                                 uint32_t batch, uint32_t width, uint32_t height, float lr, int apply_update,
                                 float* loss_out, void* stream) {
    if (!ctx || !d || !features || !targets || batch == 0) return set_error(ctx, MRT_EINVAL, "denoiser_train: bad arguments");
    if (width % 4 || height % 4) return set_error(ctx, MRT_EINVAL, "denoiser_train: width and height must be multiples of 4");
    cudaSetDevice(ctx->device);
    const int n = int(batch), h = int(height), w = int(width);
    const size_t pix = size_t(n) * h * w;
    int rc = ensure_acts(ctx, d, pix, true);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const bf16* in = reinterpret_cast<const bf16*>(features);
    const int fl = forward_launches(d);
    if (forward(d, in, n, h, w, s) != cudaSuccess) return set_error(ctx, MRT_ECUDA, "denoiser_train: forward");
    cudaMemsetAsync(d->loss, 0, 4, s);
    if (d->tc_mode == 2) {
        k_l1_loss<<<grid_for(pix), 256, 0, s>>>(d->act[kLayers - 1], in, targets, pix, nullptr, d->gz[kLayers - 1],
                                               d->loss);
        int launched = 0;
        if (backward_tc(d, in, n, h, w, s, &launched) != cudaSuccess)
            return set_error(ctx, MRT_ECUDA, "denoiser_train: backward");
        ctx->launches += fl + 1 + launched;  // + loss
    } else {
        k_l1_loss<<<grid_for(pix), 256, 0, s>>>(d->act[kLayers - 1], in, targets, pix, d->grad[kLayers - 1], nullptr,
                                               d->loss);
        // zero the gradient buffers that accumulate from several consumers
        for (int l = 0; l < kLayers - 1; ++l)
            cudaMemsetAsync(d->grad[l], 0, layer_pixels(pix, d->layers[l].scale) * d->layers[l].cout * 4, s);
        cudaMemsetAsync(d->gpool0, 0, layer_pixels(pix, 1) * 32 * 4, s);
        cudaMemsetAsync(d->gpool1, 0, layer_pixels(pix, 2) * 64 * 4, s);
        cudaMemsetAsync(d->gin, 0, pix * 16 * 4, s);
        bwd_layer(d, 10, d->act[9], nullptr, d->grad[9], nullptr, n, h, w, s);
        bwd_layer(d, 9, d->act[8], nullptr, d->grad[8], nullptr, n, h, w, s);
        bwd_layer(d, 8, d->act[7], d->act[1], d->grad[7], d->grad[1], n, h, w, s);
        bwd_layer(d, 7, d->act[6], nullptr, d->grad[6], nullptr, n, h / 2, w / 2, s);
        bwd_layer(d, 6, d->act[5], d->act[3], d->grad[5], d->grad[3], n, h / 2, w / 2, s);
        bwd_layer(d, 5, d->act[4], nullptr, d->grad[4], nullptr, n, h / 4, w / 4, s);
        bwd_layer(d, 4, d->pool1, nullptr, d->gpool1, nullptr, n, h / 4, w / 4, s);
        k_pool_bwd<<<grid_for(pix / 4 * 64), 256, 0, s>>>(d->gpool1, d->grad[3], n, h / 2, w / 2, 64);
        bwd_layer(d, 3, d->act[2], nullptr, d->grad[2], nullptr, n, h / 2, w / 2, s);
        bwd_layer(d, 2, d->pool0, nullptr, d->gpool0, nullptr, n, h / 2, w / 2, s);
        k_pool_bwd<<<grid_for(pix * 32), 256, 0, s>>>(d->gpool0, d->grad[1], n, h, w, 32);
        bwd_layer(d, 1, d->act[0], nullptr, d->grad[0], nullptr, n, h, w, s);
        bwd_layer(d, 0, in, nullptr, nullptr, nullptr, n, h, w, s);
        ctx->launches += 40;
    }
    if (apply_update) {
        d->step++;
        const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
        const float bc1 = 1.0f - std::pow(b1, float(d->step)), bc2 = 1.0f - std::pow(b2, float(d->step));
        k_adam_bf16<<<grid_for(d->n_w), 256, 0, s>>>(d->w, d->wm, d->wv, d->wg, d->w16, d->n_w, lr, b1, b2, eps, bc1,
                                                     bc2);
        d->relayout_mode = -1;
        k_adam_bf16<<<grid_for(d->n_b), 256, 0, s>>>(d->w + d->n_w, d->wm + d->n_w, d->wv + d->n_w, d->wg + d->n_w,
                                                     nullptr, d->n_b, lr, b1, b2, eps, bc1, bc2);
    }
    if (cudaGetLastError() != cudaSuccess) return set_error(ctx, MRT_ECUDA, "denoiser_train: launch");
    if (loss_out) {
        if (cudaMemcpyAsync(d->h_loss, d->loss, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return set_error(ctx, MRT_ECUDA, "denoiser_train: loss read-back");
        *loss_out = *d->h_loss;
    }
    return MRT_OK;
}

// which = 0: weights then biases (FP32 masters), 1: their gradients;
// set != 0 copies host -> device (and refreshes the BF16 weights)
int mrt_cuda_denoiser_params(mrt_ctx* ctx, mrt_denoiser* d, int which, float* host, size_t count, int set) {
    if (!ctx || !d || !host || which < 0 || which > 1 || count != d->n_w + d->n_b)
        return set_error(ctx, MRT_EINVAL, "denoiser_params: bad arguments");
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();
    float* p = which == 0 ? d->w : d->wg;
    if (!set) return cudaMemcpy(host, p, count * 4, cudaMemcpyDeviceToHost) == cudaSuccess ? MRT_OK : MRT_ECUDA;
    if (cudaMemcpy(p, host, count * 4, cudaMemcpyHostToDevice) != cudaSuccess) return MRT_ECUDA;
    if (which == 0) {
        std::vector<bf16> w16(d->n_w);
        for (size_t i = 0; i < d->n_w; ++i) w16[i] = __float2bfloat16_rn(host[i]);
        cudaMemcpy(d->w16, w16.data(), d->n_w * 2, cudaMemcpyHostToDevice);
        d->relayout_mode = -1;
    }
    return MRT_OK;
}

} // extern "C"
