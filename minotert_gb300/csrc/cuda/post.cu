// Post-processing after the path tracer: the joint bilateral filter, the
// six tonemappers and temporal reprojection, with their C ABI.
//
//   bilateral    src/gpu/denoise/bilateral.comp:23-76 (params
//                src/gfx/modules/denoiser.ixx:20-31)
//   tonemappers  src/gpu/tonemap/{linear,reinhard,hable,aces,uchimura,amd}.comp,
//                src/gpu/util.glsl:13-18 (sRGB), tonemapper.ixx:20-57
//   reprojection new: uses the motion vectors of primaryRay.comp:73-75
//
// Arithmetic is explicitly rounded (fm/fa/fs/fd) in the GLSL's order and the
// bilateral weights use exp_cw (common.cuh), so the CPU oracle reproduces
// the filter and reprojection bit for bit; the tonemap curves keep CUDA's
// powf / expf and agree with the oracle to within one 8-bit step.
#include <atomic>
#include <cmath>
#include <cstring>
#include <vector>

#include "internal.hpp"

namespace mrt {
int set_error(mrt_ctx* ctx, int code, const char* msg);
FrameParams make_frame_params(const mrt_camera_consts* c, uint32_t w, uint32_t h);
}

using namespace mrt;

namespace {

cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }

// ------------------------------------------------------------------ bilateral

constexpr int kMaxCols = 2 * MRT_BILATERAL_MAX_RADIUS + 1;
constexpr int kMaxTaps = 1900;  // > taps of radius 24 (1,849)
constexpr int kBilTile = 16;    // 16x16 pixels per block

// Tap table of the circular kernel, in the reference's loop order: column
// dx = c - radius holds the rows dy = -pt + k, k = 0..count-1, with
// pt = sqrt(r^2 - dx^2); a row between whole rows r0 + k and r0 + k + 1 at
// fraction fr (the same for the whole column).
struct BilateralTable {
    int radius, ncols;
    float near_plane, inv_thr_sq2, inv_thr_sqrt2pi;
    uint32_t frame, dither;
    int first[kMaxCols], count[kMaxCols], r0[kMaxCols];
    float fr[kMaxCols];
    float blur[kMaxTaps];  // exp(-|d|^2 / (2 sigma^2)) / (2 pi sigma^2)
};

// Builds the table on the host (IEEE float, no contraction).  Returns false
// when the radius is out of range.
bool make_table(const mrt_bilateral_params& p, BilateralTable& t) {
    const float radius = std::round(p.k_sigma * p.sigma);
    if (!(radius >= 0.0f) || radius > float(MRT_BILATERAL_MAX_RADIUS)) return false;
    const float rad_q = radius * radius;
    const float inv_sq2 = 0.5f / (p.sigma * p.sigma);
    const float inv_sq2pi = 0.31830988618379067154f * inv_sq2;
    t.radius = int(radius);
    t.ncols = 2 * t.radius + 1;
    t.near_plane = p.near_plane;
    t.inv_thr_sq2 = 0.5f / (p.threshold * p.threshold);
    t.inv_thr_sqrt2pi = 0.39894228040143267794f / p.threshold;
    t.frame = p.frame_counter;
    t.dither = p.dither;
    int n = 0;
    for (int c = 0; c < t.ncols; ++c) {
        const float dx = float(c - t.radius);
        const float pt = std::sqrt(rad_q - dx * dx);
        const float start = -pt;
        const float f0 = std::floor(start);
        t.first[c] = n;
        t.r0[c] = int(f0);
        t.fr[c] = start - f0;
        int k = 0;
        for (float dy = start; dy <= pt; dy += 1.0f, ++k) {
            if (n >= kMaxTaps) return false;
            t.blur[n++] = std::exp(-(dx * dx + dy * dy) * inv_sq2) * inv_sq2pi;
        }
        t.count[c] = k;
    }
    return true;
}

// One block filters a 16x16 tile from a shared-memory window of the colour,
// depth and normal planes covering every tap (radius columns either side,
// radius rows above, radius + 1 below for the bilinear row pair).  Every tap
// of column c interpolates between two whole rows at the column's fraction
// fr[c], so the interpolated sample at (row s, column x) -- depth turned
// into near / depth, normal and colour -- is the same for all the up to
// 2r + 1 threads of the column whose taps land on it.  Each column's samples
// are therefore computed once into a second shared-memory window
// (16 columns x 16 + count - 1 rows, two float4 per sample) and the taps
// read them:
// the same operations on the same operands as a per-tap evaluation, so the
// same bits, for a fraction of the arithmetic.  kExpChecked: the weights'
// exponential keeps its range handling (only needed when the argument can
// leave (-87, 88], i.e. 0.5 / threshold^2 > 88).
template <bool kExpChecked>
__global__ void __launch_bounds__(kBilTile * kBilTile)
k_bilateral(BilateralTable T, const float* __restrict__ color, const uint16_t* __restrict__ depth,
            const ushort4* __restrict__ normal, uint32_t W, uint32_t H, float* __restrict__ out) {
    extern __shared__ float sm[];
    const int r = T.radius;
    const int tw = kBilTile + 2 * r, th = kBilTile + 2 * r + 1, plane = tw * th;
    const int splane = kBilTile * (kBilTile + 2 * r);
    float *cr = sm, *cg = sm + plane, *cb = sm + 2 * plane, *zz = sm + 3 * plane;
    float *nx = sm + 4 * plane, *ny = sm + 5 * plane, *nz = sm + 6 * plane;
    // samples: (near / depth, normal) and (colour, 0), 16-byte aligned
    float4* sa = reinterpret_cast<float4*>(sm + ((7 * plane + 3) & ~3));
    float4* sb = sa + splane;
    const int bx = int(blockIdx.x) * kBilTile - r, by = int(blockIdx.y) * kBilTile - r;
    for (int i = threadIdx.x; i < plane; i += blockDim.x) {
        const int gx = min(max(bx + i % tw, 0), int(W) - 1), gy = min(max(by + i / tw, 0), int(H) - 1);
        const size_t p = size_t(gy) * W + gx;
        cr[i] = __ldg(color + 3 * p);
        cg[i] = __ldg(color + 3 * p + 1);
        cb[i] = __ldg(color + 3 * p + 2);
        zz[i] = h2f(__ldg(depth + p));
        const ushort4 nv = __ldg(normal + p);
        nx[i] = h2f(nv.x);
        ny[i] = h2f(nv.y);
        nz[i] = h2f(nv.z);
    }
    __syncthreads();
    const int tx = threadIdx.x % kBilTile, ty = threadIdx.x / kBilTile;
    const uint32_t x = blockIdx.x * kBilTile + tx, y = blockIdx.y * kBilTile + ty;
    const bool inside = x < W && y < H;
    const int ic = (ty + r) * tw + tx + r;
    const float cz = zz[ic];
    f3 res{cr[ic], cg[ic], cb[ic]};
    const bool filt = inside && !(cz < 0.0f);  // (all threads build the samples)
    const f3 cn{nx[ic], ny[ic], nz[ic]};
    const float ncz = filt ? fd(T.near_plane, cz) : 0.0f;
    float zb = 0.0f, ar = 0.0f, ag = 0.0f, ab = 0.0f;
    for (int c = 0; c < T.ncols; ++c) {
        const float fr = T.fr[c], gr = fs(1.0f, fr);
        const int t0 = T.first[c], cnt = T.count[c];
        // sample (s, xx): rows r + r0 + s and + 1 of tile column xx + c;
        // thread (tx, ty)'s tap k reads sample (ty + k, tx)
        const int ns = (kBilTile + cnt - 1) * kBilTile, base = (r + T.r0[c]) * tw + c;
        __syncthreads();  // the previous column's samples have been read
        for (int i = threadIdx.x; i < ns; i += blockDim.x) {
            const int ia = base + (i / kBilTile) * tw + i % kBilTile, ib = ia + tw;
            sa[i] = make_float4(fd(T.near_plane, fa(fm(zz[ia], gr), fm(zz[ib], fr))),
                                fa(fm(nx[ia], gr), fm(nx[ib], fr)), fa(fm(ny[ia], gr), fm(ny[ib], fr)),
                                fa(fm(nz[ia], gr), fm(nz[ib], fr)));
            sb[i] = make_float4(fa(fm(cr[ia], gr), fm(cr[ib], fr)), fa(fm(cg[ia], gr), fm(cg[ib], fr)),
                                fa(fm(cb[ia], gr), fm(cb[ib], fr)), 0.0f);
        }
        __syncthreads();
        if (filt) {
            // a warp's 32 threads read 32 consecutive samples: conflict-free
            const float4* pa = sa + ty * kBilTile + tx;
            const float4* pb = sb + ty * kBilTile + tx;
            const float* blur = T.blur + t0;
#pragma unroll 2
            for (int k = 0; k < cnt; ++k) {
                const float4 a = pa[k * kBilTile], b = pb[k * kBilTile];
                const float dz = fm(fs(a.x, ncz), 100.0f);
                const float dn = dot_rn(f3{a.y, a.z, a.w}, cn);
                const float arg = fm(fclamp(fs(dn, fm(dz, dz)), 0.0f, 1.0f), T.inv_thr_sq2);
                const float e = kExpChecked ? exp_cw(arg) : exp_cw_core(arg);
                const float df = fm(fm(e, T.inv_thr_sqrt2pi), blur[k]);
                zb = fa(zb, df);
                ar = fa(ar, fm(df, b.x));
                ag = fa(ag, fm(df, b.y));
                ab = fa(ab, fm(df, b.z));
            }
        }
    }
    if (!inside) return;
    if (filt) res = f3{fd(ar, zb), fd(ag, zb), fd(ab, zb)};
    if (T.dither) {
        uint32_t seed = x * 709u + y * 1153u + T.frame * 1361u;
        const float nz0 = fm(random_float(seed), 0.005f);
        res = add_rn(res, f3s(nz0));
    }
    const size_t p = size_t(y) * W + x;
    out[3 * p] = res.x;
    out[3 * p + 1] = res.y;
    out[3 * p + 2] = res.z;
}

// Shared memory of k_bilateral for radius r: the texel window (seven
// planes, padded to 16 bytes) and the samples of one column (two float4).
constexpr size_t bilateral_smem(int r) {
    return (size_t((7 * (kBilTile + 2 * r) * (kBilTile + 2 * r + 1) + 3) & ~3) +
            size_t(8) * kBilTile * (kBilTile + 2 * r)) * sizeof(float);
}

// ------------------------------------------------------------------- tonemap

struct ToneConsts {
    uint32_t mode;
    float exposure, reinhard_max;
    float u[6];                 // uchimura P a m l c b
    float contrast, shoulder, b, c;  // AMD curve (b, c precomputed)
};

MRT_DEV float srgb1(float c) {
    return c < 0.0031308f ? fm(12.92f, c) : fs(fm(1.055f, powf(c, fd(1.0f, 2.4f))), 0.055f);
}

MRT_DEV float hable_op(float x) {
    const float A = 0.15f, B = 0.50f, C = 0.10f, D = 0.20f, E = 0.02f, F = 0.30f;
    return fs(fd(fa(fm(x, fa(fm(A, x), fm(C, B))), fm(D, E)), fa(fm(x, fa(fm(A, x), B)), fm(D, F))), fd(E, F));
}

MRT_DEV f3 aces_fit(f3 v) {
    // v * ACESInputMat: component j = dot(v, row j of the table)
    const f3 i0{0.59719f, 0.35458f, 0.04823f}, i1{0.07600f, 0.90834f, 0.01566f}, i2{0.02840f, 0.13383f, 0.83777f};
    const f3 o0{1.60475f, -0.53108f, -0.07367f}, o1{-0.10208f, 1.10813f, -0.00605f},
        o2{-0.00327f, -0.07276f, 1.07602f};
    f3 c{dot_rn(v, i0), dot_rn(v, i1), dot_rn(v, i2)};
    auto rrt = [](float x) {
        const float a = fs(fm(x, fa(x, 0.0245786f)), 0.000090537f);
        const float b = fa(fm(x, fa(fm(0.983729f, x), 0.4329510f)), 0.238081f);
        return fd(a, b);
    };
    c = f3{rrt(c.x), rrt(c.y), rrt(c.z)};
    c = f3{dot_rn(c, o0), dot_rn(c, o1), dot_rn(c, o2)};
    return f3{fclamp(c.x, 0.0f, 1.0f), fclamp(c.y, 0.0f, 1.0f), fclamp(c.z, 0.0f, 1.0f)};
}

MRT_DEV float uchimura1(float x, const float* u) {
    const float P = u[0], a = u[1], m = u[2], l = u[3], c = u[4], b = u[5];
    const float l0 = fd(fm(fs(P, m), l), a);
    const float S0 = fa(m, l0);
    const float S1 = fa(m, fm(a, l0));
    const float C2 = fd(fm(a, P), fs(P, S1));
    const float CP = fd(-C2, P);
    const float t = fclamp(fd(fs(x, 0.0f), fs(m, 0.0f)), 0.0f, 1.0f);
    const float w0 = fs(1.0f, fm(fm(t, t), fs(3.0f, fm(2.0f, t))));
    const float w2 = x < fa(m, l0) ? 0.0f : 1.0f;
    const float w1 = fs(fs(1.0f, w0), w2);
    const float T = fa(fm(m, powf(fd(x, m), c)), b);
    const float S = fs(P, fm(fs(P, S1), expf(fm(CP, fs(x, S0)))));
    const float L = fa(m, fm(a, fs(x, m)));
    return fa(fa(fm(T, w0), fm(L, w1)), fm(S, w2));
}

MRT_DEV f3 amd_tone(f3 col, const ToneConsts& k) {
    float peak = fmaxf(col.x, fmaxf(col.y, col.z));
    peak = fmaxf(1e-6f, peak);
    f3 ratio = div3s(col, peak);
    const float z = powf(peak, k.contrast);
    peak = fd(z, fa(fm(powf(z, k.shoulder), k.b), k.c));
    const float sat = k.contrast, cross = fm(k.contrast, 16.0f);
    const float e = fd(sat, cross);
    ratio = f3{powf(fabsf(ratio.x), e), powf(fabsf(ratio.y), e), powf(fabsf(ratio.z), e)};
    const float mx = powf(peak, 4.0f);
    const float g = fs(1.0f, mx);
    ratio = f3{fa(fm(ratio.x, g), fm(1.0f, mx)), fa(fm(ratio.y, g), fm(1.0f, mx)), fa(fm(ratio.z, g), fm(1.0f, mx))};
    ratio = f3{powf(fabsf(ratio.x), cross), powf(fabsf(ratio.y), cross), powf(fabsf(ratio.z), cross)};
    return scale_rn(ratio, peak);
}

MRT_DEV uint32_t unorm8(float v) { return __float2uint_rn(fm(fclamp(v, 0.0f, 1.0f), 255.0f)); }

__global__ void __launch_bounds__(256) k_tonemap(ToneConsts k, const float* __restrict__ color, uint32_t n,
                                                 uchar4* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    f3 c = scale_rn(f3{__ldg(color + 3 * size_t(i)), __ldg(color + 3 * size_t(i) + 1),
                       __ldg(color + 3 * size_t(i) + 2)},
                    k.exposure);
    switch (k.mode) {
    case MRT_TONEMAP_REINHARD: {
        const float mw = fm(k.reinhard_max, k.reinhard_max);
        auto rh = [mw](float v) { return fd(fm(v, fa(1.0f, fd(v, mw))), fa(1.0f, v)); };
        c = f3{rh(c.x), rh(c.y), rh(c.z)};
        break;
    }
    case MRT_TONEMAP_HABLE: {
        const float w = hable_op(11.2f);
        c = f3{fd(hable_op(fm(2.0f, c.x)), w), fd(hable_op(fm(2.0f, c.y)), w), fd(hable_op(fm(2.0f, c.z)), w)};
        break;
    }
    case MRT_TONEMAP_ACES: c = aces_fit(c); break;
    case MRT_TONEMAP_UCHIMURA: c = f3{uchimura1(c.x, k.u), uchimura1(c.y, k.u), uchimura1(c.z, k.u)}; break;
    case MRT_TONEMAP_AMD: c = amd_tone(c, k); break;
    default: break;  // linear
    }
    out[i] = make_uchar4(uint8_t(unorm8(srgb1(c.x))), uint8_t(unorm8(srgb1(c.y))), uint8_t(unorm8(srgb1(c.z))),
                         255);
}

// AMD curve coefficients b and c (amd.comp ColToneB / ColToneC), on the host.
void amd_coefficients(const float* p, float& b, float& c) {
    const float hdr = p[0], contrast = p[1], shoulder = p[2], mid_in = p[3], mid_out = p[4];
    const float a = std::pow(mid_in, contrast);
    const float hs = std::pow(hdr, contrast * shoulder);
    const float ms = std::pow(mid_in, contrast * shoulder);
    const float hc = std::pow(hdr, contrast);
    const float num = hs * a - hc * ms * mid_out;
    const float den = hs * mid_out - ms * mid_out;
    b = -((-a + (mid_out * num) / den) / (ms * mid_out));
    c = num / den;
}

// -------------------------------------------------------------- reprojection

struct ReprojConsts {
    float max_history, normal_cos, depth_rel, near_plane;
};

__global__ void __launch_bounds__(256)
k_reproject(FrameParams fp, ReprojConsts k, mrt_gbuffer cur, mrt_gbuffer prev, const float* __restrict__ sample,
            const float* __restrict__ hist, const float* __restrict__ hist_len, float* __restrict__ out,
            float* __restrict__ out_len) {
    const uint32_t W = fp.width, H = fp.height;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W * H) return;
    const uint32_t x = i % W, y = i / W;
    const f3 s{sample[3 * size_t(i)], sample[3 * size_t(i) + 1], sample[3 * size_t(i) + 2]};
    f3 res = s;
    float len = 1.0f;
    if (cur.visibility[i] != kMiss) {
        const ushort2 mv = reinterpret_cast<const ushort2*>(cur.motion)[i];
        const float px = fs(fa(float(x), 0.5f), fm(h2f(mv.x), 0.5f));
        const float py = fa(fa(float(y), 0.5f), fm(h2f(mv.y), 0.5f));
        f3 o, d;
        primary_ray(fp, x, y, o, d);
        const f3 p = ray_at(o, d, cur.hit_t[i]);
        float q[4];
        matvec_rn(fp.ppv, p.x, p.y, p.z, 1.0f, q);
        const float exp_lin = q[3];
        const ushort4 nh = reinterpret_cast<const ushort4*>(cur.normal)[i];
        const f3 cn{h2f(nh.x), h2f(nh.y), h2f(nh.z)};
        const float fx = fs(px, 0.5f), fy = fs(py, 0.5f);
        const float x0 = floorf(fx), y0 = floorf(fy);
        if (exp_lin > 0.0f && x0 >= -1.0f && x0 <= float(W) - 1.0f && y0 >= -1.0f && y0 <= float(H) - 1.0f) {
            const float wx = fs(fx, x0), wy = fs(fy, y0);
            const float gx = fs(1.0f, wx), gy = fs(1.0f, wy);
            const float ws[4] = {fm(gx, gy), fm(wx, gy), fm(gx, wy), fm(wx, wy)};
            const float tol = fm(k.depth_rel, exp_lin);
            float sw = 0.0f, hl = 0.0f;
            f3 h{0.0f, 0.0f, 0.0f};
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const int tx = int(x0) + (t & 1), ty = int(y0) + (t >> 1);
                if (tx < 0 || ty < 0 || tx >= int(W) || ty >= int(H) || !(ws[t] > 0.0f)) continue;
                const size_t j = size_t(ty) * W + tx;
                if (prev.visibility[j] == kMiss) continue;
                const ushort4 pn = reinterpret_cast<const ushort4*>(prev.normal)[j];
                if (!(dot_rn(f3{h2f(pn.x), h2f(pn.y), h2f(pn.z)}, cn) >= k.normal_cos)) continue;
                const float tl = fd(k.near_plane, h2f(prev.depth[j]));
                if (!(fabsf(fs(tl, exp_lin)) <= tol)) continue;
                sw = fa(sw, ws[t]);
                h = add_rn(h, scale_rn(f3{hist[3 * j], hist[3 * j + 1], hist[3 * j + 2]}, ws[t]));
                hl = fa(hl, fm(hist_len[j], ws[t]));
            }
            if (sw > 0.0f) {
                h = div3s(h, sw);
                len = fminf(fa(fd(hl, sw), 1.0f), k.max_history);
                const float a = fd(1.0f, len);
                res = add_rn(h, scale_rn(sub_rn(s, h), a));
            }
        }
    }
    out[3 * size_t(i)] = res.x;
    out[3 * size_t(i) + 1] = res.y;
    out[3 * size_t(i) + 2] = res.z;
    out_len[i] = len;
}

}  // namespace

extern "C" {

void mrt_bilateral_defaults(mrt_bilateral_params* p) {
    if (!p) return;
    p->sigma = 5.0f;
    p->k_sigma = 2.0f;
    p->threshold = 0.12f;
    p->near_plane = 1.0f;
    p->frame_counter = 0;
    p->dither = 1;
}

int mrt_cuda_bilateral(mrt_ctx* ctx, const mrt_gbuffer* g, const float* color, const mrt_bilateral_params* params,
                       float* out, void* stream) {
    if (!ctx || !g || !color || !params || !out) return set_error(ctx, MRT_EINVAL, "bilateral: null argument");
    if (!g->depth || !g->normal || g->width == 0 || g->height == 0)
        return set_error(ctx, MRT_EINVAL, "bilateral: gbuffer needs depth and normal");
    if (!(params->sigma > 0.0f) || !(params->threshold > 0.0f) || !(params->near_plane > 0.0f))
        return set_error(ctx, MRT_EINVAL, "bilateral: sigma, threshold and near_plane must be positive");
    if (color == out) return set_error(ctx, MRT_EINVAL, "bilateral: out aliases color");
    static thread_local BilateralTable table;
    if (!make_table(*params, table)) return set_error(ctx, MRT_ERANGE, "bilateral: radius above the maximum");
    cudaSetDevice(ctx->device);
    const size_t smem = bilateral_smem(table.radius);
    // the exponential's argument lies in [0, 0.5 / threshold^2]
    const bool checked = !(table.inv_thr_sq2 <= 88.0f);
    // the shared-memory limit is raised to the largest radius's need once per
    // device and kernel form
    static std::atomic<uint64_t> configured[2];
    const uint64_t bit = uint64_t(1) << (ctx->device & 63);
    if ((configured[checked].load() & bit) == 0) {
        const int most = int(bilateral_smem(MRT_BILATERAL_MAX_RADIUS));
        const cudaError_t e = checked
            ? cudaFuncSetAttribute(k_bilateral<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, most)
            : cudaFuncSetAttribute(k_bilateral<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
        if (e != cudaSuccess) return set_error(ctx, MRT_ECUDA, "bilateral: shared memory size");
        configured[checked].fetch_or(bit);
    }
    const dim3 grid((g->width + kBilTile - 1) / kBilTile, (g->height + kBilTile - 1) / kBilTile);
    const ushort4* nrm = reinterpret_cast<const ushort4*>(g->normal);
    if (checked)
        k_bilateral<true><<<grid, kBilTile * kBilTile, smem, as_stream(stream)>>>(table, color, g->depth, nrm,
                                                                                 g->width, g->height, out);
    else
        k_bilateral<false><<<grid, kBilTile * kBilTile, smem, as_stream(stream)>>>(table, color, g->depth, nrm,
                                                                                  g->width, g->height, out);
    if (cudaGetLastError() != cudaSuccess) return set_error(ctx, MRT_ECUDA, "bilateral: launch");
    ctx->launches++;
    return MRT_OK;
}

void mrt_tonemap_defaults(mrt_tonemap_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->mode = MRT_TONEMAP_AMD;
    p->exposure = 1.0f;
    p->reinhard_max = 8.0f;
    const float u[6] = {1.0f, 1.0f, 0.22f, 0.4f, 1.33f, 0.0f};
    const float a[5] = {16.0f, 2.0f, 1.0f, 0.18f, 0.18f};
    std::memcpy(p->uchimura, u, sizeof(u));
    std::memcpy(p->amd, a, sizeof(a));
}

int mrt_cuda_tonemap(mrt_ctx* ctx, const float* color, uint32_t width, uint32_t height,
                     const mrt_tonemap_params* params, uint8_t* out, void* stream) {
    if (!ctx || !color || !params || !out) return set_error(ctx, MRT_EINVAL, "tonemap: null argument");
    if (params->mode > MRT_TONEMAP_AMD) return set_error(ctx, MRT_EINVAL, "tonemap: unknown mode");
    const uint64_t n = uint64_t(width) * height;
    if (n == 0) return MRT_OK;
    if (n > 0xFFFFFFFFull) return set_error(ctx, MRT_ERANGE, "tonemap: image too large");
    ToneConsts k{};
    k.mode = params->mode;
    k.exposure = params->exposure;
    k.reinhard_max = params->reinhard_max;
    std::memcpy(k.u, params->uchimura, sizeof(k.u));
    k.contrast = params->amd[1];
    k.shoulder = params->amd[2];
    amd_coefficients(params->amd, k.b, k.c);
    cudaSetDevice(ctx->device);
    k_tonemap<<<uint32_t((n + 255) / 256), 256, 0, as_stream(stream)>>>(k, color, uint32_t(n),
                                                                         reinterpret_cast<uchar4*>(out));
    if (cudaGetLastError() != cudaSuccess) return set_error(ctx, MRT_ECUDA, "tonemap: launch");
    ctx->launches++;
    return MRT_OK;
}

int mrt_cuda_reproject(mrt_ctx* ctx, const mrt_gbuffer* cur, const mrt_gbuffer* prev, const mrt_camera_consts* consts,
                       const float* sample, const float* hist, const float* hist_len,
                       const mrt_reproject_params* params, float* out, float* out_len, void* stream) {
    if (!ctx || !cur || !prev || !consts || !sample || !hist || !hist_len || !params || !out || !out_len)
        return set_error(ctx, MRT_EINVAL, "reproject: null argument");
    if (cur->width != prev->width || cur->height != prev->height || cur->width == 0 || cur->height == 0)
        return set_error(ctx, MRT_EINVAL, "reproject: g-buffer sizes differ");
    if (!cur->visibility || !cur->hit_t || !cur->normal || !cur->motion || !prev->visibility || !prev->depth ||
        !prev->normal)
        return set_error(ctx, MRT_EINVAL, "reproject: g-buffer planes missing");
    if (out == hist || out_len == hist_len) return set_error(ctx, MRT_EINVAL, "reproject: output aliases history");
    if (!(params->max_history >= 1.0f)) return set_error(ctx, MRT_EINVAL, "reproject: max_history < 1");
    const uint64_t n = uint64_t(cur->width) * cur->height;
    if (n > 0xFFFFFFFFull) return set_error(ctx, MRT_ERANGE, "reproject: image too large");
    cudaSetDevice(ctx->device);
    const FrameParams fp = make_frame_params(consts, cur->width, cur->height);
    ReprojConsts k{params->max_history, params->normal_cos, params->depth_rel, consts->projection[3 * 4 + 2]};
    k_reproject<<<uint32_t((n + 255) / 256), 256, 0, as_stream(stream)>>>(fp, k, *cur, *prev, sample, hist, hist_len,
                                                                           out, out_len);
    if (cudaGetLastError() != cudaSuccess) return set_error(ctx, MRT_ECUDA, "reproject: launch");
    ctx->launches++;
    return MRT_OK;
}

}  // extern "C"
