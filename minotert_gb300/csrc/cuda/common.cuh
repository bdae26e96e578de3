// Device-side helpers shared by the ray-tracing kernels.
//
// Arithmetic that must reproduce the CPU oracle bit for bit is written with
// explicitly rounded intrinsics (__fmul_rn / __fadd_rn never contract into
// an FMA; fmaf is a single correctly rounded FMA on both sides), so the
// compiler's default FMA contraction cannot change a result.
#pragma once

#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "mrt_cuda.h"

#define MRT_DEV __device__ __forceinline__

namespace mrt {

constexpr uint32_t kMiss = 0xFFFFFFFFu;

struct f3 { float x, y, z; };

MRT_DEV f3 mk(float x, float y, float z) { return f3{x, y, z}; }
MRT_DEV f3 sub_rn(f3 a, f3 b) { return f3{__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)}; }
MRT_DEV f3 add_rn(f3 a, f3 b) { return f3{__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)}; }
MRT_DEV f3 scale_rn(f3 a, float s) { return f3{__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s)}; }
MRT_DEV f3 mul_rn(f3 a, f3 b) { return f3{__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y), __fmul_rn(a.z, b.z)}; }
// minote.math dot: ((0 + a.x*b.x) + a.y*b.y) + a.z*b.z, no contraction
MRT_DEV float dot_rn(f3 a, f3 b) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
// v / length(v) with IEEE sqrt and division
MRT_DEV f3 normalize_rn(f3 v) {
    float len = __fsqrt_rn(dot_rn(v, v));
    return f3{__fdiv_rn(v.x, len), __fdiv_rn(v.y, len), __fdiv_rn(v.z, len)};
}

// column-major 4x4 matrix times vec4 as a sequential non-FMA dot per row
// (minote.math operator*(mat, vec), math.ixx:699-706)
MRT_DEV void matvec_rn(const float* m, float x, float y, float z, float w, float out[4]) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        float acc = __fmul_rn(m[0 * 4 + r], x);
        acc = __fadd_rn(acc, __fmul_rn(m[1 * 4 + r], y));
        acc = __fadd_rn(acc, __fmul_rn(m[2 * 4 + r], z));
        acc = __fadd_rn(acc, __fmul_rn(m[3 * 4 + r], w));
        out[r] = acc;
    }
}

// PCG hash step (random.glsl:22-27)
MRT_DEV uint32_t pcg(uint32_t& v) {
    uint32_t state = v * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    v = (word >> 22u) ^ word;
    return v;
}
// 24-bit float in [0,1) (random.glsl:29-31)
MRT_DEV float random_float(uint32_t& s) { return float(pcg(s) & 0xFFFFFFu) * (1.0f / 16777216.0f); }
// Cranley-Patterson rotation fract(r + rot) (secondaryRays.comp:60-62)
MRT_DEV float rotated_random(uint32_t& s, float rot) {
    float x = __fadd_rn(random_float(s), rot);
    return __fsub_rn(x, floorf(x));
}
// sin and cos of a binary32 angle evaluated in binary64 and rounded once
// to binary32 -- the CPU oracle's evaluation.  Out of line so the default
// (sincosf) path of the register-capped kernels does not carry it.
static __device__ __noinline__ void sincos_binary64(float a, float* sn, float* cs) {
    *sn = float(sin(double(a)));
    *cs = float(cos(double(a)));
}

// uniform point on the unit sphere from (x, y) in [-1,1)^2 (random.glsl:10-19);
// exact: sin/cos through sincos_binary64 (mrt_trace_params.exact_trig)
MRT_DEV f3 random_sphere_point(float rx, float ry, uint32_t exact = 0u) {
    const float Pi = 3.14159265359f;
    float ang1 = __fmul_rn(__fadd_rn(rx, 1.0f), Pi);
    float u = ry;
    float u2 = __fmul_rn(u, u);
    float s = __fsqrt_rn(__fsub_rn(1.0f, u2));
    float sn, cs;
    if (exact) sincos_binary64(ang1, &sn, &cs);
    else sincosf(ang1, &sn, &cs);
    return f3{__fmul_rn(s, cs), __fmul_rn(s, sn), u};
}

// Self-intersection-free origin offset along the geometric normal:
// Waechter & Binder, "A Fast and Robust Method for Avoiding
// Self-Intersection", Ray Tracing Gems (2019), ch. 6.
MRT_DEV float offset_axis(float p, float n) {
    const float kOrigin = 1.0f / 32.0f, kFloatScale = 1.0f / 65536.0f, kIntScale = 256.0f;
    int of = __float2int_rz(__fmul_rn(kIntScale, n));
    float pi = __int_as_float(__float_as_int(p) + (p < 0.0f ? -of : of));
    return fabsf(p) < kOrigin ? fmaf(kFloatScale, n, p) : pi;
}
constexpr float kInvPi = 0.318309886183790671538f;  // 1 / pi, Lambertian BRDF normalisation

MRT_DEV f3 offset_ray(f3 p, f3 n) { return f3{offset_axis(p.x, n.x), offset_axis(p.y, n.y), offset_axis(p.z, n.z)}; }

// e^x reproducible bit for bit on the CPU: Cody-Waite reduction
// x = n ln2 + r (n = rint(x log2 e), ln2 split into a 16-bit head and a
// tail so n * head is exact), the degree-7 Taylor polynomial of e^r on
// |r| <= ln2/2 in Horner form with correctly rounded FMAs (truncation
// r^8/8! < 6e-9 relative), then an exact scale by 2^n.  Results below
// 2^-126 flush to 0.  Used where an expression cancels and would turn
// a last-bit difference between two exp implementations into a visible one.
// exp_cw without its range handling: equal to exp_cw for -87 < x <= 88
// (there n = rint(x / ln 2) lies in [-125, 127], so the scale is a normal
// power of two).
MRT_DEV float exp_cw_core(float x) {
    const float n = rintf(__fmul_rn(x, 1.44269502f));
    float r = fmaf(-n, 0.693145752f, x);
    r = fmaf(-n, 1.42860677e-6f, r);
    float p = 1.98412701e-4f;
    p = fmaf(p, r, 1.38888892e-3f);
    p = fmaf(p, r, 8.33333377e-3f);
    p = fmaf(p, r, 4.16666679e-2f);
    p = fmaf(p, r, 1.66666672e-1f);
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    return __fmul_rn(p, __int_as_float((int(n) + 127) << 23));
}

MRT_DEV float exp_cw(float x) {
    if (!(x > -87.0f)) return x != x ? x : 0.0f;
    if (x > 88.0f) return __int_as_float(0x7F800000);
    const float n = rintf(__fmul_rn(x, 1.44269502f));
    float r = fmaf(-n, 0.693145752f, x);
    r = fmaf(-n, 1.42860677e-6f, r);
    float p = 1.98412701e-4f;           // 1/7!
    p = fmaf(p, r, 1.38888892e-3f);     // 1/6!
    p = fmaf(p, r, 8.33333377e-3f);     // 1/5!
    p = fmaf(p, r, 4.16666679e-2f);     // 1/4!
    p = fmaf(p, r, 1.66666672e-1f);     // 1/3!
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    const int e = int(n);
    if (e < -126) return 0.0f;
    return __fmul_rn(p, __int_as_float((e + 127) << 23));
}

MRT_DEV uint16_t f2h(float x) { return __half_as_ushort(__float2half_rn(x)); }
MRT_DEV float h2f(uint16_t x) { return __half2float(__ushort_as_half(x)); }

MRT_DEV uint32_t lane_id() { return threadIdx.x & 31u; }

} // namespace mrt
