// Sky / atmosphere: LUT addressing, the participating-medium model, the
// single-scattering ray march and the miss shader skyColor().
//
// Restates the Hillaire (2020) "scalable sky and atmosphere" technique as
// the reference uses it: src/gpu/sky/sky.glsl (medium, march, sun disc),
// src/gpu/sky/skyAccess.glsl (LUT parameterisations) and
// src/gpu/secondaryRays.comp:36-58 (skyColor).  Every +,-,*,/ is an
// explicitly rounded intrinsic so that the FMA contraction of the
// translation unit that includes this header cannot change a result; the
// CPU oracle evaluates the same expressions in the same order.  LUTs are
// float4 texel arrays (RGB + 1), sampled bilinearly in software with
// clamp-to-edge and full FP32 weights (a sampler's fixed-point weights and
// the reference's FP16 / B10G11R11 storage are not emulated).  The
// exponentials are exp_cw (common.cuh), which the oracle reproduces bit for
// bit: the march's segment integral (S - S e^-x) / sigma cancels for
// optically thin segments and would magnify any exp difference.
#pragma once

#include "common.cuh"

namespace mrt {

constexpr float kSkyPi = 3.14159265358979323846f;  // constants.glsl PI
constexpr float kPlanetOffset = 0.01f;             // sky.glsl PLANET_RADIUS_OFFSET
constexpr uint32_t kTransW = 256, kTransH = 64;    // sky.ixx:24
constexpr uint32_t kMsW = 32, kMsH = 32;           // sky.ixx:27
constexpr uint32_t kViewW = 192, kViewH = 108;     // sky.ixx:184

// Miss-shader state: a sky-view LUT at the camera plus the transmittance
// LUT for the sun disc.  view == nullptr selects the constant sky.
struct SkyDev {
    const float4* view;
    const float4* trans;
    float bottom, top;
    float sun[3], sun_e[3];
    float cam[3];
};

MRT_DEV float fm(float a, float b) { return __fmul_rn(a, b); }
MRT_DEV float fa(float a, float b) { return __fadd_rn(a, b); }
MRT_DEV float fs(float a, float b) { return __fsub_rn(a, b); }
MRT_DEV float fd(float a, float b) { return __fdiv_rn(a, b); }
MRT_DEV float fclamp(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }

MRT_DEV f3 f3s(float s) { return f3{s, s, s}; }
MRT_DEV f3 div3(f3 a, f3 b) { return f3{fd(a.x, b.x), fd(a.y, b.y), fd(a.z, b.z)}; }
MRT_DEV f3 div3s(f3 a, float s) { return f3{fd(a.x, s), fd(a.y, s), fd(a.z, s)}; }
MRT_DEV f3 exp3(f3 a) { return f3{exp_cw(a.x), exp_cw(a.y), exp_cw(a.z)}; }
MRT_DEV float len3(f3 a) { return __fsqrt_rn(dot_rn(a, a)); }
MRT_DEV f3 cross_rn(f3 a, f3 b) {
    return f3{fs(fm(a.y, b.z), fm(a.z, b.y)), fs(fm(a.z, b.x), fm(a.x, b.z)), fs(fm(a.x, b.y), fm(a.y, b.x))};
}

// (u + 0.5/res) * (res/(res+1)) and its inverse (skyAccess.glsl:11-17)
MRT_DEV float unit_to_sub(float u, float res) { return fm(fa(u, fd(0.5f, res)), fd(res, fa(res, 1.0f))); }
MRT_DEV float sub_to_unit(float u, float res) { return fm(fs(u, fd(0.5f, res)), fd(res, fs(res, 1.0f))); }

// Bilinear clamp-to-edge fetch at normalised (u, v); texel centres at
// (i + 0.5) / w.  A NaN coordinate reads as 0.
MRT_DEV f3 lut_sample(const float4* lut, uint32_t w, uint32_t h, float u, float v) {
    float x = fs(fm(u, float(w)), 0.5f), y = fs(fm(v, float(h)), 0.5f);
    if (!(x == x)) x = 0.0f;
    if (!(y == y)) y = 0.0f;
    x = fclamp(x, -1.0f, float(w));
    y = fclamp(y, -1.0f, float(h));
    const float x0 = floorf(x), y0 = floorf(y);
    const float fx = fs(x, x0), fy = fs(y, y0);
    const int ix = int(x0), iy = int(y0);
    const int wi = int(w) - 1, hi = int(h) - 1;
    const int xa = min(max(ix, 0), wi), xb = min(max(ix + 1, 0), wi);
    const int ya = min(max(iy, 0), hi), yb = min(max(iy + 1, 0), hi);
    const float4 a = __ldg(lut + ya * int(w) + xa), b = __ldg(lut + ya * int(w) + xb);
    const float4 c = __ldg(lut + yb * int(w) + xa), d = __ldg(lut + yb * int(w) + xb);
    const float gx = fs(1.0f, fx), gy = fs(1.0f, fy);
    const f3 top{fa(fm(a.x, gx), fm(b.x, fx)), fa(fm(a.y, gx), fm(b.y, fx)), fa(fm(a.z, gx), fm(b.z, fx))};
    const f3 bot{fa(fm(c.x, gx), fm(d.x, fx)), fa(fm(c.y, gx), fm(d.y, fx)), fa(fm(c.z, gx), fm(d.z, fx))};
    return f3{fa(fm(top.x, gy), fm(bot.x, fy)), fa(fm(top.y, gy), fm(bot.y, fy)), fa(fm(top.z, gy), fm(bot.z, fy))};
}

// Distance to the nearest intersection with a sphere, or -1
// (sky.glsl raySphereIntersectNearest)
MRT_DEV float sky_sphere_nearest(f3 r0, f3 rd, f3 s0, float sr) {
    const float a = dot_rn(rd, rd);
    const f3 sr0 = sub_rn(r0, s0);
    const float b = fm(2.0f, dot_rn(rd, sr0));
    const float c = fs(dot_rn(sr0, sr0), fm(sr, sr));
    const float delta = fs(fm(b, b), fm(fm(4.0f, a), c));
    if (delta < 0.0f || a == 0.0f) return -1.0f;
    const float sq = __fsqrt_rn(delta), den = fm(2.0f, a);
    const float s0v = fd(fs(-b, sq), den), s1v = fd(fa(-b, sq), den);
    if (s0v < 0.0f && s1v < 0.0f) return -1.0f;
    if (s0v < 0.0f) return fmaxf(0.0f, s1v);
    if (s1v < 0.0f) return fmaxf(0.0f, s0v);
    return fmaxf(0.0f, fminf(s0v, s1v));
}

// (view height, cos zenith) -> transmittance LUT uv (skyAccess.glsl:36-53)
MRT_DEV void trans_uv(float h, float mu, float bottom, float top, float& u, float& v) {
    const float H = __fsqrt_rn(fmaxf(0.0f, fs(fm(top, top), fm(bottom, bottom))));
    const float rho = __fsqrt_rn(fmaxf(0.0f, fs(fm(h, h), fm(bottom, bottom))));
    const float disc = fa(fm(fm(h, h), fs(fm(mu, mu), 1.0f)), fm(top, top));
    const float d = fmaxf(0.0f, fa(fm(-h, mu), __fsqrt_rn(disc)));
    const float dmin = fs(top, h), dmax = fa(rho, H);
    u = fd(fs(d, dmin), fs(dmax, dmin));
    v = fd(rho, H);
}

// transmittance LUT uv -> (view height, cos zenith) (skyAccess.glsl:19-34)
MRT_DEV void trans_params(float u, float v, float bottom, float top, float& h, float& mu) {
    const float H = __fsqrt_rn(fs(fm(top, top), fm(bottom, bottom)));
    const float rho = fm(H, v);
    h = __fsqrt_rn(fa(fm(rho, rho), fm(bottom, bottom)));
    const float dmin = fs(top, h), dmax = fa(rho, H);
    const float d = fa(dmin, fm(u, fs(dmax, dmin)));
    mu = d == 0.0f ? 1.0f : fd(fs(fs(fm(H, H), fm(rho, rho)), fm(d, d)), fm(fm(2.0f, h), d));
    mu = fclamp(mu, -1.0f, 1.0f);
}

// (ground?, cos zenith, cos light-view) -> sky-view LUT uv
// (skyAccess.glsl:85-116, non-linear parameterisation)
MRT_DEV void view_uv(bool ground, float mu, float lv, float h, float bottom, float& u, float& v) {
    const float vh = __fsqrt_rn(fs(fm(h, h), fm(bottom, bottom)));
    const float beta = acosf(fd(vh, h));
    const float zha = fs(kSkyPi, beta);
    if (!ground) {
        float c = fd(acosf(mu), zha);
        c = fs(1.0f, __fsqrt_rn(fs(1.0f, c)));
        v = fm(c, 0.5f);
    } else {
        float c = fd(fs(acosf(mu), zha), beta);
        c = __fsqrt_rn(c);
        v = fa(fm(c, 0.5f), 0.5f);
    }
    u = __fsqrt_rn(fa(fm(-lv, 0.5f), 0.5f));
    u = unit_to_sub(u, float(kViewW));
    v = unit_to_sub(v, float(kViewH));
}

// sky-view LUT uv -> (cos zenith, cos light-view) (skyAccess.glsl:55-83)
MRT_DEV void view_params(float u, float v, float h, float bottom, float& mu, float& lv) {
    u = sub_to_unit(u, float(kViewW));
    v = sub_to_unit(v, float(kViewH));
    const float vh = __fsqrt_rn(fs(fm(h, h), fm(bottom, bottom)));
    const float beta = acosf(fd(vh, h));
    const float zha = fs(kSkyPi, beta);
    if (v < 0.5f) {
        float c = fm(2.0f, v);
        c = fs(1.0f, c);
        c = fm(c, c);
        c = fs(1.0f, c);
        mu = cosf(fm(zha, c));
    } else {
        float c = fs(fm(v, 2.0f), 1.0f);
        c = fm(c, c);
        mu = cosf(fa(zha, fm(beta, c)));
    }
    const float c = fm(u, u);
    lv = -fs(fm(c, 2.0f), 1.0f);
}

// Sun disc luminance (sky.glsl getSunLuminance): limb-darkened disc of
// angular radius 0.2525 deg, scaled by the transmittance to the sun over
// the transmittance straight up.
MRT_DEV f3 sun_luminance(const SkyDev& s, f3 pos, f3 dir) {
    const float radius = fd(fm(fm(0.5f, 0.505f), 3.14159f), 180.0f);
    const f3 sun{s.sun[0], s.sun[1], s.sun[2]};
    if (!(dot_rn(dir, sun) > cosf(radius))) return f3s(0.0f);
    if (sky_sphere_nearest(pos, dir, f3s(0.0f), s.bottom) >= 0.0f) return f3s(0.0f);
    float uu, vu, us, vs;
    trans_uv(s.bottom, 1.0f, s.bottom, s.top, uu, vu);
    const float ph = len3(pos);
    const f3 up = div3s(pos, ph);
    trans_uv(ph, dot_rn(sun, up), s.bottom, s.top, us, vs);
    const float ang = acosf(fclamp(dot_rn(dir, sun), -1.0f, 1.0f));
    const float rr = fd(ang, radius);
    const float limb = __fsqrt_rn(fclamp(fs(1.0f, fm(rr, rr)), 0.0001f, 1.0f));
    const f3 tu = lut_sample(s.trans, kTransW, kTransH, uu, vu);
    const f3 ts = lut_sample(s.trans, kTransW, kTransH, us, vs);
    const f3 space = div3(f3{s.sun_e[0], s.sun_e[1], s.sun_e[2]}, tu);
    return scale_rn(mul_rn(space, ts), limb);
}

// skyColor(dir) (secondaryRays.comp:36-58): the sky-view LUT in the frame
// of the camera and the sun plus the sun disc scaled to 120000 lux.
MRT_DEV f3 sky_color(const SkyDev& s, f3 dir) {
    const f3 pos{s.cam[0], s.cam[1], fa(s.cam[2], s.bottom)};
    const f3 up = normalize_rn(pos);
    const float mu = dot_rn(dir, up);
    const float h = len3(pos);
    const f3 sun{s.sun[0], s.sun[1], s.sun[2]};
    const f3 side = normalize_rn(cross_rn(up, dir));
    const f3 fwd = normalize_rn(cross_rn(side, up));
    float lx = dot_rn(sun, fwd), ly = dot_rn(sun, side);
    const float ll = __fsqrt_rn(fa(fm(lx, lx), fm(ly, ly)));
    lx = fd(lx, ll);
    const bool ground = sky_sphere_nearest(pos, dir, f3s(0.0f), s.bottom) >= 0.0f;
    float u, v;
    view_uv(ground, mu, lx, h, s.bottom, u, v);
    const f3 sv = lut_sample(s.view, kViewW, kViewH, u, v);
    const f3 e{s.sun_e[0], s.sun_e[1], s.sun_e[2]};
    const f3 sl = mul_rn(sun_luminance(s, pos, dir), div3(f3s(120000.0f), e));
    return add_rn(sv, sl);
}

}  // namespace mrt
