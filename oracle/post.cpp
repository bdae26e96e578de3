// CPU oracle, part 2 (TEST INFRASTRUCTURE ONLY): sky / atmosphere LUTs and
// miss shader, joint bilateral filter, tonemappers, temporal reprojection.
//
// Pinned to the reference's own shaders compiled for the host (oracle/glsl,
// tests/test_oracle_glsl_pins.py): the sky LUTs and the tonemappers agree
// bit for bit, the bilateral filter to 1e-5 (its sample positions).
// This file restates the reference's shader arithmetic in plain FP32 C++
// (compiled with -ffp-contract=off, so every + - * / rounds separately),
// expression by expression and in the same evaluation order as the GLSL:
//   sky:      src/gpu/sky/sky.glsl, skyAccess.glsl, genTransmittance.comp,
//             genMultiScattering.comp, genView.comp,
//             src/gpu/secondaryRays.comp:36-58, src/gfx/modules/sky.ixx
//   filter:   src/gpu/denoise/bilateral.comp:23-76, denoiser.ixx:25-31
//   tonemap:  src/gpu/tonemap/*.comp, src/gpu/util.glsl:13-18,
//             tonemapper.ixx:46-54
// Texture reads are bilinear clamp-to-edge with FP32 weights on float
// texels; the reference's FP16 / B10G11R11 / UNORM8 storage and a
// sampler's fixed-point weights are not emulated (the CUDA kernels do the
// same).  Only tests/, the smoke check and bench.py's CPU baseline load it.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>

namespace {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kOffset = 0.01f;
constexpr int kTW = 256, kTH = 64, kMW = 32, kMH = 32, kVW = 192, kVH = 108;

struct V3 {
    float x, y, z;
};
inline V3 v3(float s) { return V3{s, s, s}; }
inline V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(V3 a, V3 b) { return V3{a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 operator*(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
inline V3 operator/(V3 a, V3 b) { return V3{a.x / b.x, a.y / b.y, a.z / b.z}; }
inline V3 operator/(V3 a, float s) { return V3{a.x / s, a.y / s, a.z / s}; }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float length(V3 a) { return std::sqrt(dot(a, a)); }
inline V3 normalize(V3 a) { return a / length(a); }
inline V3 cross(V3 a, V3 b) { return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
// e^x as the CUDA kernels compute it (exp_cw in common.cuh): Cody-Waite
// reduction x = n ln2 + r with a 16-bit head of ln2, the degree-7 Taylor
// polynomial of e^r in Horner form with fma, an exact scale by 2^n.
float exp_cw(float x) {
    if (!(x > -87.0f)) return std::isnan(x) ? x : 0.0f;
    if (x > 88.0f) return INFINITY;
    const float n = std::nearbyint(x * 1.44269502f);
    float r = std::fma(-n, 0.693145752f, x);
    r = std::fma(-n, 1.42860677e-6f, r);
    float p = 1.98412701e-4f;
    p = std::fma(p, r, 1.38888892e-3f);
    p = std::fma(p, r, 8.33333377e-3f);
    p = std::fma(p, r, 4.16666679e-2f);
    p = std::fma(p, r, 1.66666672e-1f);
    p = std::fma(p, r, 0.5f);
    p = std::fma(p, r, 1.0f);
    p = std::fma(p, r, 1.0f);
    const int e = int(n);
    if (e < -126) return 0.0f;
    const uint32_t bits = uint32_t(e + 127) << 23;
    float s;
    std::memcpy(&s, &bits, 4);
    return p * s;
}
// binary32 transcendental functions evaluated in binary64 and rounded once:
// the same bits on every host (the C library's binary32 versions differ
// between x86-64 and AArch64 in the last place)
inline float acos_(float x) { return float(std::acos(double(x))); }
inline float cos_(float x) { return float(std::cos(double(x))); }
inline float sin_(float x) { return float(std::sin(double(x))); }
inline float pow_(float x, float y) { return float(std::pow(double(x), double(y))); }
inline float exp_(float x) { return float(std::exp(double(x))); }
inline V3 vexp(V3 a) { return V3{exp_cw(a.x), exp_cw(a.y), exp_cw(a.z)}; }
inline float clampf(float x, float lo, float hi) { return std::fmin(std::fmax(x, lo), hi); }

struct Atmo {  // mrt_atmosphere_params
    float bottom, top, ray_exp;
    float ray_scat[3];
    float mie_exp;
    float mie_scat[3], mie_ext[3], mie_abs[3];
    float mie_g;
    float oz_width, oz_c0, oz_l0, oz_c1, oz_l1;
    float oz_ext[3];
    float ground[3];
};
inline V3 ld(const float* p) { return V3{p[0], p[1], p[2]}; }

float to_sub(float u, float res) { return (u + 0.5f / res) * (res / (res + 1.0f)); }
float from_sub(float u, float res) { return (u - 0.5f / res) * (res / (res - 1.0f)); }

// texture(lut, uv) with a linear clamp-to-edge sampler
V3 sample(const float* lut, int w, int h, float u, float v) {
    float x = u * float(w) - 0.5f, y = v * float(h) - 0.5f;
    if (std::isnan(x)) x = 0.0f;
    if (std::isnan(y)) y = 0.0f;
    x = clampf(x, -1.0f, float(w));
    y = clampf(y, -1.0f, float(h));
    const float x0 = std::floor(x), y0 = std::floor(y);
    const float fx = x - x0, fy = y - y0;
    const int ix = int(x0), iy = int(y0);
    const int xa = std::min(std::max(ix, 0), w - 1), xb = std::min(std::max(ix + 1, 0), w - 1);
    const int ya = std::min(std::max(iy, 0), h - 1), yb = std::min(std::max(iy + 1, 0), h - 1);
    const float* a = lut + 4 * (ya * w + xa);
    const float* b = lut + 4 * (ya * w + xb);
    const float* c = lut + 4 * (yb * w + xa);
    const float* d = lut + 4 * (yb * w + xb);
    float r[3];
    for (int k = 0; k < 3; ++k) {
        const float t = a[k] * (1.0f - fx) + b[k] * fx;
        const float s = c[k] * (1.0f - fx) + d[k] * fx;
        r[k] = t * (1.0f - fy) + s * fy;
    }
    return V3{r[0], r[1], r[2]};
}

// sky.glsl raySphereIntersectNearest
float sphere_nearest(V3 r0, V3 rd, V3 s0, float sr) {
    const float a = dot(rd, rd);
    const V3 d = r0 - s0;
    const float b = 2.0f * dot(rd, d);
    const float c = dot(d, d) - sr * sr;
    const float delta = b * b - 4.0f * a * c;
    if (delta < 0.0f || a == 0.0f) return -1.0f;
    const float s0v = (-b - std::sqrt(delta)) / (2.0f * a);
    const float s1v = (-b + std::sqrt(delta)) / (2.0f * a);
    if (s0v < 0.0f && s1v < 0.0f) return -1.0f;
    if (s0v < 0.0f) return std::fmax(0.0f, s1v);
    if (s1v < 0.0f) return std::fmax(0.0f, s0v);
    return std::fmax(0.0f, std::fmin(s0v, s1v));
}

// skyAccess.glsl lutTransmittanceParamsToUv
void trans_uv(float h, float mu, float bottom, float top, float& u, float& v) {
    const float H = std::sqrt(std::fmax(0.0f, top * top - bottom * bottom));
    const float rho = std::sqrt(std::fmax(0.0f, h * h - bottom * bottom));
    const float disc = h * h * (mu * mu - 1.0f) + top * top;
    const float d = std::fmax(0.0f, -h * mu + std::sqrt(disc));
    const float dmin = top - h, dmax = rho + H;
    u = (d - dmin) / (dmax - dmin);
    v = rho / H;
}

// skyAccess.glsl uvToLutTransmittanceParams
void trans_params(float u, float v, float bottom, float top, float& h, float& mu) {
    const float H = std::sqrt(top * top - bottom * bottom);
    const float rho = H * v;
    h = std::sqrt(rho * rho + bottom * bottom);
    const float dmin = top - h, dmax = rho + H;
    const float d = dmin + u * (dmax - dmin);
    mu = d == 0.0f ? 1.0f : (H * H - rho * rho - d * d) / (2.0f * h * d);
    mu = clampf(mu, -1.0f, 1.0f);
}

// skyAccess.glsl skyViewLutParamsToUv (non-linear)
void view_uv(bool ground, float mu, float lv, float h, float bottom, float& u, float& v) {
    const float vh = std::sqrt(h * h - bottom * bottom);
    const float beta = acos_(vh / h);
    const float zha = kPi - beta;
    if (!ground) {
        float c = acos_(mu) / zha;
        c = 1.0f - c;
        c = std::sqrt(c);
        c = 1.0f - c;
        v = c * 0.5f;
    } else {
        float c = (acos_(mu) - zha) / beta;
        c = std::sqrt(c);
        v = c * 0.5f + 0.5f;
    }
    u = std::sqrt(-lv * 0.5f + 0.5f);
    u = to_sub(u, float(kVW));
    v = to_sub(v, float(kVH));
}

// skyAccess.glsl uvToSkyViewLutParams
void view_params(float u, float v, float h, float bottom, float& mu, float& lv) {
    u = from_sub(u, float(kVW));
    v = from_sub(v, float(kVH));
    const float vh = std::sqrt(h * h - bottom * bottom);
    const float beta = acos_(vh / h);
    const float zha = kPi - beta;
    if (v < 0.5f) {
        float c = 2.0f * v;
        c = 1.0f - c;
        c *= c;
        c = 1.0f - c;
        mu = cos_(zha * c);
    } else {
        float c = v * 2.0f - 1.0f;
        c *= c;
        mu = cos_(zha + beta * c);
    }
    float c = u;
    c *= c;
    lv = -(c * 2.0f - 1.0f);
}

struct Medium {
    V3 scat, ext, scat_mie, scat_ray;
};

// sky.glsl sampleMediumRGB
Medium medium(const Atmo& a, V3 p) {
    const float h = length(p) - a.bottom;
    const float dm = exp_cw(a.mie_exp * h);
    const float dr = exp_cw(a.ray_exp * h);
    const float dz = clampf(h < a.oz_width ? a.oz_l0 * h + a.oz_c0 : a.oz_l1 * h + a.oz_c1, 0.0f, 1.0f);
    Medium m;
    m.scat_mie = ld(a.mie_scat) * dm;
    const V3 ext_mie = ld(a.mie_ext) * dm;
    m.scat_ray = ld(a.ray_scat) * dr;
    const V3 ext_ozo = ld(a.oz_ext) * dz;
    m.scat = m.scat_mie + m.scat_ray;
    m.ext = ext_mie + m.scat_ray + ext_ozo;
    return m;
}

struct March {
    V3 L, od, ms_as1;
};

// sky.glsl integrateScatteredLuminance (unused outputs dropped)
March integrate(const Atmo& a, V3 pos, V3 dir, V3 sun, bool ground, float count, bool variable, bool mie_ray,
                V3 light, const float* trans, const float* ms) {
    March r{v3(0.0f), v3(0.0f), v3(0.0f)};
    const float tb = sphere_nearest(pos, dir, v3(0.0f), a.bottom);
    const float tt = sphere_nearest(pos, dir, v3(0.0f), a.top);
    float tmax = 0.0f;
    if (tb < 0.0f) {
        if (tt < 0.0f) return r;
        tmax = tt;
    } else if (tt > 0.0f) {
        tmax = std::fmin(tt, tb);
    }
    tmax = std::fmin(tmax, 9000000.0f);
    float n = count, nfloor = count, tmax_floor = tmax;
    if (variable) {
        const float w = clampf(tmax * 0.01f, 0.0f, 1.0f);
        n = 4.0f * (1.0f - w) + 14.0f * w;  // mix(4, 14, w)
        nfloor = std::floor(n);
        tmax_floor = tmax * nfloor / n;
    }
    const float ct = dot(sun, dir);
    const float g = a.mie_g;
    const float mc = -ct;  // cornetteShanksMiePhaseFunction(g, -cosTheta)
    const float k = 3.0f / (8.0f * kPi) * (1.0f - g * g) / (2.0f + g * g);
    const float mie_phase = k * (1.0f + mc * mc) / pow_(1.0f + g * g - 2.0f * g * -mc, 1.5f);
    const float ray_phase = 3.0f / (16.0f * kPi) * (1.0f + ct * ct);
    const float uni = 1.0f / (4.0f * kPi);
    V3 thr = v3(1.0f);
    float t = 0.0f, dt = 0.0f;
    for (float s = 0.0f; s < n; s += 1.0f) {
        if (variable) {
            float t0 = s / nfloor, t1 = (s + 1.0f) / nfloor;
            t0 = t0 * t0;
            t1 = t1 * t1;
            t0 = tmax_floor * t0;
            if (t1 > 1.0f)
                t1 = tmax;
            else
                t1 = tmax_floor * t1;
            t = t0 + (t1 - t0) * 0.3f;
            dt = t1 - t0;
        } else {
            const float nt = tmax * (s + 0.3f) / n;
            dt = nt - t;
            t = nt;
        }
        const V3 P = pos + dir * t;
        const Medium m = medium(a, P);
        const V3 sod = m.ext * dt;
        const V3 st = vexp(V3{-sod.x, -sod.y, -sod.z});
        r.od = r.od + sod;
        const float ph = length(P);
        const V3 up = P / ph;
        const float sz = dot(sun, up);
        float u, v;
        trans_uv(ph, sz, a.bottom, a.top, u, v);
        const V3 tsun = trans ? sample(trans, kTW, kTH, u, v) : v3(0.0f);
        const V3 pts = mie_ray ? m.scat_mie * mie_phase + m.scat_ray * ray_phase : m.scat * uni;
        const float te = sphere_nearest(P, sun, up * kOffset, a.bottom);
        const float shadow = te >= 0.0f ? 0.0f : 1.0f;
        V3 msl = v3(0.0f);
        if (ms) {
            const float mu = clampf(sz * 0.5f + 0.5f, 0.0f, 1.0f);
            const float mv = clampf((ph - a.bottom) / (a.top - a.bottom), 0.0f, 1.0f);
            msl = sample(ms, kMW, kMH, to_sub(mu, float(kMW)), to_sub(mv, float(kMH)));
        }
        const V3 S = light * (tsun * shadow * pts + msl * m.scat);
        const V3 msint = (m.scat - m.scat * st) / m.ext;
        r.ms_as1 = r.ms_as1 + thr * msint;
        const V3 sint = (S - S * st) / m.ext;
        r.L = r.L + thr * sint;
        thr = thr * st;
    }
    if (ground && tmax == tb && tb > 0.0f) {
        const V3 P = pos + dir * tb;
        const float ph = length(P);
        const V3 up = P / ph;
        float u, v;
        trans_uv(ph, dot(sun, up), a.bottom, a.top, u, v);
        const V3 tsun = trans ? sample(trans, kTW, kTH, u, v) : v3(0.0f);
        const float ndl = clampf(dot(normalize(up), normalize(sun)), 0.0f, 1.0f);
        r.L = r.L + light * tsun * thr * ndl * ld(a.ground) / kPi;
    }
    return r;
}

V3 sun_luminance(const Atmo& a, const float* trans, V3 pos, V3 dir, V3 sun, V3 sun_e) {
    const float radius = 0.5f * 0.505f * 3.14159f / 180.0f;
    if (!(dot(dir, sun) > cos_(radius))) return v3(0.0f);
    if (sphere_nearest(pos, dir, v3(0.0f), a.bottom) >= 0.0f) return v3(0.0f);
    float uu, vu, us, vs;
    trans_uv(a.bottom, 1.0f, a.bottom, a.top, uu, vu);
    const float ph = length(pos);
    const V3 up = pos / ph;
    trans_uv(ph, dot(sun, up), a.bottom, a.top, us, vs);
    const float ang = acos_(clampf(dot(dir, sun), -1.0f, 1.0f));
    const float rr = ang / radius;
    const float limb = std::sqrt(clampf(1.0f - rr * rr, 0.0001f, 1.0f));
    const V3 space = sun_e / sample(trans, kTW, kTH, uu, vu);
    return space * sample(trans, kTW, kTH, us, vs) * limb;
}

}  // namespace

extern "C" {

// genTransmittance.comp
void orc_sky_transmittance(const Atmo* a, float* out) {
    for (int y = 0; y < kTH; ++y)
        for (int x = 0; x < kTW; ++x) {
            const float u = (float(x) + 0.5f) / float(kTW), v = (float(y) + 0.5f) / float(kTH);
            float h, mu;
            trans_params(u, v, a->bottom, a->top, h, mu);
            const V3 dir{0.0f, std::sqrt(1.0f - mu * mu), mu};
            const March m = integrate(*a, V3{0.0f, 0.0f, h}, dir, v3(1.0f), false, 40.0f, false, false, v3(1.0f),
                                      nullptr, nullptr);
            float* o = out + 4 * (y * kTW + x);
            o[0] = exp_cw(-m.od.x);
            o[1] = exp_cw(-m.od.y);
            o[2] = exp_cw(-m.od.z);
            o[3] = 1.0f;
        }
}

// genMultiScattering.comp, with the 64 -> 1 tree reduction in its order
void orc_sky_multiscatter(const Atmo* a, const float* trans, float* out) {
    const float sphere = 4.0f * kPi;
    for (int y = 0; y < kMH; ++y)
        for (int x = 0; x < kMW; ++x) {
            float u = (float(x) + 0.5f) / float(kMW), v = (float(y) + 0.5f) / float(kMH);
            u = from_sub(u, float(kMW));
            v = from_sub(v, float(kMH));
            const float cs = u * 2.0f - 1.0f;
            const V3 sun{0.0f, std::sqrt(clampf(1.0f - cs * cs, 0.0f, 1.0f)), cs};
            const float h = a->bottom + clampf(v + kOffset, 0.0f, 1.0f) * (a->top - a->bottom - kOffset);
            V3 sms[64], sl[64];
            for (int z = 0; z < 64; ++z) {
                const float iv = 0.5f + float(z / 8), jv = 0.5f + float(z % 8);
                const float theta = 2.0f * kPi * (iv / 8.0f), phi = kPi * (jv / 8.0f);
                const V3 dir{cos_(theta) * sin_(phi), sin_(theta) * sin_(phi), cos_(phi)};
                const March m = integrate(*a, V3{0.0f, 0.0f, h}, dir, sun, true, 20.0f, false, false, v3(1.0f),
                                          trans, nullptr);
                sms[z] = m.ms_as1 * sphere / 64.0f;
                sl[z] = m.L * sphere / 64.0f;
            }
            for (int half = 32; half >= 1; half >>= 1)
                for (int z = 0; z < half; ++z) {
                    sms[z] = sms[z] + sms[z + half];
                    sl[z] = sl[z] + sl[z + half];
                }
            const float iso = 1.0f / sphere;
            const V3 r = sms[0] * iso, L1 = sl[0] * iso;
            const V3 r2 = r * r;
            const V3 L = L1 * (v3(1.0f) + r + r2 + r * r2 + r2 * r2);
            float* o = out + 4 * (y * kMW + x);
            o[0] = L.x;
            o[1] = L.y;
            o[2] = L.z;
            o[3] = 1.0f;
        }
}

// genView.comp
void orc_sky_view(const Atmo* a, const float* trans, const float* ms, const float* probe, const float* sun_w,
                  const float* light, float* out) {
    for (int y = 0; y < kVH; ++y)
        for (int x = 0; x < kVW; ++x) {
            V3 pos{probe[0], probe[1], probe[2] + a->bottom};
            const float u = float(x) / float(kVW), v = float(y) / float(kVH);
            const float h = length(pos);
            float mu, lv;
            view_params(u, v, h, a->bottom, mu, lv);
            const V3 up = pos / h;
            const float sz = dot(up, ld(sun_w));
            const V3 sun = normalize(V3{std::sqrt(1.0f - sz * sz), 0.0f, sz});
            pos = V3{0.0f, 0.0f, h};
            const float sv = std::sqrt(1.0f - mu * mu);
            const V3 dir{sv * lv, sv * std::sqrt(1.0f - lv * lv), mu};
            float* o = out + 4 * (y * kVW + x);
            if (h > a->top) {  // moveToTopAtmosphere
                const float tt = sphere_nearest(pos, dir, v3(0.0f), a->top);
                if (!(tt >= 0.0f)) {
                    o[0] = o[1] = o[2] = 0.0f;
                    o[3] = 1.0f;
                    continue;
                }
                pos = pos + dir * tt + (pos / h) * -kOffset;
            }
            const March m = integrate(*a, pos, dir, sun, false, 30.0f, true, true, ld(light), trans, ms);
            o[0] = m.L.x;
            o[1] = m.L.y;
            o[2] = m.L.z;
            o[3] = 1.0f;
        }
}

// skyColor (secondaryRays.comp:36-58) for n directions
void orc_sky_color(const Atmo* a, const float* trans, const float* view, const float* cam, const float* sun_dir,
                   const float* sun_e, const float* dirs, uint32_t n, float* out) {
    const V3 pos{cam[0], cam[1], cam[2] + a->bottom};
    const V3 sun = ld(sun_dir), e = ld(sun_e);
    for (uint32_t i = 0; i < n; ++i) {
        const V3 dir = ld(dirs + 3 * i);
        const V3 up = normalize(pos);
        const float mu = dot(dir, up);
        const float h = length(pos);
        const V3 side = normalize(cross(up, dir));
        const V3 fwd = normalize(cross(side, up));
        float lx = dot(sun, fwd), ly = dot(sun, side);
        const float ll = std::sqrt(lx * lx + ly * ly);
        lx = lx / ll;
        const bool ground = sphere_nearest(pos, dir, v3(0.0f), a->bottom) >= 0.0f;
        float u, v;
        view_uv(ground, mu, lx, h, a->bottom, u, v);
        const V3 sv = sample(view, kVW, kVH, u, v);
        const V3 sl = sun_luminance(*a, trans, pos, dir, sun, e) * (v3(120000.0f) / e);
        const V3 c = sv + sl;
        out[3 * i] = c.x;
        out[3 * i + 1] = c.y;
        out[3 * i + 2] = c.z;
    }
}

}  // extern "C"

// ---- sky binding for the path-tracing oracle (oracle.cpp) ----------------
namespace {
struct SkyBinding {
    bool on = false;
    Atmo a{};
    float trans[kTW * kTH * 4];
    float view[kVW * kVH * 4];
    float cam[3], sun[3], sun_e[3];
};
SkyBinding g_sky;
}  // namespace

extern "C" {

// Binds (atmo != NULL) or unbinds the sky that escaping paths of the FP32
// path-tracing oracle see, like mrt_cuda_set_sky.
void orc_sky_bind(const Atmo* a, const float* trans, const float* view, const float* cam, const float* sun_dir,
                  const float* sun_e) {
    g_sky.on = a != nullptr;
    if (!a) return;
    g_sky.a = *a;
    std::memcpy(g_sky.trans, trans, sizeof(g_sky.trans));
    std::memcpy(g_sky.view, view, sizeof(g_sky.view));
    for (int k = 0; k < 3; ++k) {
        g_sky.cam[k] = cam[k];
        g_sky.sun[k] = sun_dir[k];
        g_sky.sun_e[k] = sun_e[k];
    }
}

// Radiance of a path escaping along `dir` under the bound sky; 0 when no
// sky is bound (the caller then uses its constant sky).
int orc_sky_escape(const float* dir, float* out) {
    if (!g_sky.on) return 0;
    orc_sky_color(&g_sky.a, g_sky.trans, g_sky.view, g_sky.cam, g_sky.sun, g_sky.sun_e, dir, 1, out);
    return 1;
}

}  // extern "C"

// ---- joint bilateral filter (bilateral.comp:23-76) ------------------------
// Float planes: color RGB, depth (R16F widened), normal xyz (widened).  The
// reference's taps texture(tex, uv + d/size) land on whole columns and at
// row y + d.y; here row y + d.y is read as the rows y + floor(d.y) and
// y + floor(d.y) + 1 at weight frac(d.y), clamped to the image.
extern "C" float orc_exp_cw(float x) { return exp_cw(x); }

extern "C" int orc_bilateral(const float* color, const float* depth, const float* normal, uint32_t w, uint32_t h,
                             float sigma, float k_sigma, float threshold, float near_plane, uint32_t frame,
                             int dither, float* out) {
    const float radius = std::round(k_sigma * sigma);
    if (!(radius >= 0.0f) || radius > 24.0f) return -1;
    const float rad_q = radius * radius;
    const float inv_sq2 = 0.5f / (sigma * sigma);
    const float inv_sq2pi = 0.31830988618379067154f * inv_sq2;
    const float inv_thr_sq2 = 0.5f / (threshold * threshold);
    const float inv_thr_sqrt2pi = 0.39894228040143267794f / threshold;
    const int r = int(radius);
    auto at = [&](int x, int y) {
        x = std::min(std::max(x, 0), int(w) - 1);
        y = std::min(std::max(y, 0), int(h) - 1);
        return size_t(y) * w + size_t(x);
    };
    for (uint32_t y = 0; y < h; ++y)
        for (uint32_t x = 0; x < w; ++x) {
            const size_t ic = size_t(y) * w + x;
            float res[3] = {color[3 * ic], color[3 * ic + 1], color[3 * ic + 2]};
            const float cz = depth[ic];
            if (!(cz < 0.0f)) {
                const float cn[3] = {normal[3 * ic], normal[3 * ic + 1], normal[3 * ic + 2]};
                const float ncz = near_plane / cz;
                float zb = 0.0f, acc[3] = {0.0f, 0.0f, 0.0f};
                for (int c = 0; c <= 2 * r; ++c) {
                    const float dx = float(c - r);
                    const float pt = std::sqrt(rad_q - dx * dx);
                    const float f0 = std::floor(-pt);
                    const float fr = -pt - f0, gr = 1.0f - fr;
                    int row = int(y) + int(f0);
                    for (float dy = -pt; dy <= pt; dy += 1.0f, ++row) {
                        const float blur = exp_(-(dx * dx + dy * dy) * inv_sq2) * inv_sq2pi;
                        const size_t a = at(int(x) + c - r, row), b = at(int(x) + c - r, row + 1);
                        const float wz = depth[a] * gr + depth[b] * fr;
                        const float wn[3] = {normal[3 * a] * gr + normal[3 * b] * fr,
                                             normal[3 * a + 1] * gr + normal[3 * b + 1] * fr,
                                             normal[3 * a + 2] * gr + normal[3 * b + 2] * fr};
                        float dz = near_plane / wz - ncz;
                        dz = dz * 100.0f;
                        const float dn = wn[0] * cn[0] + wn[1] * cn[1] + wn[2] * cn[2];
                        const float arg = clampf(dn - dz * dz, 0.0f, 1.0f) * inv_thr_sq2;
                        const float df = exp_cw(arg) * inv_thr_sqrt2pi * blur;
                        zb = zb + df;
                        for (int k = 0; k < 3; ++k) acc[k] = acc[k] + df * (color[3 * a + k] * gr + color[3 * b + k] * fr);
                    }
                }
                for (int k = 0; k < 3; ++k) res[k] = acc[k] / zb;
            }
            if (dither) {
                uint32_t seed = x * 709u + y * 1153u + frame * 1361u;
                // random.glsl pcg + randomFloat
                const uint32_t state = seed * 747796405u + 2891336453u;
                const uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
                seed = (word >> 22u) ^ word;
                const float nz = float(seed & 0xFFFFFFu) * (1.0f / 16777216.0f) * 0.005f;
                for (int k = 0; k < 3; ++k) res[k] = res[k] + nz;
            }
            for (int k = 0; k < 3; ++k) out[3 * ic + k] = res[k];
        }
    return 0;
}

// ---- tonemappers (src/gpu/tonemap/*.comp, util.glsl:13-18) ----------------
namespace {

float srgb1(float c) { return c < 0.0031308f ? 12.92f * c : 1.055f * pow_(c, 1.0f / 2.4f) - 0.055f; }

float hable_op(float x) {
    const float A = 0.15f, B = 0.50f, C = 0.10f, D = 0.20f, E = 0.02f, F = 0.30f;
    return ((x * (A * x + C * B) + D * E) / (x * (A * x + B) + D * F)) - E / F;
}

float rrt(float v) {
    const float a = v * (v + 0.0245786f) - 0.000090537f;
    const float b = v * (0.983729f * v + 0.4329510f) + 0.238081f;
    return a / b;
}

float uchimura1(float x, const float* u) {
    const float P = u[0], a = u[1], m = u[2], l = u[3], c = u[4], b = u[5];
    const float l0 = ((P - m) * l) / a;
    const float S0 = m + l0;
    const float S1 = m + a * l0;
    const float C2 = (a * P) / (P - S1);
    const float CP = -C2 / P;
    const float t = clampf((x - 0.0f) / (m - 0.0f), 0.0f, 1.0f);  // smoothstep(0, m, x)
    const float w0 = 1.0f - t * t * (3.0f - 2.0f * t);
    const float w2 = x < m + l0 ? 0.0f : 1.0f;                       // step(m + l0, x)
    const float w1 = 1.0f - w0 - w2;
    const float T = m * pow_(x / m, c) + b;
    const float S = P - (P - S1) * exp_(CP * (x - S0));
    const float L = m + a * (x - m);
    return T * w0 + L * w1 + S * w2;
}

}  // namespace

// mode: 0 linear, 1 reinhard, 2 hable, 3 aces, 4 uchimura, 5 amd.
// params: exposure, reinhard max, uchimura[6], amd[5] (hdr max, contrast,
// shoulder, mid in, mid out).  out: RGBA8.
extern "C" void orc_tonemap(const float* color, uint32_t n, uint32_t mode, const float* params, uint8_t* out) {
    const float exposure = params[0], rmax = params[1];
    const float* u = params + 2;
    const float* amd = params + 8;
    // amd.comp ColToneB / ColToneC
    const float hdr = amd[0], contrast = amd[1], shoulder = amd[2], mid_in = amd[3], mid_out = amd[4];
    const float pa = pow_(mid_in, contrast), hs = pow_(hdr, contrast * shoulder);
    const float ms = pow_(mid_in, contrast * shoulder), hc = pow_(hdr, contrast);
    const float bb = -((-pa + (mid_out * (hs * pa - hc * ms * mid_out)) / (hs * mid_out - ms * mid_out)) /
                       (ms * mid_out));
    const float cc = (hs * pa - hc * ms * mid_out) / (hs * mid_out - ms * mid_out);
    const float hw = hable_op(11.2f);
    for (uint32_t i = 0; i < n; ++i) {
        float c[3] = {color[3 * i] * exposure, color[3 * i + 1] * exposure, color[3 * i + 2] * exposure};
        if (mode == 1) {
            for (int k = 0; k < 3; ++k) c[k] = (c[k] * (1.0f + c[k] / (rmax * rmax))) / (1.0f + c[k]);
        } else if (mode == 2) {
            for (int k = 0; k < 3; ++k) c[k] = hable_op(2.0f * c[k]) / hw;
        } else if (mode == 3) {
            const float in[3][3] = {{0.59719f, 0.35458f, 0.04823f}, {0.07600f, 0.90834f, 0.01566f},
                                    {0.02840f, 0.13383f, 0.83777f}};
            const float ou[3][3] = {{1.60475f, -0.53108f, -0.07367f}, {-0.10208f, 1.10813f, -0.00605f},
                                    {-0.00327f, -0.07276f, 1.07602f}};
            float t[3];
            for (int j = 0; j < 3; ++j) t[j] = rrt(c[0] * in[j][0] + c[1] * in[j][1] + c[2] * in[j][2]);
            for (int j = 0; j < 3; ++j) c[j] = clampf(t[0] * ou[j][0] + t[1] * ou[j][1] + t[2] * ou[j][2], 0.0f, 1.0f);
        } else if (mode == 4) {
            for (int k = 0; k < 3; ++k) c[k] = uchimura1(c[k], u);
        } else if (mode == 5) {
            float peak = std::fmax(c[0], std::fmax(c[1], c[2]));
            peak = std::fmax(1e-6f, peak);
            float ratio[3] = {c[0] / peak, c[1] / peak, c[2] / peak};
            const float z = pow_(peak, contrast);
            peak = z / (pow_(z, shoulder) * bb + cc);
            const float cross = contrast * 16.0f, e = contrast / cross;
            const float mx = pow_(peak, 4.0f);
            for (int k = 0; k < 3; ++k) {
                float q = pow_(std::fabs(ratio[k]), e);
                q = q * (1.0f - mx) + 1.0f * mx;  // mix(ratio, white, pow(peak, crosstalk))
                q = pow_(std::fabs(q), cross);
                c[k] = q * peak;
            }
        }
        for (int k = 0; k < 3; ++k) {
            const float v = clampf(srgb1(c[k]), 0.0f, 1.0f) * 255.0f;
            out[4 * i + k] = uint8_t(std::nearbyint(v));
        }
        out[4 * i + 3] = 255;
    }
}
