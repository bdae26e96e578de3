// Atmosphere LUTs (transmittance, multiple scattering, sky view) and the
// sky C ABI.
//
// Replaces the reference's Atmosphere / Sky modules
// (src/gfx/modules/sky.ixx:18-262) and their compute shaders
// (src/gpu/sky/genTransmittance.comp, genMultiScattering.comp,
// genView.comp), which the reference runs every frame.  Each LUT is one
// small launch: 256x64 transmittance texels (40-step optical-depth march),
// 32x32 multi-scattering texels with 64 sphere directions each (one
// 64-thread block per texel, tree reduction in shared memory), and a
// 192x108 sky view at the camera (variable 4-14 step march with Mie +
// Rayleigh phases).  All three together take well under 0.1 ms; the miss
// shader that reads them lives in sky.cuh.
#include <cstring>
#include <new>

#include "internal.hpp"
#include "sky.cuh"

namespace mrt {
int set_error(mrt_ctx* ctx, int code, const char* msg);
}

using namespace mrt;

struct mrt_sky {
    float4* trans = nullptr;  // kTransW x kTransH
    float4* ms = nullptr;     // kMsW x kMsH
    float4* view = nullptr;   // kViewW x kViewH
    mrt_atmosphere_params atmo{};
    bool has_atmo = false, has_view = false;
    float sun[3] = {0.0f, 0.0f, 1.0f}, sun_e[3] = {0.0f, 0.0f, 0.0f};
};

namespace {

using Atmo = mrt_atmosphere_params;

MRT_DEV f3 ld3(const float* p) { return f3{p[0], p[1], p[2]}; }

// Participating medium at `p` (sky.glsl sampleMediumRGB): exponential
// Mie and Rayleigh layers plus a tent-shaped ozone layer.
struct Medium {
    f3 scat, ext, scat_mie, scat_ray;
};

MRT_DEV Medium sample_medium(const Atmo& a, f3 p) {
    const float h = fs(len3(p), a.bottom_radius);
    const float dm = exp_cw(fm(a.mie_density_exp_scale, h));
    const float dr = exp_cw(fm(a.rayleigh_density_exp_scale, h));
    const float dz = fclamp(h < a.absorption_density0_layer_width
                                ? fa(fm(a.absorption_density0_linear_term, h), a.absorption_density0_constant_term)
                                : fa(fm(a.absorption_density1_linear_term, h), a.absorption_density1_constant_term),
                            0.0f, 1.0f);
    Medium m;
    m.scat_mie = scale_rn(ld3(a.mie_scattering), dm);
    const f3 ext_mie = scale_rn(ld3(a.mie_extinction), dm);
    m.scat_ray = scale_rn(ld3(a.rayleigh_scattering), dr);
    const f3 ext_ozo = scale_rn(ld3(a.absorption_extinction), dz);
    m.scat = add_rn(m.scat_mie, m.scat_ray);
    m.ext = add_rn(add_rn(ext_mie, m.scat_ray), ext_ozo);
    return m;
}

struct March {
    f3 L, od, ms_as1;
};

// Single-scattering ray march (sky.glsl integrateScatteredLuminance).
// kVariable: 4-14 quadratically spaced samples (sky view); otherwise
// `count` uniform samples.  kMieRay: Cornette-Shanks Mie + Rayleigh phase
// (else isotropic).  kGround: light bounced off the planet when the ray
// ends on it.  trans / ms: LUTs, or nullptr for zero.
template <bool kVariable, bool kMieRay, bool kGround>
MRT_DEV March integrate(const Atmo& a, f3 pos, f3 dir, f3 sun, float count, f3 light, const float4* trans,
                        const float4* ms) {
    March r{f3s(0.0f), f3s(0.0f), f3s(0.0f)};
    const float tb = sky_sphere_nearest(pos, dir, f3s(0.0f), a.bottom_radius);
    const float tt = sky_sphere_nearest(pos, dir, f3s(0.0f), a.top_radius);
    float tmax = 0.0f;
    if (tb < 0.0f) {
        if (tt < 0.0f) return r;
        tmax = tt;
    } else if (tt > 0.0f) {
        tmax = fminf(tt, tb);
    }
    tmax = fminf(tmax, 9000000.0f);

    float n = count, nfloor = count, tmax_floor = tmax;
    if (kVariable) {
        const float w = fclamp(fm(tmax, 0.01f), 0.0f, 1.0f);
        n = fa(fm(4.0f, fs(1.0f, w)), fm(14.0f, w));
        nfloor = floorf(n);
        tmax_floor = fd(fm(tmax, nfloor), n);
    }
    const float cos_t = dot_rn(sun, dir);
    const float g = a.mie_phase_g;
    // Cornette-Shanks with the negated angle (dir is an "in" direction)
    const float k = fd(fm(fd(3.0f, fm(8.0f, kSkyPi)), fs(1.0f, fm(g, g))), fa(2.0f, fm(g, g)));
    const float mie_phase = fd(fm(k, fa(1.0f, fm(cos_t, cos_t))),
                               powf(fs(fa(1.0f, fm(g, g)), fm(fm(2.0f, g), cos_t)), 1.5f));
    const float ray_phase = fm(fd(3.0f, fm(16.0f, kSkyPi)), fa(1.0f, fm(cos_t, cos_t)));
    const float uni_phase = fd(1.0f, fm(4.0f, kSkyPi));

    f3 thr = f3s(1.0f);
    float t = 0.0f, dt = 0.0f;
    for (float s = 0.0f; s < n; s = fa(s, 1.0f)) {
        if (kVariable) {
            float t0 = fd(s, nfloor), t1 = fd(fa(s, 1.0f), nfloor);
            t0 = fm(t0, t0);
            t1 = fm(t1, t1);
            t0 = fm(tmax_floor, t0);
            t1 = t1 > 1.0f ? tmax : fm(tmax_floor, t1);
            t = fa(t0, fm(fs(t1, t0), 0.3f));
            dt = fs(t1, t0);
        } else {
            const float nt = fd(fm(tmax, fa(s, 0.3f)), n);
            dt = fs(nt, t);
            t = nt;
        }
        const f3 P = add_rn(pos, scale_rn(dir, t));
        const Medium m = sample_medium(a, P);
        const f3 sod = scale_rn(m.ext, dt);
        const f3 st = exp3(f3{-sod.x, -sod.y, -sod.z});
        r.od = add_rn(r.od, sod);
        const float ph = len3(P);
        const f3 up = div3s(P, ph);
        const float sun_zen = dot_rn(sun, up);
        f3 t_sun = f3s(0.0f);
        if (trans) {
            float u, v;
            trans_uv(ph, sun_zen, a.bottom_radius, a.top_radius, u, v);
            t_sun = lut_sample(trans, kTransW, kTransH, u, v);
        }
        const f3 pts = kMieRay ? add_rn(scale_rn(m.scat_mie, mie_phase), scale_rn(m.scat_ray, ray_phase))
                               : scale_rn(m.scat, uni_phase);
        const float te = sky_sphere_nearest(P, sun, scale_rn(up, kPlanetOffset), a.bottom_radius);
        const float shadow = te >= 0.0f ? 0.0f : 1.0f;
        f3 msl = f3s(0.0f);
        if (ms) {
            const float mu = fclamp(fa(fm(sun_zen, 0.5f), 0.5f), 0.0f, 1.0f);
            const float mv = fclamp(fd(fs(ph, a.bottom_radius), fs(a.top_radius, a.bottom_radius)), 0.0f, 1.0f);
            msl = lut_sample(ms, kMsW, kMsH, unit_to_sub(mu, float(kMsW)), unit_to_sub(mv, float(kMsH)));
        }
        const f3 S = mul_rn(light, add_rn(mul_rn(scale_rn(t_sun, shadow), pts), mul_rn(msl, m.scat)));
        const f3 msint = div3(sub_rn(m.scat, mul_rn(m.scat, st)), m.ext);
        r.ms_as1 = add_rn(r.ms_as1, mul_rn(thr, msint));
        const f3 sint = div3(sub_rn(S, mul_rn(S, st)), m.ext);
        r.L = add_rn(r.L, mul_rn(thr, sint));
        thr = mul_rn(thr, st);
    }
    if (kGround && tmax == tb && tb > 0.0f) {
        const f3 P = add_rn(pos, scale_rn(dir, tb));
        const float ph = len3(P);
        const f3 up = div3s(P, ph);
        float u, v;
        trans_uv(ph, dot_rn(sun, up), a.bottom_radius, a.top_radius, u, v);
        const f3 t_sun = trans ? lut_sample(trans, kTransW, kTransH, u, v) : f3s(0.0f);
        const float ndl = fclamp(dot_rn(normalize_rn(up), normalize_rn(sun)), 0.0f, 1.0f);
        const f3 gl = mul_rn(scale_rn(mul_rn(mul_rn(light, t_sun), thr), ndl), ld3(a.ground_albedo));
        r.L = add_rn(r.L, div3s(gl, kSkyPi));
    }
    return r;
}

// genTransmittance.comp:21-44: exp(-optical depth) from each (height,
// zenith angle) to the top of the atmosphere, 40 uniform steps.
__global__ void __launch_bounds__(256) k_sky_transmittance(Atmo a, float4* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kTransW * kTransH) return;
    const uint32_t x = i % kTransW, y = i / kTransW;
    const float u = fd(fa(float(x), 0.5f), float(kTransW)), v = fd(fa(float(y), 0.5f), float(kTransH));
    float h, mu;
    trans_params(u, v, a.bottom_radius, a.top_radius, h, mu);
    const f3 pos{0.0f, 0.0f, h};
    const f3 dir{0.0f, __fsqrt_rn(fs(1.0f, fm(mu, mu))), mu};
    const March m = integrate<false, false, false>(a, pos, dir, f3s(1.0f), 40.0f, f3s(1.0f), nullptr, nullptr);
    out[i] = make_float4(exp_cw(-m.od.x), exp_cw(-m.od.y), exp_cw(-m.od.z), 1.0f);
}

// genMultiScattering.comp:26-146: per (sun zenith, height) texel, second-
// order luminance and the multi-scattering transfer over 8x8 sphere
// directions, folded into the truncated power series 1 + r + ... + r^4.
__global__ void __launch_bounds__(64) k_sky_multiscatter(Atmo a, const float4* trans, float4* out) {
    __shared__ f3 s_ms[64], s_l[64];
    const uint32_t x = blockIdx.x % kMsW, y = blockIdx.x / kMsW, z = threadIdx.x;
    float u = fd(fa(float(x), 0.5f), float(kMsW)), v = fd(fa(float(y), 0.5f), float(kMsH));
    u = sub_to_unit(u, float(kMsW));
    v = sub_to_unit(v, float(kMsH));
    const float cs = fs(fm(u, 2.0f), 1.0f);
    const f3 sun{0.0f, __fsqrt_rn(fclamp(fs(1.0f, fm(cs, cs)), 0.0f, 1.0f)), cs};
    const float h = fa(a.bottom_radius, fm(fclamp(fa(v, kPlanetOffset), 0.0f, 1.0f),
                                           fs(fs(a.top_radius, a.bottom_radius), kPlanetOffset)));
    const float sphere = fm(4.0f, kSkyPi);
    const float iv = fa(0.5f, float(z / 8u)), jv = fa(0.5f, float(z % 8u));
    const float theta = fm(fm(2.0f, kSkyPi), fd(iv, 8.0f)), phi = fm(kSkyPi, fd(jv, 8.0f));
    const float cp = cosf(phi), sp = sinf(phi), ct = cosf(theta), st = sinf(theta);
    const f3 dir{fm(ct, sp), fm(st, sp), cp};
    const March m = integrate<false, false, true>(a, f3{0.0f, 0.0f, h}, dir, sun, 20.0f, f3s(1.0f), trans, nullptr);
    s_ms[z] = div3s(scale_rn(m.ms_as1, sphere), 64.0f);
    s_l[z] = div3s(scale_rn(m.L, sphere), 64.0f);
    __syncthreads();
#pragma unroll
    for (uint32_t half = 32; half >= 1; half >>= 1) {
        if (z < half) {
            s_ms[z] = add_rn(s_ms[z], s_ms[z + half]);
            s_l[z] = add_rn(s_l[z], s_l[z + half]);
        }
        __syncthreads();
    }
    if (z != 0) return;
    const float iso = fd(1.0f, sphere);
    const f3 r = scale_rn(s_ms[0], iso);
    const f3 L1 = scale_rn(s_l[0], iso);
    const f3 r2 = mul_rn(r, r);
    const f3 series = add_rn(add_rn(add_rn(add_rn(f3s(1.0f), r), r2), mul_rn(r, r2)), mul_rn(r2, r2));
    const f3 L = mul_rn(L1, series);
    out[blockIdx.x] = make_float4(L.x, L.y, L.z, 1.0f);
}

// genView.comp:33-77: sky luminance around a probe, parameterised by view
// zenith and light-view azimuth (sun rotated into the x-z plane).
__global__ void __launch_bounds__(128) k_sky_view(Atmo a, const float4* trans, const float4* ms, f3 probe, f3 sun_w,
                                                  f3 light, float4* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kViewW * kViewH) return;
    const uint32_t x = i % kViewW, y = i / kViewW;
    f3 pos = f3{probe.x, probe.y, fa(probe.z, a.bottom_radius)};
    const float u = fd(float(x), float(kViewW)), v = fd(float(y), float(kViewH));
    const float h = len3(pos);
    float mu, lv;
    view_params(u, v, h, a.bottom_radius, mu, lv);
    const f3 up = div3s(pos, h);
    const float sz = dot_rn(up, sun_w);
    const f3 sun = normalize_rn(f3{__fsqrt_rn(fs(1.0f, fm(sz, sz))), 0.0f, sz});
    pos = f3{0.0f, 0.0f, h};
    const float sv = __fsqrt_rn(fs(1.0f, fm(mu, mu)));
    const f3 dir{fm(sv, lv), fm(sv, __fsqrt_rn(fs(1.0f, fm(lv, lv)))), mu};
    // moveToTopAtmosphere (sky.glsl)
    if (h > a.top_radius) {
        const float ttop = sky_sphere_nearest(pos, dir, f3s(0.0f), a.top_radius);
        if (!(ttop >= 0.0f)) {
            out[i] = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
            return;
        }
        const f3 upo = scale_rn(div3s(pos, h), -kPlanetOffset);
        pos = add_rn(add_rn(pos, scale_rn(dir, ttop)), upo);
    }
    const March m = integrate<true, true, false>(a, pos, dir, sun, 30.0f, light, trans, ms);
    out[i] = make_float4(m.L.x, m.L.y, m.L.z, 1.0f);
}

__global__ void k_sky_eval(SkyDev s, const float* dirs, uint32_t n, float* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const f3 c = sky_color(s, f3{dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]});
    out[3 * i] = c.x;
    out[3 * i + 1] = c.y;
    out[3 * i + 2] = c.z;
}

cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }

}  // namespace

namespace mrt {
// Miss-shader state of a bound sky for a camera at `cam`; view = nullptr
// when no sky is bound or its view has not been built.
SkyDev sky_dev(const mrt_sky* s, const float cam[3]) {
    SkyDev d{};
    if (!s || !s->has_view) return d;
    d.view = s->view;
    d.trans = s->trans;
    d.bottom = s->atmo.bottom_radius;
    d.top = s->atmo.top_radius;
    for (int k = 0; k < 3; ++k) {
        d.sun[k] = s->sun[k];
        d.sun_e[k] = s->sun_e[k];
        d.cam[k] = cam[k];
    }
    return d;
}
}  // namespace mrt

extern "C" {

void mrt_atmosphere_earth(mrt_atmosphere_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    // sky.ixx:59-83 (kilometres)
    p->bottom_radius = 6360.0f;
    p->top_radius = 6460.0f;
    p->rayleigh_density_exp_scale = -1.0f / 8.0f;
    p->rayleigh_scattering[0] = 0.005802f;
    p->rayleigh_scattering[1] = 0.013558f;
    p->rayleigh_scattering[2] = 0.033100f;
    p->mie_density_exp_scale = -1.0f / 1.2f;
    for (int k = 0; k < 3; ++k) {
        p->mie_scattering[k] = 0.003996f;
        p->mie_extinction[k] = 0.004440f;
        p->mie_absorption[k] = p->mie_extinction[k] - p->mie_scattering[k] > 0.0f
                                   ? p->mie_extinction[k] - p->mie_scattering[k]
                                   : 0.0f;
    }
    p->mie_phase_g = 0.8f;
    p->absorption_density0_layer_width = 25.0f;
    p->absorption_density0_constant_term = -2.0f / 3.0f;
    p->absorption_density0_linear_term = 1.0f / 15.0f;
    p->absorption_density1_constant_term = 8.0f / 3.0f;
    p->absorption_density1_linear_term = -1.0f / 15.0f;
    p->absorption_extinction[0] = 0.000650f;
    p->absorption_extinction[1] = 0.001881f;
    p->absorption_extinction[2] = 0.000085f;
}

int mrt_cuda_sky_create(mrt_ctx* ctx, mrt_sky** out) {
    if (!ctx || !out) return set_error(ctx, MRT_EINVAL, "sky_create: null argument");
    *out = nullptr;
    cudaSetDevice(ctx->device);
    mrt_sky* s = new (std::nothrow) mrt_sky;
    if (!s) return set_error(ctx, MRT_ENOMEM, "sky_create: host allocation");
    if (cudaMalloc(&s->trans, kTransW * kTransH * sizeof(float4)) != cudaSuccess ||
        cudaMalloc(&s->ms, kMsW * kMsH * sizeof(float4)) != cudaSuccess ||
        cudaMalloc(&s->view, kViewW * kViewH * sizeof(float4)) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(s->trans); cudaFree(s->ms); cudaFree(s->view);
        delete s;
        return set_error(ctx, MRT_ENOMEM, "sky_create: LUT allocation");
    }
    *out = s;
    return MRT_OK;
}

int mrt_cuda_sky_destroy(mrt_ctx* ctx, mrt_sky* s) {
    if (!s) return MRT_OK;
    if (ctx) {
        cudaSetDevice(ctx->device);
        if (ctx->sky == s) ctx->sky = nullptr;
    }
    cudaFree(s->trans); cudaFree(s->ms); cudaFree(s->view);
    delete s;
    return MRT_OK;
}

int mrt_cuda_sky_atmosphere(mrt_ctx* ctx, mrt_sky* s, const mrt_atmosphere_params* p, void* stream) {
    if (!ctx || !s || !p) return set_error(ctx, MRT_EINVAL, "sky_atmosphere: null argument");
    if (!(p->bottom_radius > 0.0f) || !(p->top_radius > p->bottom_radius + kPlanetOffset))
        return set_error(ctx, MRT_EINVAL, "sky_atmosphere: need 0 < bottom_radius < top_radius");
    cudaSetDevice(ctx->device);
    const cudaStream_t st = as_stream(stream);
    k_sky_transmittance<<<(kTransW * kTransH + 255) / 256, 256, 0, st>>>(*p, s->trans);
    k_sky_multiscatter<<<kMsW * kMsH, 64, 0, st>>>(*p, s->trans, s->ms);
    if (cudaGetLastError() != cudaSuccess) return set_error(ctx, MRT_ECUDA, "sky_atmosphere: launch");
    ctx->launches += 2;
    s->atmo = *p;
    s->has_atmo = true;
    s->has_view = false;
    return MRT_OK;
}

int mrt_cuda_sky_view(mrt_ctx* ctx, mrt_sky* s, const float probe_pos[3], const float sun_dir[3],
                      const float sun_illuminance[3], void* stream) {
    if (!ctx || !s || !probe_pos || !sun_dir || !sun_illuminance)
        return set_error(ctx, MRT_EINVAL, "sky_view: null argument");
    if (!s->has_atmo) return set_error(ctx, MRT_EINVAL, "sky_view: atmosphere LUTs not built");
    cudaSetDevice(ctx->device);
    const f3 probe{probe_pos[0], probe_pos[1], probe_pos[2]};
    const f3 sun{sun_dir[0], sun_dir[1], sun_dir[2]};
    const f3 light{sun_illuminance[0], sun_illuminance[1], sun_illuminance[2]};
    k_sky_view<<<(kViewW * kViewH + 127) / 128, 128, 0, as_stream(stream)>>>(s->atmo, s->trans, s->ms, probe, sun,
                                                                            light, s->view);
    if (cudaGetLastError() != cudaSuccess) return set_error(ctx, MRT_ECUDA, "sky_view: launch");
    ctx->launches++;
    for (int k = 0; k < 3; ++k) {
        s->sun[k] = sun_dir[k];
        s->sun_e[k] = sun_illuminance[k];
    }
    s->has_view = true;
    return MRT_OK;
}

int mrt_cuda_sky_lut(mrt_ctx* ctx, const mrt_sky* s, int which, float* host_rgba, size_t count) {
    if (!ctx || !s || !host_rgba) return set_error(ctx, MRT_EINVAL, "sky_lut: null argument");
    const float4* src = which == 0 ? s->trans : which == 1 ? s->ms : which == 2 ? s->view : nullptr;
    const size_t n = which == 0 ? kTransW * kTransH : which == 1 ? kMsW * kMsH : kViewW * kViewH;
    if (!src) return set_error(ctx, MRT_EINVAL, "sky_lut: which must be 0, 1 or 2");
    if (count < n * 4) return set_error(ctx, MRT_ERANGE, "sky_lut: host buffer too small");
    cudaSetDevice(ctx->device);
    if (cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(host_rgba, src, n * sizeof(float4), cudaMemcpyDeviceToHost) != cudaSuccess)
        return set_error(ctx, MRT_ECUDA, "sky_lut: copy");
    return MRT_OK;
}

int mrt_cuda_sky_eval(mrt_ctx* ctx, const mrt_sky* s, const float camera_pos[3], const float* dirs, uint32_t n,
                      float* out_rgb, void* stream) {
    if (!ctx || !s || !camera_pos || (n && (!dirs || !out_rgb)))
        return set_error(ctx, MRT_EINVAL, "sky_eval: null argument");
    if (!s->has_view) return set_error(ctx, MRT_EINVAL, "sky_eval: sky view not built");
    if (n == 0) return MRT_OK;
    cudaSetDevice(ctx->device);
    k_sky_eval<<<(n + 127) / 128, 128, 0, as_stream(stream)>>>(sky_dev(s, camera_pos), dirs, n, out_rgb);
    if (cudaGetLastError() != cudaSuccess) return set_error(ctx, MRT_ECUDA, "sky_eval: launch");
    ctx->launches++;
    return MRT_OK;
}

int mrt_cuda_set_sky(mrt_ctx* ctx, const mrt_sky* s) {
    if (!ctx) return MRT_EINVAL;
    if (s && !s->has_view) return set_error(ctx, MRT_EINVAL, "set_sky: sky view not built");
    ctx->sky = s;
    return MRT_OK;
}

}  // extern "C"
