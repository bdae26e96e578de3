// Ray-tracing kernels for sm_103a.
//
//   k_primary_tri / k_primary_sphere    primaryRay.comp:38-76 (pinhole ray,
//                                       closest hit, g-buffer stores)
//   k_secondary_sphere                  secondaryRays.comp:64-135 (the
//                                       reference's per-pixel sample/bounce
//                                       loop over analytic spheres)
//   k_shade_primary / k_shade           wavefront shade: throughput x albedo,
//   k_trace_ext / k_trace_shadow        cosine-weighted blue-noise-rotated
//   k_finalize                          bounce (secondaryRays.comp:60-72,
//                                       94-96), directional-light shadow
//                                       rays, compaction, accumulation
//   k_trace_rays                        generic closest/any-hit queries
#include "internal.hpp"

#include <cfloat>

namespace mrt {


// g-buffer extras: depth = (P V hit).z / w as R16F, normal RGBA16F (the ray
// direction on a miss), motion = (proj - prev proj).xy / pitch as RG16F
// (primaryRay.comp:62-75).  A miss (undefined in the reference) stores
// depth 0 and motion 0.
MRT_DEV void store_extras(const FrameParams& fp, const mrt_gbuffer& g, size_t pi, bool hit, f3 pos, f3 n) {
    float depth = 0.0f, mx = 0.0f, my = 0.0f;
    if (hit && (g.depth || g.motion)) {
        float ph[4], pp[4];
        matvec_rn(fp.pv, pos.x, pos.y, pos.z, 1.0f, ph);
        const float px = __fdiv_rn(ph[0], ph[3]), py = __fdiv_rn(ph[1], ph[3]);
        depth = __fdiv_rn(ph[2], ph[3]);
        if (g.motion) {
            matvec_rn(fp.ppv, pos.x, pos.y, pos.z, 1.0f, pp);
            const float qx = __fdiv_rn(pp[0], pp[3]), qy = __fdiv_rn(pp[1], pp[3]);
            mx = __fdiv_rn(__fsub_rn(px, qx), fp.pitch_x);
            my = __fdiv_rn(__fsub_rn(py, qy), fp.pitch_y);
        }
    }
    if (g.depth) g.depth[pi] = f2h(depth);
    if (g.normal) {
        ushort4 v = make_ushort4(f2h(n.x), f2h(n.y), f2h(n.z), f2h(0.0f));
        reinterpret_cast<ushort4*>(g.normal)[pi] = v;
    }
    if (g.motion) reinterpret_cast<ushort2*>(g.motion)[pi] = make_ushort2(f2h(mx), f2h(my));
}

// Material of original triangle `prim`; an out-of-range id (corrupt scene
// data) raises MRT_STATUS_BAD_TRI and shades as black.
MRT_DEV mrt_material load_mat(const DevScene& sc, uint32_t prim, uint32_t* status) {
    if (prim < sc.mat_count) return sc.mats[prim];
    atomicOr(status, MRT_STATUS_BAD_TRI);
    mrt_material m;
    m.normal[0] = 0.0f; m.normal[1] = 0.0f; m.normal[2] = 1.0f;
    m.albedo_rgba8 = 0u;
    return m;
}

MRT_DEV f3 facing_normal(const mrt_material& m, f3 d) {
    f3 n{m.normal[0], m.normal[1], m.normal[2]};
    if (dot_rn(n, d) > 0.0f) n = f3{-n.x, -n.y, -n.z};
    return n;
}

// Pixel of thread: blocks of 16x8 pixels, each warp an 8x4 tile.
MRT_DEV bool tile_pixel(uint32_t w, uint32_t h, uint32_t& x, uint32_t& y) {
    const uint32_t wi = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    x = blockIdx.x * 16u + (wi & 1u) * 8u + (lane & 7u);
    y = blockIdx.y * 8u + (wi >> 1) * 4u + (lane >> 3);
    return x < w && y < h;
}

// kSpread: the warp steps its 32 rays together with the triangle tests of
// each step spread over its lanes (trav_step_spread).
template <bool kCount, bool kSpread = false>
__global__ void __launch_bounds__(kTraceBlock, kTraceMinBlocks)
k_primary_tri(DevScene sc, FrameParams fp, mrt_gbuffer g, uint32_t* status, unsigned long long* totals) {
    __shared__ uint2 stk[kStackDepth * kTraceBlock];
    __shared__ unsigned long long slots[kSpread ? kTraceBlock : 1];
    uint32_t x, y;
    const bool inside = tile_pixel(fp.width, fp.height, x, y);
    if (!kSpread && !inside) return;
    if (kSpread && !__any_sync(0xFFFFFFFFu, inside)) return;  // warp-uniform
    f3 o{0.0f, 0.0f, 0.0f}, d{0.0f, 0.0f, 1.0f};
    if (inside) primary_ray(fp, x, y, o, d);
    uint32_t prim, st = 0u, cn = 0u, ct = 0u;
    float t;
    if (kSpread) {
        Trav s{};
        trav_init(s, o, d, 0.0f, INFINITY);
        bool have = inside;
        while (__any_sync(0xFFFFFFFFu, have)) {
            if (trav_step_spread<false, kStackDepth>(sc, s, have, stk + threadIdx.x, kTraceBlock, st,
                                                     slots + (threadIdx.x & ~31u)))
                have = false;
        }
        prim = s.best;
        t = prim == kMiss ? s.tmax : s.tbest;
    } else {
        trace_bvh8<false, kCount, kStackDepth>(sc, o, d, 0.0f, INFINITY, prim, t, stk + threadIdx.x, kTraceBlock,
                                               st, cn, ct);
    }
    if (st) atomicOr(status, st);  // (a lane outside the image may have tested another lane's triangle)
    if (kCount) {
        atomicAdd(totals + kTotNodesPrim, (unsigned long long)cn);
        atomicAdd(totals + kTotTrisPrim, (unsigned long long)ct);
    }
    if (!inside) return;
    const size_t pi = size_t(y) * fp.width + x;
    g.visibility[pi] = prim;
    if (g.hit_t) g.hit_t[pi] = t;
    if (g.depth || g.normal || g.motion) {
        const bool hit = prim != kMiss;
        f3 pos = o, n = d;
        if (hit) {
            pos = ray_at(o, d, t);
            n = facing_normal(load_mat(sc, prim, status), d);
        }
        store_extras(fp, g, pi, hit, pos, n);
    }
}

MRT_DEV uint32_t warp_refill(uint32_t* fetch, uint32_t n, bool need, bool& exhausted,
                             uint32_t min_idle = 1u);

// Persistent primary rays with per-lane refill.  Ray index i maps to pixel
// tile i/32 (8x4 pixels, row-major tiles) and lane i%32 inside it, so the
// rays a warp fetches together are neighbours.
template <bool kCount>
__global__ void __launch_bounds__(kTraceBlock, kTraceMinBlocks)
k_primary_tri_dyn(DevScene sc, FrameParams fp, mrt_gbuffer g, uint32_t* status, unsigned long long* totals,
                  uint32_t* fetch, uint32_t refill_min) {
    __shared__ uint2 stk[kStackDepth * kTraceBlock];
    const uint32_t tiles_x = (fp.width + 7u) / 8u, tiles_y = (fp.height + 3u) / 4u;
    const uint32_t n = tiles_x * tiles_y * 32u;
    uint2* my = stk + threadIdx.x;
    uint32_t st = 0u, cn = 0u, ct = 0u, px = 0u, py = 0u;
    Trav s;
    bool have = false, exhausted = false;
    while (true) {
        const uint32_t idx = warp_refill(fetch, n, !have, exhausted, refill_min);
        if (idx != kMiss) {
            const uint32_t tile = idx >> 5, l = idx & 31u;
            const uint32_t x = (tile % tiles_x) * 8u + (l & 7u), y = (tile / tiles_x) * 4u + (l >> 3);
            if (x < fp.width && y < fp.height) {
                f3 o, d;
                primary_ray(fp, x, y, o, d);
                trav_init(s, o, d, 0.0f, INFINITY);
                px = x;
                py = y;
                have = true;
            }
        }
        const bool any = __any_sync(0xFFFFFFFFu, have);
        if (!any && exhausted) break;
        if (have && trav_step<false, kCount, kStackDepth>(sc, s, my, kTraceBlock, st, cn, ct)) {
            have = false;
            const uint32_t prim = s.best;
            const float t = prim == kMiss ? s.tmax : s.tbest;
            const size_t pi = size_t(py) * fp.width + px;
            g.visibility[pi] = prim;
            if (g.hit_t) g.hit_t[pi] = t;
            if (g.depth || g.normal || g.motion) {
                f3 o, d;
                primary_ray(fp, px, py, o, d);
                const bool hit = prim != kMiss;
                f3 pos = o, nrm = d;
                if (hit) {
                    pos = ray_at(o, d, t);
                    nrm = facing_normal(load_mat(sc, prim, status), d);
                }
                store_extras(fp, g, pi, hit, pos, nrm);
            }
        }
    }
    if (st) atomicOr(status, st);
    if (kCount) {
        atomicAdd(totals + kTotNodesPrim, (unsigned long long)cn);
        atomicAdd(totals + kTotTrisPrim, (unsigned long long)ct);
    }
}

MRT_DEV void sphere_at(const DevScene& sc, uint32_t i, f3& c, float& r) {
    const float4 s = sc.spheres[2 * i];
    c = f3{s.x, s.y, s.z};
    r = s.w;
}

__global__ void __launch_bounds__(128) k_primary_sphere(DevScene sc, FrameParams fp, mrt_gbuffer g) {
    uint32_t x, y;
    if (!tile_pixel(fp.width, fp.height, x, y)) return;
    f3 o, d;
    primary_ray(fp, x, y, o, d);
    // tracePrimaryRay (primaryRay.comp:23-36): first nearest t >= 0
    uint32_t prim = kMiss;
    float tb = 0.0f;
    for (uint32_t i = 0; i < sc.sphere_count; ++i) {
        f3 c; float r;
        sphere_at(sc, i, c, r);
        const float t = ray_sphere(o, d, c, r);
        if (t >= 0.0f && (prim == kMiss || t < tb)) { tb = t; prim = i; }
    }
    const size_t pi = size_t(y) * fp.width + x;
    g.visibility[pi] = prim;
    const bool hit = prim != kMiss;
    if (g.hit_t) g.hit_t[pi] = hit ? tb : INFINITY;
    f3 pos = o, n = d;
    if (hit) {
        f3 c; float r;
        sphere_at(sc, prim, c, r);
        pos = ray_at(o, d, tb);
        n = normalize_rn(sub_rn(pos, c));
    }
    store_extras(fp, g, pi, hit, pos, n);
}

MRT_DEV uint32_t initial_seed(uint32_t mode, uint32_t frame, uint32_t pixel) {
    uint32_t s = (frame << 1u) | 1u; // secondaryRays.comp:124
    if (mode == MRT_RNG_PER_PIXEL) {
        uint32_t h = pixel * 0x9E3779B1u + s;
        s = pcg(h) | 1u;
    }
    return s;
}

MRT_DEV float2 bn_rot(const BlueNoise& bn, uint32_t x, uint32_t y) { return bn.rot[(y % bn.h) * bn.w + (x % bn.w)]; }

// secondaryRays.comp:102-135 with the reference's sample/bounce loop.
// skyColor() is the bound atmosphere (sky.cuh) or a constant radiance.
__global__ void __launch_bounds__(128)
k_secondary_sphere(DevScene sc, FrameParams fp, mrt_gbuffer g, TraceParams tp, BlueNoise bn, float* color,
                   uint32_t accumulate, uint32_t frame_index) {
    uint32_t x, y;
    if (!tile_pixel(fp.width, fp.height, x, y)) return;
    const size_t pi = size_t(y) * fp.width + x;
    const float uvx = __fmul_rn(__fadd_rn(float(x), 0.5f), fp.pitch_x);
    const float uvy = __fsub_rn(1.0f, __fmul_rn(__fadd_rn(float(y), 0.5f), fp.pitch_y));
    // reconstruct the primary hit from the g-buffer (:114-123)
    const uint32_t prim0 = g.visibility[pi];
    const ushort4 nh = reinterpret_cast<const ushort4*>(g.normal)[pi];
    const f3 n0{h2f(nh.x), h2f(nh.y), h2f(nh.z)};
    const float depth = h2f(g.depth[pi]);
    float vp[4], wp[4];
    matvec_rn(fp.c.inv_projection, __fsub_rn(__fmul_rn(uvx, 2.0f), 1.0f), __fsub_rn(__fmul_rn(uvy, 2.0f), 1.0f),
              depth, 1.0f, vp);
    vp[0] = __fdiv_rn(vp[0], vp[3]);
    vp[1] = __fdiv_rn(vp[1], vp[3]);
    vp[2] = __fdiv_rn(vp[2], vp[3]);
    matvec_rn(fp.c.inv_view, vp[0], vp[1], vp[2], 1.0f, wp);
    const f3 p0{wp[0], wp[1], wp[2]};
    uint32_t rng = initial_seed(tp.rng_mode, fp.c.frame_counter, uint32_t(pi));
    const float2 rot = bn_rot(bn, x, y);

    f3 acc{0.0f, 0.0f, 0.0f};
    for (uint32_t s = 0; s < tp.samples; ++s) {
        // traceSecondaryRays (:64-100)
        f3 col{1.0f, 1.0f, 1.0f}, hp = p0, hn = n0, res{0.0f, 0.0f, 0.0f};
        uint32_t hprim = prim0;
        for (uint32_t i = 0; i < tp.max_bounces + 1u; ++i) {
            if (i > 0) {
                const f3 ro = add_rn(hp, scale_rn(hn, 0.000001f));
                const float u1 = rotated_random(rng, rot.x);
                const float u2 = rotated_random(rng, rot.y);
                const f3 sp = random_sphere_point(__fsub_rn(__fmul_rn(u1, 2.0f), 1.0f),
                                                  __fsub_rn(__fmul_rn(u2, 2.0f), 1.0f), tp.exact_trig);
                const f3 rd = normalize_rn(add_rn(hn, sp));
                hprim = kMiss;
                float ht = -1.0f;
                for (uint32_t k = 0; k < sc.sphere_count; ++k) {
                    f3 c; float r;
                    sphere_at(sc, k, c, r);
                    const float t = ray_sphere(ro, rd, c, r);
                    if (t >= 0.0f && (t < ht || ht < 0.0f)) { hprim = k; ht = t; }
                }
                if (hprim != kMiss) {
                    f3 c; float r;
                    sphere_at(sc, hprim, c, r);
                    hp = ray_at(ro, rd, ht);
                    hn = normalize_rn(sub_rn(hp, c));
                } else {
                    hn = rd;
                }
            }
            if (hprim != kMiss) {
                const float4 al = sc.spheres[2 * hprim + 1];
                col = mul_rn(col, f3{al.x, al.y, al.z});
            } else {
                res = mul_rn(col, escape_radiance(tp, hn));
                break;
            }
        }
        acc = add_rn(acc, res);
    }
    const float ns = float(tp.samples);
    f3 mean{__fdiv_rn(acc.x, ns), __fdiv_rn(acc.y, ns), __fdiv_rn(acc.z, ns)};
    float* out = color + pi * 3;
    if (accumulate && frame_index > 0u) {  // frame 0 starts the mean: old contents are ignored
        const float w = float(frame_index + 1u);
        mean.x = __fadd_rn(out[0], __fdiv_rn(__fsub_rn(mean.x, out[0]), w));
        mean.y = __fadd_rn(out[1], __fdiv_rn(__fsub_rn(mean.y, out[1]), w));
        mean.z = __fadd_rn(out[2], __fdiv_rn(__fsub_rn(mean.z, out[2]), w));
    }
    out[0] = mean.x;
    out[1] = mean.y;
    out[2] = mean.z;
}

// ---------------------------------------------------------------- wavefront


struct VertexOut {
    bool shadow;
    bool ext;
    ShadowRay sr;
    PathRay pr;
};

// Shade one path vertex: directional-light shadow ray (MRT_EST_NEE),
// throughput *= albedo (secondaryRays.comp:94), next cosine-weighted
// direction normalize(n + uniformSpherePoint) with blue-noise-rotated PCG
// numbers (:70-72), Russian roulette on bounces > rr_start.
MRT_DEV VertexOut shade_vertex(const DevScene& sc, const TraceParams& tp, const BlueNoise& bn, uint32_t width,
                               uint32_t vertex, uint32_t pix, f3 p, f3 d, uint32_t prim, f3 beta, uint32_t& rng,
                               uint32_t* status) {
    VertexOut vo;
    vo.shadow = false;
    vo.ext = false;
    const mrt_material m = load_mat(sc, prim, status);
    const f3 n = facing_normal(m, d);
    const f3 rho{__fdiv_rn(float(m.albedo_rgba8 & 0xFFu), 255.0f),
                 __fdiv_rn(float((m.albedo_rgba8 >> 8) & 0xFFu), 255.0f),
                 __fdiv_rn(float((m.albedo_rgba8 >> 16) & 0xFFu), 255.0f)};
    if (tp.estimator == MRT_EST_NEE) {
        const f3 sun{tp.sun[0], tp.sun[1], tp.sun[2]};
        const float cosl = dot_rn(n, sun);
        if (cosl > 0.0f) {
            const f3 os = offset_ray(p, n);
            const float k = __fmul_rn(cosl, kInvPi);
            const f3 c = scale_rn(mul_rn(mul_rn(beta, rho), f3{tp.sun_e[0], tp.sun_e[1], tp.sun_e[2]}), k);
            vo.shadow = true;
            vo.sr.o_pix = make_float4(os.x, os.y, os.z, __uint_as_float(pix));
            vo.sr.contrib = make_float4(c.x, c.y, c.z, 0.0f);
        }
    }
    beta = mul_rn(beta, rho);
    if (vertex >= tp.max_bounces) return vo;
    const float2 rot = bn_rot(bn, pix % width, pix / width);
    const float u1 = rotated_random(rng, rot.x);
    const float u2 = rotated_random(rng, rot.y);
    const f3 sp = random_sphere_point(__fsub_rn(__fmul_rn(u1, 2.0f), 1.0f), __fsub_rn(__fmul_rn(u2, 2.0f), 1.0f),
                                      tp.exact_trig);
    f3 nd = add_rn(n, sp);
    if (dot_rn(nd, nd) == 0.0f) nd = n;
    nd = normalize_rn(nd);
    if (tp.rr_start != 0u && vertex + 1u > tp.rr_start) {
        float q = fmaxf(fmaxf(beta.x, beta.y), beta.z);
        q = fminf(fmaxf(q, 0.05f), 1.0f);
        const float u3 = rotated_random(rng, rot.x);
        if (u3 >= q) return vo;
        beta = f3{__fdiv_rn(beta.x, q), __fdiv_rn(beta.y, q), __fdiv_rn(beta.z, q)};
    }
    const f3 oe = offset_ray(p, n);
    vo.ext = true;
    vo.pr.o_pix = make_float4(oe.x, oe.y, oe.z, __uint_as_float(pix));
    vo.pr.d = make_float4(nd.x, nd.y, nd.z, 0.0f);
    vo.pr.beta = make_float4(beta.x, beta.y, beta.z, 0.0f);
    return vo;
}

MRT_DEV void add_L(float4* L, uint32_t pix, f3 v) {
    float4 a = L[pix];
    a.x = __fadd_rn(a.x, v.x);
    a.y = __fadd_rn(a.y, v.y);
    a.z = __fadd_rn(a.z, v.z);
    L[pix] = a;
}


// emit for a whole block: the shadow and extension rays of the block's
// threads get their queue slots with one global atomic per queue and block
// instead of one per warp (the shading kernels' warps otherwise queue on
// the two counters' atomics).  All threads of the block must call it the
// same number of times.
MRT_DEV void emit_block(const VertexOut& vo, const WaveBuffers& wb, uint32_t vertex) {
    constexpr int kWarps = kShadeBlock / 32;
    __shared__ uint32_t wsum[2][kWarps];
    __shared__ uint32_t base[2];
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    const uint32_t m0 = __ballot_sync(0xFFFFFFFFu, vo.shadow), m1 = __ballot_sync(0xFFFFFFFFu, vo.ext);
    if (lane == 0u) {
        wsum[0][warp] = __popc(m0);
        wsum[1][warp] = __popc(m1);
    }
    __syncthreads();
    if (threadIdx.x < 2u) {  // thread q: exclusive scan of the warps' counts of queue q, one atomic
        const uint32_t q = threadIdx.x;
        uint32_t acc = 0u;
        for (int w = 0; w < kWarps; ++w) {
            const uint32_t c = wsum[q][w];
            wsum[q][w] = acc;
            acc += c;
        }
        uint32_t* counter = q ? wb.counters + kCntExt + vertex + 1u : wb.counters + kCntShadow + vertex;
        base[q] = acc ? atomicAdd(counter, acc) : 0u;
    }
    __syncthreads();
    const uint32_t lt = (1u << lane) - 1u;
    if (vo.shadow) wb.sq[base[0] + wsum[0][warp] + __popc(m0 & lt)] = vo.sr;
    PathRay* q = ((vertex + 1u) & 1u) ? wb.q[1] : wb.q[0];
    if (vo.ext) q[base[1] + wsum[1][warp] + __popc(m1 & lt)] = vo.pr;
    __syncthreads();  // wsum and base are reused by the next call
}

// Vertex 0: the primary hit from the g-buffer (visibility + FP32 hit_t).
__global__ void __launch_bounds__(kShadeBlock, kShadeMinBlocks)
k_shade_primary(DevScene sc, FrameParams fp, mrt_gbuffer g, TraceParams tp, BlueNoise bn, WaveBuffers wb,
                uint32_t sample, uint32_t* status) {
    const uint32_t npix = fp.width * fp.height;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t rounded = (npix + kShadeBlock - 1u) / kShadeBlock * kShadeBlock;  // same trip count per block
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < rounded; i += stride) {
        const bool valid = i < npix;
        VertexOut vo;
        vo.shadow = vo.ext = false;
        if (valid) {
            uint32_t rng = sample == 0u ? initial_seed(tp.rng_mode, fp.c.frame_counter, i) : wb.rng[i];
            if (sample == 0u) wb.L[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            const uint32_t prim = g.visibility[i];
            const uint32_t x = i % fp.width, y = i / fp.width;
            f3 o, d;
            primary_ray(fp, x, y, o, d);
            if (prim == kMiss) {
                add_L(wb.L, i, escape_radiance(tp, d));
            } else {
                const f3 p = ray_at(o, d, g.hit_t[i]);
                vo = shade_vertex(sc, tp, bn, fp.width, 0u, i, p, d, prim, f3{1.0f, 1.0f, 1.0f}, rng, status);
            }
            wb.rng[i] = rng;
        }
        emit_block(vo, wb, 0u);
    }
}

// Vertex `vertex` >= 1: hits of the extension rays of bounce `vertex`.
__global__ void __launch_bounds__(kShadeBlock, kShadeMinBlocks)
k_shade(DevScene sc, TraceParams tp, BlueNoise bn, WaveBuffers wb, uint32_t width, uint32_t vertex,
        uint32_t* status) {
    const uint32_t n = wb.counters[kCntExt + vertex];
    const PathRay* q = ext_queue(wb, vertex);
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t rounded = (n + kShadeBlock - 1u) / kShadeBlock * kShadeBlock;  // same trip count per block
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < rounded; i += stride) {
        VertexOut vo;
        vo.shadow = vo.ext = false;
        if (i < n) {
            const PathRay pr = q[i];
            const uint2 h = wb.hits[i];
            const uint32_t pix = __float_as_uint(pr.o_pix.w);
            const f3 beta{pr.beta.x, pr.beta.y, pr.beta.z};
            if (h.x == kMiss) {
                add_L(wb.L, pix, mul_rn(beta, escape_radiance(tp, f3{pr.d.x, pr.d.y, pr.d.z})));
            } else {
                uint32_t rng = wb.rng[pix];
                const f3 o{pr.o_pix.x, pr.o_pix.y, pr.o_pix.z}, d{pr.d.x, pr.d.y, pr.d.z};
                const f3 p = ray_at(o, d, __uint_as_float(h.y));
                vo = shade_vertex(sc, tp, bn, width, vertex, pix, p, d, h.x, beta, rng, status);
                wb.rng[pix] = rng;
            }
        }
        emit_block(vo, wb, vertex);
    }
}

// Per-lane work refill for persistent traversal (Aila & Laine, "Understanding
// the efficiency of ray traversal on GPUs", HPG 2009, dynamic fetch): the
// lanes that `need` a ray share one atomic on the work counter.  Returns the
// lane's new ray index or kMiss.  `exhausted` is warp-uniform and stops all
// further fetches once the counter has passed n, so the counter grows by at
// most n + 32 per warp.  While fewer than `min_idle` lanes need a ray (and
// not all do) nobody fetches: the warp pays for the fetch and the ray setup
// once for several lanes.  Must be called by all 32 lanes.
MRT_DEV uint32_t warp_refill(uint32_t* fetch, uint32_t n, bool need, bool& exhausted, uint32_t min_idle) {
    if (exhausted) return kMiss;
    const uint32_t mask = __ballot_sync(0xFFFFFFFFu, need);
    if (!mask) return kMiss;
    if (mask != 0xFFFFFFFFu && uint32_t(__popc(mask)) < min_idle) return kMiss;  // wait for more idle lanes
    const uint32_t lane = lane_id(), leader = __ffs(mask) - 1u, cnt = __popc(mask);
    uint32_t base = 0u;
    if (lane == leader) base = atomicAdd(fetch, cnt);
    base = __shfl_sync(0xFFFFFFFFu, base, leader);
    if (base + cnt >= n) exhausted = true;
    if (!need) return kMiss;
    const uint32_t i = base + __popc(mask & ((1u << lane) - 1u));
    return i < n ? i : kMiss;
}

// Persistent closest-hit over the extension queue of bounce `bounce`.
// kDyn: idle lanes refill after every traversal step; otherwise each warp
// fetches 32 rays and runs them all to completion.
template <bool kCount, bool kDyn, bool kSpread = false>
__global__ void __launch_bounds__(kTraceBlock, kTraceMinBlocks)
k_trace_ext(DevScene sc, WaveBuffers wb, uint32_t bounce, uint32_t* status, uint32_t refill_min) {
    __shared__ uint2 stk[kStackDepth * kTraceBlock];
    __shared__ unsigned long long slots[kSpread ? kTraceBlock : 1];
    const uint32_t n = wb.counters[kCntExt + bounce];
    const PathRay* q = ext_queue(wb, bounce);
    uint32_t* fetch = wb.counters + kCntFetchExt + bounce;
    uint2* my = stk + threadIdx.x;
    uint32_t st = 0u, cn = 0u, ct = 0u;
    if (kDyn) {
        Trav s{};
        bool have = false, exhausted = false;
        uint32_t ri = 0u;
        while (true) {
            const uint32_t idx = warp_refill(fetch, n, !have, exhausted, refill_min);
            if (idx != kMiss) {
                const float4 a = q[idx].o_pix, b = q[idx].d;
                trav_init(s, f3{a.x, a.y, a.z}, f3{b.x, b.y, b.z}, 0.0f, INFINITY);
                ri = idx;
                have = true;
            }
            if (!__any_sync(0xFFFFFFFFu, have)) break;
            bool fin;
            if (kSpread)
                fin = trav_step_spread<false, kStackDepth>(sc, s, have, my, kTraceBlock, st,
                                                           slots + (threadIdx.x & ~31u));
            else
                fin = have && trav_step<false, kCount, kStackDepth>(sc, s, my, kTraceBlock, st, cn, ct);
            if (have && fin) {
                wb.hits[ri] = make_uint2(s.best, __float_as_uint(s.best == kMiss ? s.tmax : s.tbest));
                have = false;
            }
        }
    } else {
        const uint32_t lane = lane_id();
        while (true) {
            uint32_t base = 0u;
            if (lane == 0u) base = atomicAdd(fetch, 32u);
            base = __shfl_sync(0xFFFFFFFFu, base, 0);
            if (base >= n) break;
            const uint32_t i = base + lane;
            if (kSpread) {  // the warp steps its rays together; finished lanes keep testing triangles
                Trav s{};
                bool have = i < n;
                if (have) {
                    const float4 a = q[i].o_pix, b = q[i].d;
                    trav_init(s, f3{a.x, a.y, a.z}, f3{b.x, b.y, b.z}, 0.0f, INFINITY);
                }
                while (__any_sync(0xFFFFFFFFu, have)) {
                    if (trav_step_spread<false, kStackDepth>(sc, s, have, my, kTraceBlock, st,
                                                             slots + (threadIdx.x & ~31u))) {
                        wb.hits[i] = make_uint2(s.best, __float_as_uint(s.best == kMiss ? s.tmax : s.tbest));
                        have = false;
                    }
                }
            } else if (i < n) {
                const float4 a = q[i].o_pix, b = q[i].d;
                uint32_t prim;
                float t;
                trace_bvh8<false, kCount, kStackDepth>(sc, f3{a.x, a.y, a.z}, f3{b.x, b.y, b.z}, 0.0f, INFINITY,
                                                       prim, t, my, kTraceBlock, st, cn, ct);
                wb.hits[i] = make_uint2(prim, __float_as_uint(t));
            }
        }
    }
    if (st) atomicOr(status, st);
    if (kCount) {
        atomicAdd(wb.totals + kTotNodesExt + bounce, (unsigned long long)cn);
        atomicAdd(wb.totals + kTotTrisExt + bounce, (unsigned long long)ct);
    }
}

// Persistent any-hit over the shadow queue of vertex `vertex`; unoccluded
// rays add their contribution to the pixel's radiance.
template <bool kCount, bool kDyn, bool kSpread = false>
__global__ void __launch_bounds__(kTraceBlock, kTraceMinBlocks)
k_trace_shadow(DevScene sc, WaveBuffers wb, TraceParams tp, uint32_t vertex, uint32_t* status, uint32_t refill_min) {
    __shared__ uint2 stk[kStackDepth * kTraceBlock];
    __shared__ unsigned long long slots[kSpread ? kTraceBlock : 1];
    const uint32_t n = wb.counters[kCntShadow + vertex];
    uint32_t* fetch = wb.counters + kCntFetchShadow + vertex;
    const f3 sun{tp.sun[0], tp.sun[1], tp.sun[2]};
    uint2* my = stk + threadIdx.x;
    uint32_t st = 0u, cn = 0u, ct = 0u;
    if (kDyn) {
        Trav s{};
        bool have = false, exhausted = false;
        uint32_t ri = 0u;
        while (true) {
            const uint32_t idx = warp_refill(fetch, n, !have, exhausted, refill_min);
            if (idx != kMiss) {
                const float4 a = wb.sq[idx].o_pix;
                trav_init(s, f3{a.x, a.y, a.z}, sun, 0.0f, INFINITY);
                ri = idx;
                have = true;
            }
            if (!__any_sync(0xFFFFFFFFu, have)) break;
            bool fin;
            if (kSpread)
                fin = trav_step_spread<true, kStackDepth>(sc, s, have, my, kTraceBlock, st,
                                                          slots + (threadIdx.x & ~31u));
            else
                fin = have && trav_step<true, kCount, kStackDepth>(sc, s, my, kTraceBlock, st, cn, ct);
            if (have && fin) {
                if (s.best == kMiss) {
                    const ShadowRay sr = wb.sq[ri];
                    add_L(wb.L, __float_as_uint(sr.o_pix.w), f3{sr.contrib.x, sr.contrib.y, sr.contrib.z});
                }
                have = false;
            }
        }
    } else {
        const uint32_t lane = lane_id();
        while (true) {
            uint32_t base = 0u;
            if (lane == 0u) base = atomicAdd(fetch, 32u);
            base = __shfl_sync(0xFFFFFFFFu, base, 0);
            if (base >= n) break;
            const uint32_t i = base + lane;
            if (kSpread) {  // the warp steps its rays together; finished lanes keep testing triangles
                Trav s{};
                bool have = i < n;
                if (have) {
                    const float4 a = wb.sq[i].o_pix;
                    trav_init(s, f3{a.x, a.y, a.z}, sun, 0.0f, INFINITY);
                }
                while (__any_sync(0xFFFFFFFFu, have)) {
                    if (trav_step_spread<true, kStackDepth>(sc, s, have, my, kTraceBlock, st,
                                                            slots + (threadIdx.x & ~31u))) {
                        if (s.best == kMiss) {
                            const ShadowRay sr = wb.sq[i];
                            add_L(wb.L, __float_as_uint(sr.o_pix.w), f3{sr.contrib.x, sr.contrib.y, sr.contrib.z});
                        }
                        have = false;
                    }
                }
            } else if (i < n) {
                const ShadowRay sr = wb.sq[i];
                uint32_t prim;
                float t;
                trace_bvh8<true, kCount, kStackDepth>(sc, f3{sr.o_pix.x, sr.o_pix.y, sr.o_pix.z}, sun, 0.0f,
                                                      INFINITY, prim, t, my, kTraceBlock, st, cn, ct);
                if (prim == kMiss)
                    add_L(wb.L, __float_as_uint(sr.o_pix.w), f3{sr.contrib.x, sr.contrib.y, sr.contrib.z});
            }
        }
    }
    if (st) atomicOr(status, st);
    if (kCount) {
        atomicAdd(wb.totals + kTotNodesShadow, (unsigned long long)cn);
        atomicAdd(wb.totals + kTotTrisShadow, (unsigned long long)ct);
    }
}

// The path tail: one persistent launch finishes every path of the
// extension queue of bounce `first` — closest hit, shading, shadow ray and
// the following bounces — instead of 3 launches per remaining bounce whose
// small queues leave the GPU waiting on its longest ray each time.  Each
// warp takes 32 paths, each lane runs its path to the end.  A pixel's
// radiance receives the same additions in the same order as in the wavefront
// passes (escape, then shadow, vertex by vertex) and the RNG state advances
// identically, so the image is bit-identical; the ray counters of the
// bounces and vertices it covers are incremented as the wavefront's queues
// would have been, so ray statistics are unchanged.  Up to 128 registers (4
// resident blocks per SM): the tail is latency bound, and the traversal and
// shading code together spill at 64.
__global__ void __launch_bounds__(kTraceBlock, 4)
k_tail(DevScene sc, TraceParams tp, BlueNoise bn, WaveBuffers wb, uint32_t width, uint32_t first, uint32_t from_hits,
       uint32_t* status) {
    __shared__ uint2 stk[kStackDepth * kTraceBlock];
    const uint32_t n = wb.counters[kCntExt + first];
    const PathRay* q = ext_queue(wb, first);
    // from_hits: k_trace_ext has used the queue's own work counter; the
    // shadow-ray counter of vertex `first` is free (the tail traces those
    // shadow rays itself)
    uint32_t* fetch = wb.counters + (from_hits ? kCntFetchShadow : kCntFetchExt) + first;
    uint2* my = stk + threadIdx.x;
    const f3 sun{tp.sun[0], tp.sun[1], tp.sun[2]};
    uint32_t st = 0u, cn = 0u, ct = 0u;
    bool exhausted = false;
    while (true) {
        const uint32_t idx = warp_refill(fetch, n, true, exhausted);
        if (!__any_sync(0xFFFFFFFFu, idx != kMiss)) break;
        if (idx == kMiss) continue;
        const PathRay pr = q[idx];
        const uint32_t pix = __float_as_uint(pr.o_pix.w);
        f3 o{pr.o_pix.x, pr.o_pix.y, pr.o_pix.z}, d{pr.d.x, pr.d.y, pr.d.z}, beta{pr.beta.x, pr.beta.y, pr.beta.z};
        for (uint32_t b = first;; ++b) {
            uint32_t prim;
            float t;
            if (from_hits && b == first) {  // bounce `first` was traced by the wavefront kernel
                const uint2 h = wb.hits[idx];
                prim = h.x;
                t = __uint_as_float(h.y);
            } else {
                trace_bvh8<false, false, kStackDepth>(sc, o, d, 0.0f, INFINITY, prim, t, my, kTraceBlock, st, cn, ct);
            }
            if (prim == kMiss) {
                add_L(wb.L, pix, mul_rn(beta, escape_radiance(tp, d)));
                break;
            }
            uint32_t rng = wb.rng[pix];
            const VertexOut vo = shade_vertex(sc, tp, bn, width, b, pix, ray_at(o, d, t), d, prim, beta, rng, status);
            wb.rng[pix] = rng;
            if (vo.shadow) {
                atomicAdd(wb.counters + kCntShadow + b, 1u);
                uint32_t sp;
                float stt;
                trace_bvh8<true, false, kStackDepth>(sc, f3{vo.sr.o_pix.x, vo.sr.o_pix.y, vo.sr.o_pix.z}, sun, 0.0f,
                                                     INFINITY, sp, stt, my, kTraceBlock, st, cn, ct);
                if (sp == kMiss) add_L(wb.L, pix, f3{vo.sr.contrib.x, vo.sr.contrib.y, vo.sr.contrib.z});
            }
            if (!vo.ext) break;
            atomicAdd(wb.counters + kCntExt + b + 1u, 1u);
            o = f3{vo.pr.o_pix.x, vo.pr.o_pix.y, vo.pr.o_pix.z};
            d = f3{vo.pr.d.x, vo.pr.d.y, vo.pr.d.z};
            beta = f3{vo.pr.beta.x, vo.pr.beta.y, vo.pr.beta.z};
        }
    }
    if (st) atomicOr(status, st);
}

__global__ void k_tally(WaveBuffers wb) {
    const uint32_t j = threadIdx.x;
    if (j < kCntFetchExt) atomicAdd(wb.totals + j, (unsigned long long)wb.counters[j]);
}

__global__ void __launch_bounds__(kShadeBlock)
k_finalize(WaveBuffers wb, float* color, uint32_t npix, uint32_t samples, uint32_t accumulate, uint32_t frame_index) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npix) return;
    const float4 l = wb.L[i];
    const float ns = float(samples);
    float m[3] = {__fdiv_rn(l.x, ns), __fdiv_rn(l.y, ns), __fdiv_rn(l.z, ns)};
    float* out = color + size_t(i) * 3;
    if (accumulate && frame_index > 0u) {  // frame 0 starts the mean: old contents are ignored
        const float w = float(frame_index + 1u);
        for (int k = 0; k < 3; ++k) m[k] = __fadd_rn(out[k], __fdiv_rn(__fsub_rn(m[k], out[k]), w));
    }
    out[0] = m[0];
    out[1] = m[1];
    out[2] = m[2];
}

template <bool kAnyHit, bool kCount>
__global__ void __launch_bounds__(kTraceBlock, kTraceMinBlocks)
k_trace_rays(DevScene sc, const mrt_ray* rays, uint32_t n, mrt_hit* hits, uint32_t* nodes_v, uint32_t* tris_v,
             uint32_t* status) {
    __shared__ uint2 stk[kStackDepth * kTraceBlock];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4* rp = reinterpret_cast<const float4*>(rays + i);
    const float4 a = rp[0], b = rp[1];
    uint32_t prim, st = 0u, cn = 0u, ct = 0u;
    float t;
    trace_bvh8<kAnyHit, kCount, kStackDepth>(sc, f3{a.x, a.y, a.z}, f3{b.x, b.y, b.z}, a.w, b.w, prim, t,
                                             stk + threadIdx.x, kTraceBlock, st, cn, ct);
    hits[i].prim = prim;
    hits[i].t = t;
    if (kCount) {
        nodes_v[i] = cn;
        tris_v[i] = ct;
    }
    if (st) atomicOr(status, st);
}

template <bool kAnyHit>
__global__ void __launch_bounds__(128)
k_trace_rays_sphere(DevScene sc, const mrt_ray* rays, uint32_t n, mrt_hit* hits) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const mrt_ray r = rays[i];
    const f3 o{r.org[0], r.org[1], r.org[2]}, d{r.dir[0], r.dir[1], r.dir[2]};
    uint32_t prim = kMiss;
    float tb = r.tmax;
    for (uint32_t k = 0; k < sc.sphere_count; ++k) {
        f3 c; float rad;
        sphere_at(sc, k, c, rad);
        const float t = ray_sphere(o, d, c, rad);
        if (t > r.tmin && t < tb) {
            tb = t;
            prim = k;
            if (kAnyHit) break;
        }
    }
    hits[i].prim = prim;
    hits[i].t = tb;
}

// ------------------------------------------------------------------ launchers

cudaError_t launch_primary_tri(const DevScene& sc, const FrameParams& fp, const mrt_gbuffer& g, uint32_t* status,
                               unsigned long long* totals, uint32_t* fetch, int blocks, bool spread,
                               uint32_t refill_min, cudaStream_t s) {
    if (fetch) {
        cudaError_t e = cudaMemsetAsync(fetch, 0, sizeof(uint32_t), s);
        if (e != cudaSuccess) return e;
        if (totals)
            k_primary_tri_dyn<true><<<blocks, kTraceBlock, 0, s>>>(sc, fp, g, status, totals, fetch, refill_min);
        else
            k_primary_tri_dyn<false><<<blocks, kTraceBlock, 0, s>>>(sc, fp, g, status, nullptr, fetch, refill_min);
        return cudaGetLastError();
    }
    dim3 grid((fp.width + 15) / 16, (fp.height + 7) / 8);
    if (totals) k_primary_tri<true><<<grid, kTraceBlock, 0, s>>>(sc, fp, g, status, totals);
    else if (spread) k_primary_tri<false, true><<<grid, kTraceBlock, 0, s>>>(sc, fp, g, status, nullptr);
    else k_primary_tri<false><<<grid, kTraceBlock, 0, s>>>(sc, fp, g, status, nullptr);
    return cudaGetLastError();
}

cudaError_t launch_primary_sphere(const DevScene& sc, const FrameParams& fp, const mrt_gbuffer& g, cudaStream_t s) {
    dim3 grid((fp.width + 15) / 16, (fp.height + 7) / 8);
    k_primary_sphere<<<grid, 128, 0, s>>>(sc, fp, g);
    return cudaGetLastError();
}

cudaError_t launch_secondary_sphere(const DevScene& sc, const FrameParams& fp, const mrt_gbuffer& g,
                                    const TraceParams& tp, BlueNoise bn, float* color, uint32_t accumulate,
                                    uint32_t frame_index, cudaStream_t s) {
    dim3 grid((fp.width + 15) / 16, (fp.height + 7) / 8);
    k_secondary_sphere<<<grid, 128, 0, s>>>(sc, fp, g, tp, bn, color, accumulate, frame_index);
    return cudaGetLastError();
}

cudaError_t launch_trace_rays(const DevScene& sc, const mrt_ray* rays, uint32_t n, mrt_hit* hits, bool any_hit,
                              uint32_t* nodes_v, uint32_t* tris_v, uint32_t* status, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const uint32_t blocks = (n + kTraceBlock - 1) / kTraceBlock;
    if (sc.sphere_count) {
        if (any_hit) k_trace_rays_sphere<true><<<blocks, 128, 0, s>>>(sc, rays, n, hits);
        else k_trace_rays_sphere<false><<<blocks, 128, 0, s>>>(sc, rays, n, hits);
    } else if (nodes_v) {
        k_trace_rays<false, true><<<blocks, kTraceBlock, 0, s>>>(sc, rays, n, hits, nodes_v, tris_v, status);
    } else if (any_hit) {
        k_trace_rays<true, false><<<blocks, kTraceBlock, 0, s>>>(sc, rays, n, hits, nullptr, nullptr, status);
    } else {
        k_trace_rays<false, false><<<blocks, kTraceBlock, 0, s>>>(sc, rays, n, hits, nullptr, nullptr, status);
    }
    return cudaGetLastError();
}

static int shade_blocks(uint32_t n) {
    uint32_t b = (n + kShadeBlock - 1) / kShadeBlock;
    return int(b < 1 ? 1 : (b > 4096 ? 4096 : b));
}

cudaError_t launch_shade_primary(const DevScene& sc, const FrameParams& fp, const mrt_gbuffer& g, const TraceParams& tp,
                                 BlueNoise bn, const WaveBuffers& wb, uint32_t sample, uint32_t* status,
                                 cudaStream_t s) {
    k_shade_primary<<<shade_blocks(fp.width * fp.height), kShadeBlock, 0, s>>>(sc, fp, g, tp, bn, wb, sample, status);
    return cudaGetLastError();
}

cudaError_t launch_trace_ext(const DevScene& sc, const WaveBuffers& wb, uint32_t bounce, int blocks, uint32_t* status,
                             bool count, int mode, uint32_t refill_min, cudaStream_t s) {
#define MRT_EXT(C, D, P) k_trace_ext<C, D, P><<<blocks, kTraceBlock, 0, s>>>(sc, wb, bounce, status, refill_min)
    if (count) {  // the counting kernels test each lane's own triangles
        if (mode == kFetchDynamic || mode == kFetchSpread) MRT_EXT(true, true, false);
        else MRT_EXT(true, false, false);
    } else {
        switch (mode) {
        case kFetchDynamic: MRT_EXT(false, true, false); break;
        case kFetchSpread: MRT_EXT(false, true, true); break;
        case kFetchBatchSpread: MRT_EXT(false, false, true); break;
        default: MRT_EXT(false, false, false); break;
        }
    }
#undef MRT_EXT
    return cudaGetLastError();
}

// The path tail with the traversal steps of a warp's lanes taken together
// (trav_step_spread_mixed): each lane is a small state machine -- idle,
// tracing its path's extension ray (closest hit) or its vertex's shadow ray
// (any hit) -- and every iteration the warp refills idle lanes, then takes
// one traversal step of all its rays with the triangle tests spread over
// the lanes.  The shading, the counters and a pixel's radiance additions
// happen in k_tail's order, so the image is the same.
__global__ void __launch_bounds__(kTraceBlock, 4)
k_tail_spread(DevScene sc, TraceParams tp, BlueNoise bn, WaveBuffers wb, uint32_t width, uint32_t first,
              uint32_t from_hits, uint32_t* status) {
    __shared__ uint2 stk[kStackDepth * kTraceBlock];
    __shared__ unsigned long long slots[kTraceBlock];
    const uint32_t n = wb.counters[kCntExt + first];
    const PathRay* q = ext_queue(wb, first);
    uint32_t* fetch = wb.counters + (from_hits ? kCntFetchShadow : kCntFetchExt) + first;
    uint2* my = stk + threadIdx.x;
    unsigned long long* wslots = slots + (threadIdx.x & ~31u);
    const f3 sun{tp.sun[0], tp.sun[1], tp.sun[2]};
    uint32_t st = 0u;
    bool exhausted = false;
    int mode = 0;  // 0 idle, 1 extension ray, 2 shadow ray
    Trav s{};
    uint32_t pix = 0u, b = 0u;
    f3 o{0.0f, 0.0f, 0.0f}, d{0.0f, 0.0f, 1.0f}, beta{0.0f, 0.0f, 0.0f}, contrib{0.0f, 0.0f, 0.0f};
    bool next_ext = false;
    f3 no{0.0f, 0.0f, 0.0f}, nd{0.0f, 0.0f, 1.0f}, nbeta{0.0f, 0.0f, 0.0f};
    // after the shadow ray of vertex b (or without one): the next bounce
    auto cont = [&]() {
        if (!next_ext) { mode = 0; return; }
        atomicAdd(wb.counters + kCntExt + b + 1u, 1u);
        o = no; d = nd; beta = nbeta;
        ++b;
        trav_init(s, o, d, 0.0f, INFINITY);
        mode = 1;
    };
    // the extension ray of bounce b found `prim` at t (or escaped)
    auto hit = [&](uint32_t prim, float t) {
        if (prim == kMiss) {
            add_L(wb.L, pix, mul_rn(beta, escape_radiance(tp, d)));
            mode = 0;
            return;
        }
        uint32_t rng = wb.rng[pix];
        const VertexOut vo = shade_vertex(sc, tp, bn, width, b, pix, ray_at(o, d, t), d, prim, beta, rng, status);
        wb.rng[pix] = rng;
        next_ext = vo.ext;
        no = f3{vo.pr.o_pix.x, vo.pr.o_pix.y, vo.pr.o_pix.z};
        nd = f3{vo.pr.d.x, vo.pr.d.y, vo.pr.d.z};
        nbeta = f3{vo.pr.beta.x, vo.pr.beta.y, vo.pr.beta.z};
        if (vo.shadow) {
            atomicAdd(wb.counters + kCntShadow + b, 1u);
            contrib = f3{vo.sr.contrib.x, vo.sr.contrib.y, vo.sr.contrib.z};
            trav_init(s, f3{vo.sr.o_pix.x, vo.sr.o_pix.y, vo.sr.o_pix.z}, sun, 0.0f, INFINITY);
            mode = 2;
        } else {
            cont();
        }
    };
    while (true) {
        const uint32_t idx = warp_refill(fetch, n, mode == 0, exhausted);
        if (idx != kMiss) {
            const PathRay pr = q[idx];
            pix = __float_as_uint(pr.o_pix.w);
            o = f3{pr.o_pix.x, pr.o_pix.y, pr.o_pix.z};
            d = f3{pr.d.x, pr.d.y, pr.d.z};
            beta = f3{pr.beta.x, pr.beta.y, pr.beta.z};
            b = first;
            if (from_hits) {
                const uint2 h = wb.hits[idx];
                hit(h.x, __uint_as_float(h.y));
            } else {
                trav_init(s, o, d, 0.0f, INFINITY);
                mode = 1;
            }
        }
        if (!__any_sync(0xFFFFFFFFu, mode != 0)) {
            if (exhausted) break;
            continue;
        }
        const bool busy = mode != 0;
        if (trav_step_spread_mixed<kStackDepth>(sc, s, busy, mode == 2, my, kTraceBlock, st, wslots) && busy) {
            if (mode == 1) {
                hit(s.best, s.best == kMiss ? s.tmax : s.tbest);
            } else {
                if (s.best == kMiss) add_L(wb.L, pix, contrib);
                cont();
            }
        }
    }
    if (st) atomicOr(status, st);
}

cudaError_t launch_tail(const DevScene& sc, const TraceParams& tp, BlueNoise bn, const WaveBuffers& wb,
                        uint32_t width, uint32_t first, bool from_hits, bool spread, int blocks, uint32_t* status,
                        cudaStream_t s) {
    if (spread)
        k_tail_spread<<<blocks, kTraceBlock, 0, s>>>(sc, tp, bn, wb, width, first, from_hits ? 1u : 0u, status);
    else
        k_tail<<<blocks, kTraceBlock, 0, s>>>(sc, tp, bn, wb, width, first, from_hits ? 1u : 0u, status);
    return cudaGetLastError();
}

cudaError_t launch_trace_shadow(const DevScene& sc, const WaveBuffers& wb, const TraceParams& tp, uint32_t vertex,
                                int blocks, uint32_t* status, bool count, int mode, uint32_t refill_min,
                                cudaStream_t s) {
#define MRT_SH(C, D, P) \
    k_trace_shadow<C, D, P><<<blocks, kTraceBlock, 0, s>>>(sc, wb, tp, vertex, status, refill_min)
    if (count) {  // the counting kernels test each lane's own triangles
        if (mode == kFetchDynamic || mode == kFetchSpread) MRT_SH(true, true, false);
        else MRT_SH(true, false, false);
    } else {
        switch (mode) {
        case kFetchDynamic: MRT_SH(false, true, false); break;
        case kFetchSpread: MRT_SH(false, true, true); break;
        case kFetchBatchSpread: MRT_SH(false, false, true); break;
        default: MRT_SH(false, false, false); break;
        }
    }
#undef MRT_SH
    return cudaGetLastError();
}

// The extension rays of bounce `bounce` and the shadow rays of vertex
// `vertex` = bounce - 1 in one persistent launch (mrt_tuning.overlap_shadow
// 2).  The two queues are independent — only the shadow rays add radiance,
// each pixel at most once per vertex, and the shading after this launch
// adds the next — so a warp refills its idle lanes from the extension queue
// and, once that is drained, from the shadow queue, and steps all its rays
// together with the mixed spread step (closest hit or any hit per lane,
// the triangle tests spread over the warp).  The GPU then drains one wave
// tail instead of two launches', which two streams overlap only in part
// (a launch's resident blocks take all of an SM's registers).  Same hits
// and the same radiance additions as the two launches.
__global__ void __launch_bounds__(kTraceBlock, kTraceMinBlocks)
k_trace_merged(DevScene sc, WaveBuffers wb, TraceParams tp, uint32_t bounce, uint32_t vertex, uint32_t* status,
               uint32_t refill_min) {
    __shared__ uint2 stk[kStackDepth * kTraceBlock];
    __shared__ unsigned long long slots[kTraceBlock];
    const uint32_t n_ext = wb.counters[kCntExt + bounce], n_sh = wb.counters[kCntShadow + vertex];
    uint2* my = stk + threadIdx.x;
    uint32_t st = 0u;
    Trav s{};
    bool have = false, any_hit = false, ext_done = false, sh_done = false;
    uint32_t ri = 0u;
    while (true) {
        if (!ext_done) {  // warp-uniform (warp_refill sets it from the warp's shared fetch)
            const uint32_t idx = warp_refill(wb.counters + kCntFetchExt + bounce, n_ext, !have, ext_done, refill_min);
            if (idx != kMiss) {
                const PathRay* q = ext_queue(wb, bounce);
                const float4 a = q[idx].o_pix, b = q[idx].d;
                trav_init(s, f3{a.x, a.y, a.z}, f3{b.x, b.y, b.z}, 0.0f, INFINITY);
                ri = idx;
                have = true;
                any_hit = false;
            }
        }
        if (ext_done) {
            const uint32_t idx =
                warp_refill(wb.counters + kCntFetchShadow + vertex, n_sh, !have, sh_done, refill_min);
            if (idx != kMiss) {
                const float4 a = wb.sq[idx].o_pix;
                trav_init(s, f3{a.x, a.y, a.z}, f3{tp.sun[0], tp.sun[1], tp.sun[2]}, 0.0f, INFINITY);
                ri = idx;
                have = true;
                any_hit = true;
            }
        }
        if (!__any_sync(0xFFFFFFFFu, have)) break;
        const bool fin = trav_step_spread_mixed<kStackDepth>(sc, s, have, any_hit, my, kTraceBlock, st,
                                                             slots + (threadIdx.x & ~31u));
        if (have && fin) {
            if (!any_hit) {
                wb.hits[ri] = make_uint2(s.best, __float_as_uint(s.best == kMiss ? s.tmax : s.tbest));
            } else if (s.best == kMiss) {
                const ShadowRay sr = wb.sq[ri];
                add_L(wb.L, __float_as_uint(sr.o_pix.w), f3{sr.contrib.x, sr.contrib.y, sr.contrib.z});
            }
            have = false;
        }
    }
    if (st) atomicOr(status, st);
}

cudaError_t launch_trace_merged(const DevScene& sc, const WaveBuffers& wb, const TraceParams& tp, uint32_t bounce,
                                int blocks, uint32_t* status, uint32_t refill_min, cudaStream_t s) {
    k_trace_merged<<<blocks, kTraceBlock, 0, s>>>(sc, wb, tp, bounce, bounce - 1u, status, refill_min);
    return cudaGetLastError();
}

cudaError_t launch_shade(const DevScene& sc, const TraceParams& tp, BlueNoise bn, const WaveBuffers& wb,
                         uint32_t width, uint32_t bounce, uint32_t* status, cudaStream_t s) {
    k_shade<<<shade_blocks(uint32_t(wb.cap)), kShadeBlock, 0, s>>>(sc, tp, bn, wb, width, bounce, status);
    return cudaGetLastError();
}

// ---- learned radiance cache: training samples and cache-terminated shading

constexpr int kTrainMaxVerts = 9;

MRT_DEV void cache_query_row(const DevScene& sc, f3 p, f3 n, f3 wo, float* q) {
    q[0] = __fmul_rn(__fsub_rn(p.x, sc.lo[0]), sc.inv_ext[0]);
    q[1] = __fmul_rn(__fsub_rn(p.y, sc.lo[1]), sc.inv_ext[1]);
    q[2] = __fmul_rn(__fsub_rn(p.z, sc.lo[2]), sc.inv_ext[2]);
    q[3] = n.x; q[4] = n.y; q[5] = n.z;
    q[6] = wo.x; q[7] = wo.y; q[8] = wo.z;
}

// One thread per training path from a hashed pixel of this frame's camera:
// the plain estimator (shadow ray per vertex, cosine-weighted bounces,
// Russian roulette past rr_start) up to `bounces` bounces; afterwards the
// suffix radiance L_o(x_v, -d_v) of every vertex is a training target for
// the cache query (x_v, n_v, -d_v).
__global__ void __launch_bounds__(kTraceBlock)
k_cache_train_paths(DevScene sc, FrameParams fp, TraceParams tp, uint32_t bounces, uint32_t n_paths,
                    uint32_t frame, float* out_q, float* out_t, uint32_t* count, uint32_t cap, uint32_t* status) {
    __shared__ uint2 stk[kStackDepth * kTraceBlock];
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t alive = __ballot_sync(0xFFFFFFFFu, p < n_paths);  // a prefix of the warp's lanes
    if (p >= n_paths) return;
    uint32_t st = 0u, cn = 0u, ct = 0u;
    uint32_t h = p * 0x9E3779B1u + frame * 0x85EBCA6Bu + 0x632BE5ABu;
    const uint32_t pix = pcg(h) % (fp.width * fp.height);
    uint32_t rng = pcg(h) | 1u;
    f3 o, d;
    primary_ray(fp, pix % fp.width, pix / fp.width, o, d);
    const f3 sun{tp.sun[0], tp.sun[1], tp.sun[2]};
    float qv[kTrainMaxVerts][9];
    f3 nee[kTrainMaxVerts], rho[kTrainMaxVerts];
    float wcont[kTrainMaxVerts];
    int nv = 0;
    bool escaped = false;
    const uint32_t maxb = bounces < uint32_t(kTrainMaxVerts - 1) ? bounces : uint32_t(kTrainMaxVerts - 1);
    for (uint32_t v = 0;; ++v) {
        uint32_t prim;
        float t;
        trace_bvh8<false, false, kStackDepth>(sc, o, d, 0.0f, INFINITY, prim, t, stk + threadIdx.x, kTraceBlock, st,
                                              cn, ct);
        if (prim == kMiss) { escaped = v > 0; break; }
        const mrt_material m = load_mat(sc, prim, status);
        const f3 n = facing_normal(m, d);
        const f3 x = ray_at(o, d, t);
        cache_query_row(sc, x, n, f3{-d.x, -d.y, -d.z}, qv[nv]);
        rho[nv] = f3{__fdiv_rn(float(m.albedo_rgba8 & 0xFFu), 255.0f),
                     __fdiv_rn(float((m.albedo_rgba8 >> 8) & 0xFFu), 255.0f),
                     __fdiv_rn(float((m.albedo_rgba8 >> 16) & 0xFFu), 255.0f)};
        nee[nv] = f3{0.0f, 0.0f, 0.0f};
        wcont[nv] = 0.0f;
        if (tp.estimator == MRT_EST_NEE) {
            const float cosl = dot_rn(n, sun);
            if (cosl > 0.0f) {
                uint32_t sp;
                float stt;
                trace_bvh8<true, false, kStackDepth>(sc, offset_ray(x, n), sun, 0.0f, INFINITY, sp, stt,
                                                     stk + threadIdx.x, kTraceBlock, st, cn, ct);
                if (sp == kMiss)
                    nee[nv] = scale_rn(mul_rn(rho[nv], f3{tp.sun_e[0], tp.sun_e[1], tp.sun_e[2]}),
                                       __fmul_rn(cosl, kInvPi));
            }
        }
        ++nv;
        if (v >= maxb) break;
        const float u1 = random_float(rng), u2 = random_float(rng);
        f3 nd = add_rn(n, random_sphere_point(__fsub_rn(__fmul_rn(u1, 2.0f), 1.0f),
                                              __fsub_rn(__fmul_rn(u2, 2.0f), 1.0f), tp.exact_trig));
        if (dot_rn(nd, nd) == 0.0f) nd = n;
        nd = normalize_rn(nd);
        float w = 1.0f;
        if (tp.rr_start != 0u && v + 1u > tp.rr_start) {
            const f3 b = rho[nv - 1];
            const float q = fminf(fmaxf(fmaxf(fmaxf(b.x, b.y), b.z), 0.05f), 1.0f);
            if (random_float(rng) >= q) break;
            w = 1.0f / q;
        }
        wcont[nv - 1] = w;
        o = offset_ray(x, n);
        d = nd;
    }
    if (st) atomicOr(status, st);
    // suffix radiance, last vertex first; each vertex's sample is its
    // indirect outgoing radiance (the suffix without its own direct light,
    // which the frame adds exactly with a shadow ray)
    f3 next = escaped ? escape_radiance(tp, d) : f3{0.0f, 0.0f, 0.0f};
    // the warp's samples get their slots with one atomic: an inclusive scan
    // of nv over the warp's live lanes (a prefix of the lanes)
    __syncwarp(alive);
    const uint32_t lane = lane_id();
    uint32_t incl = uint32_t(nv);
    for (uint32_t off = 1; off < 32u; off <<= 1) {
        const uint32_t v = __shfl_up_sync(alive, incl, int(off));
        if (lane >= off) incl += v;
    }
    const uint32_t last = 31u - uint32_t(__clz(alive));
    const uint32_t total = __shfl_sync(alive, incl, int(last));
    uint32_t base = 0u;
    if (lane == 0u && total) base = atomicAdd(count, total);
    base = __shfl_sync(alive, base, 0) + incl - uint32_t(nv);
    for (int v = nv - 1; v >= 0; --v) {
        const float w = wcont[v];
        const f3 Li{rho[v].x * w * next.x, rho[v].y * w * next.y, rho[v].z * w * next.z};
        const uint32_t slot = base++;
        if (slot < cap) {
            for (int k = 0; k < 9; ++k) out_q[size_t(slot) * 9 + k] = qv[v][k];
            out_t[size_t(slot) * 3 + 0] = Li.x;
            out_t[size_t(slot) * 3 + 1] = Li.y;
            out_t[size_t(slot) * 3 + 2] = Li.z;
        }
        next = f3{nee[v].x + Li.x, nee[v].y + Li.y, nee[v].z + Li.z};
    }
}

// For each bounce-1 extension ray that hit: the cache query row at the hit
// and (throughput, pixel) for the apply.  Escaped rays were shaded (sky) by
// k_shade, which also sent the hit's direct-light shadow ray.
__global__ void __launch_bounds__(kShadeBlock)
k_cache_query(DevScene sc, TraceParams tp, WaveBuffers wb, float* q, float4* pb, uint32_t* status) {
    const uint32_t n = wb.counters[kCntExt + 1];
    const PathRay* qin = ext_queue(wb, 1);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const PathRay pr = qin[i];
        const uint2 h = wb.hits[i];
        const uint32_t pix = __float_as_uint(pr.o_pix.w);
        const f3 beta{pr.beta.x, pr.beta.y, pr.beta.z};
        float* row = q + size_t(i) * 9;
        if (h.x == kMiss) {
            for (int k = 0; k < 9; ++k) row[k] = 0.0f;
            pb[i] = make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(pix));
        } else {
            const f3 o{pr.o_pix.x, pr.o_pix.y, pr.o_pix.z}, d{pr.d.x, pr.d.y, pr.d.z};
            const mrt_material m = load_mat(sc, h.x, status);
            const f3 nrm = facing_normal(m, d);
            cache_query_row(sc, ray_at(o, d, __uint_as_float(h.y)), nrm, f3{-d.x, -d.y, -d.z}, row);
            pb[i] = make_float4(beta.x, beta.y, beta.z, __uint_as_float(pix));
        }
    }
}

// For each primary hit: the cache query row at the hit (outgoing direction
// toward the camera) with unit throughput; misses and the hit's direct light
// were shaded by k_shade_primary.
__global__ void __launch_bounds__(kShadeBlock)
k_cache_query_primary(DevScene sc, FrameParams fp, mrt_gbuffer g, float* q, float4* pb, uint32_t* status) {
    const uint32_t npix = fp.width * fp.height;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += gridDim.x * blockDim.x) {
        float* row = q + size_t(i) * 9;
        const uint32_t prim = g.visibility[i];
        if (prim == kMiss) {
            for (int k = 0; k < 9; ++k) row[k] = 0.0f;
            pb[i] = make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(i));
            continue;
        }
        f3 o, d;
        primary_ray(fp, i % fp.width, i / fp.width, o, d);
        const mrt_material m = load_mat(sc, prim, status);
        cache_query_row(sc, ray_at(o, d, g.hit_t[i]), facing_normal(m, d), f3{-d.x, -d.y, -d.z}, row);
        pb[i] = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(i));
    }
}

// L[pixel] += throughput x prediction for the first n_dev[0] (or n) rows.
__global__ void __launch_bounds__(kShadeBlock)
k_cache_apply(WaveBuffers wb, const uint32_t* n_dev, uint32_t n_max, const float* pred, const float4* pb) {
    const uint32_t n = n_dev ? min(*n_dev, n_max) : n_max;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 b = pb[i];
        if (b.x == 0.0f && b.y == 0.0f && b.z == 0.0f) continue;
        const f3 y{fmaxf(pred[3 * size_t(i)], 0.0f), fmaxf(pred[3 * size_t(i) + 1], 0.0f),
                   fmaxf(pred[3 * size_t(i) + 2], 0.0f)};
        add_L(wb.L, __float_as_uint(b.w), mul_rn(f3{b.x, b.y, b.z}, y));
    }
}

cudaError_t launch_cache_train_paths(const DevScene& sc, const FrameParams& fp, const TraceParams& tp,
                                     uint32_t bounces, uint32_t n_paths, uint32_t frame, float* q, float* t,
                                     uint32_t* count, uint32_t cap, uint32_t* status, cudaStream_t s) {
    k_cache_train_paths<<<(n_paths + kTraceBlock - 1) / kTraceBlock, kTraceBlock, 0, s>>>(
        sc, fp, tp, bounces, n_paths, frame, q, t, count, cap, status);
    return cudaGetLastError();
}

cudaError_t launch_cache_query(const DevScene& sc, const TraceParams& tp, const WaveBuffers& wb, float* q, float4* pb,
                               uint32_t* status, cudaStream_t s) {
    const uint32_t b = uint32_t((wb.cap + kShadeBlock - 1) / kShadeBlock);
    k_cache_query<<<b < 4096 ? b : 4096, kShadeBlock, 0, s>>>(sc, tp, wb, q, pb, status);
    return cudaGetLastError();
}

cudaError_t launch_cache_query_primary(const DevScene& sc, const FrameParams& fp, const mrt_gbuffer& g, float* q,
                                       float4* pb, uint32_t* status, cudaStream_t s) {
    const uint32_t b = (fp.width * fp.height + kShadeBlock - 1) / kShadeBlock;
    k_cache_query_primary<<<b < 4096 ? b : 4096, kShadeBlock, 0, s>>>(sc, fp, g, q, pb, status);
    return cudaGetLastError();
}

cudaError_t launch_cache_apply(const WaveBuffers& wb, const uint32_t* n_dev, uint32_t n_max, const float* pred,
                               const float4* pb, cudaStream_t s) {
    const uint32_t b = (n_max + kShadeBlock - 1) / kShadeBlock;
    k_cache_apply<<<b < 4096 ? (b ? b : 1) : 4096, kShadeBlock, 0, s>>>(wb, n_dev, n_max, pred, pb);
    return cudaGetLastError();
}

// ---- ray sorting between bounces: one counting-sort pass on a 12-bit key,
// direction octant (3 bits) above a 9-bit Morton code of the origin in the
// scene box (3 bits per axis), so rays sharing a direction octant and a
// region of space trace side by side.  Order inside a bin is arbitrary;
// results do not depend on it (each pixel owns one path).
constexpr uint32_t kSortBins = 4096;

MRT_DEV uint32_t sort_key(const DevScene& sc, const PathRay& r) {
    uint32_t key = (r.d.x < 0.0f ? 1u : 0u) | (r.d.y < 0.0f ? 2u : 0u) | (r.d.z < 0.0f ? 4u : 0u);
    const float o[3] = {r.o_pix.x, r.o_pix.y, r.o_pix.z};
    uint32_t q[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float u = (o[a] - sc.lo[a]) * sc.inv_ext[a];
        q[a] = uint32_t(fminf(fmaxf(u * 8.0f, 0.0f), 7.0f));
    }
    uint32_t m = 0u;
#pragma unroll
    for (int b = 2; b >= 0; --b) m = (m << 3) | (((q[0] >> b) & 1u) << 2) | (((q[1] >> b) & 1u) << 1) | ((q[2] >> b) & 1u);
    return (key << 9) | m;
}

__global__ void __launch_bounds__(kShadeBlock) k_sort_hist(DevScene sc, WaveBuffers wb, uint32_t bounce,
                                                           uint32_t min_rays) {
    __shared__ uint32_t h[kSortBins];
    const uint32_t n = wb.counters[kCntExt + bounce];
    if (n < min_rays) return;  // short queues are traced unsorted
    for (uint32_t i = threadIdx.x; i < kSortBins; i += blockDim.x) h[i] = 0u;
    __syncthreads();
    const PathRay* q = (bounce & 1u) ? wb.q[1] : wb.q[0];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t k = sort_key(sc, q[i]);
        wb.keys[i] = k;
        atomicAdd(&h[k], 1u);
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < kSortBins; i += blockDim.x)
        if (h[i]) atomicAdd(&wb.hist[i], h[i]);
}

// exclusive scan of the 4096 bin counts, one block of 1024 threads
__global__ void __launch_bounds__(1024) k_sort_scan(WaveBuffers wb) {
    __shared__ uint32_t part[1024];
    const uint32_t t = threadIdx.x;
    uint32_t v[4], s = 0u;
#pragma unroll
    for (int k = 0; k < 4; ++k) { v[k] = wb.hist[4 * t + k]; s += v[k]; }
    part[t] = s;
    __syncthreads();
    for (uint32_t off = 1; off < 1024; off <<= 1) {
        const uint32_t add = t >= off ? part[t - off] : 0u;
        __syncthreads();
        part[t] += add;
        __syncthreads();
    }
    uint32_t run = part[t] - s;
#pragma unroll
    for (int k = 0; k < 4; ++k) { wb.hist[4 * t + k] = run; run += v[k]; }
}

__global__ void __launch_bounds__(kShadeBlock) k_sort_scatter(WaveBuffers wb, uint32_t bounce, uint32_t min_rays) {
    const uint32_t n = wb.counters[kCntExt + bounce];
    if (n < min_rays) return;
    const PathRay* q = (bounce & 1u) ? wb.q[1] : wb.q[0];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t pos = atomicAdd(&wb.hist[wb.keys[i]], 1u);
        wb.qsort[pos] = q[i];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) wb.counters[kCntSorted + bounce] = 1u;
}

// Sorts the extension queue of `bounce` into wb.qsort when it holds at
// least `min_rays` rays and flags it, so the trace and shade kernels of
// that bounce read the sorted copy (ext_queue).  No host synchronisation.
cudaError_t launch_sort_ext(const DevScene& sc, const WaveBuffers& wb, uint32_t bounce, uint32_t min_rays,
                            cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(wb.hist, 0, kSortBins * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    const int blocks = shade_blocks(uint32_t(wb.cap));
    k_sort_hist<<<blocks, kShadeBlock, 0, s>>>(sc, wb, bounce, min_rays);
    k_sort_scan<<<1, 1024, 0, s>>>(wb);
    k_sort_scatter<<<blocks, kShadeBlock, 0, s>>>(wb, bounce, min_rays);
    return cudaGetLastError();
}

cudaError_t launch_finalize(const WaveBuffers& wb, float* color, uint32_t samples, uint32_t accumulate,
                            uint32_t frame_index, cudaStream_t s) {
    const uint32_t npix = uint32_t(wb.npix);
    k_finalize<<<(npix + kShadeBlock - 1) / kShadeBlock, kShadeBlock, 0, s>>>(wb, color, npix, samples, accumulate,
                                                                             frame_index);
    return cudaGetLastError();
}

cudaError_t launch_tally(const WaveBuffers& wb, cudaStream_t s) {
    k_tally<<<1, 64, 0, s>>>(wb);
    return cudaGetLastError();
}

int trace_blocks_per_sm() {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_trace_ext<false, true>, kTraceBlock, 0) != cudaSuccess ||
        b < 1)
        b = 1;
    return b;
}

} // namespace mrt
