// BVH8 traversal and watertight ray/triangle intersection.
//
// The reference finds closest hits by looping over 5 spheres
// (primaryRay.comp:23-36, secondaryRays.comp:74-89); this is the triangle
// replacement, built from published methods:
//   - watertight ray/triangle test: Woop, Benthin & Wald, "Watertight
//     Ray/Triangle Intersection", JCGT 2(1), 2013 -- per-ray shear to the
//     dominant axis, 2D edge functions, double-precision recheck on zero;
//   - compressed 8-wide BVH traversal with octant-ordered children and an
//     (base, hit-mask) group stack: Ylitie, Karras & Laine, HPG 2017;
//   - conservative slab test: Ize, "Robust BVH Ray Traversal", JCGT 2013
//     (far distances scaled up by a relative epsilon).
// Ties at equal t resolve to the lower original triangle id, so the result
// is independent of the BVH and of traversal order.
#pragma once

#include "common.cuh"

namespace mrt {

struct DevScene {
    const uint4* nodes;       // 8 x uint4 per node (128 bytes)
    const float4* tris;       // 3 x float4 per triangle, leaf order
    const mrt_material* mats; // per original triangle id
    const float4* spheres;    // 2 x float4 per sphere: center+radius, albedo
    uint32_t node_count;
    uint32_t tri_count;
    uint32_t mat_count;
    uint32_t sphere_count;
    float lo[3];        // scene bounds (ray-sort keys)
    float inv_ext[3];   // 1 / extent per axis
};

constexpr float kRobustScale = 1.0f + 1.0f / 1048576.0f; // 1 + 2^-20

struct RayPre {
    f3 o;
    float ix, iy, iz; // 1/d with |d| clamped away from 0
    uint32_t oct;     // bit a set: inverse direction negative along axis a
    int kx, ky, kz;   // watertight shear axes
    float sx, sy, sz;
    float okx, oky, okz;
};

MRT_DEV float sel3(float x, float y, float z, int k) { return k == 0 ? x : (k == 1 ? y : z); }

MRT_DEV float safe_inv(float d) {
    const float kTiny = 8.271806125530277e-25f; // 2^-80
    float dd = fabsf(d) < kTiny ? copysignf(kTiny, d) : d;
    return __frcp_rn(dd);
}

MRT_DEV RayPre ray_pre(f3 o, f3 d) {
    RayPre r;
    r.o = o;
    r.ix = safe_inv(d.x);
    r.iy = safe_inv(d.y);
    r.iz = safe_inv(d.z);
    r.oct = (r.ix < 0.0f ? 1u : 0u) | (r.iy < 0.0f ? 2u : 0u) | (r.iz < 0.0f ? 4u : 0u);
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int kz = (ax >= ay && ax >= az) ? 0 : (ay >= az ? 1 : 2);
    int kx = kz == 2 ? 0 : kz + 1;
    int ky = kx == 2 ? 0 : kx + 1;
    float dkz = sel3(d.x, d.y, d.z, kz);
    if (dkz < 0.0f) { int t = kx; kx = ky; ky = t; }
    r.kx = kx; r.ky = ky; r.kz = kz;
    r.sx = __fdiv_rn(sel3(d.x, d.y, d.z, kx), dkz);
    r.sy = __fdiv_rn(sel3(d.x, d.y, d.z, ky), dkz);
    r.sz = __frcp_rn(dkz);
    r.okx = sel3(o.x, o.y, o.z, kx);
    r.oky = sel3(o.x, o.y, o.z, ky);
    r.okz = sel3(o.x, o.y, o.z, kz);
    return r;
}

// Watertight test; returns true with t (> tmin) when the ray crosses the
// triangle (either facing).
MRT_DEV bool intersect_tri(const RayPre& r, float4 a, float4 b, float4 c, float tmin, float& t_out) {
    const float akx = __fsub_rn(sel3(a.x, a.y, a.z, r.kx), r.okx);
    const float aky = __fsub_rn(sel3(a.x, a.y, a.z, r.ky), r.oky);
    const float akz = __fsub_rn(sel3(a.x, a.y, a.z, r.kz), r.okz);
    const float bkx = __fsub_rn(sel3(b.x, b.y, b.z, r.kx), r.okx);
    const float bky = __fsub_rn(sel3(b.x, b.y, b.z, r.ky), r.oky);
    const float bkz = __fsub_rn(sel3(b.x, b.y, b.z, r.kz), r.okz);
    const float ckx = __fsub_rn(sel3(c.x, c.y, c.z, r.kx), r.okx);
    const float cky = __fsub_rn(sel3(c.x, c.y, c.z, r.ky), r.oky);
    const float ckz = __fsub_rn(sel3(c.x, c.y, c.z, r.kz), r.okz);
    const float Ax = fmaf(-r.sx, akz, akx), Ay = fmaf(-r.sy, akz, aky);
    const float Bx = fmaf(-r.sx, bkz, bkx), By = fmaf(-r.sy, bkz, bky);
    const float Cx = fmaf(-r.sx, ckz, ckx), Cy = fmaf(-r.sy, ckz, cky);
    float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
    float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
    float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = float(__dsub_rn(__dmul_rn(double(Cx), double(By)), __dmul_rn(double(Cy), double(Bx))));
        V = float(__dsub_rn(__dmul_rn(double(Ax), double(Cy)), __dmul_rn(double(Ay), double(Cx))));
        W = float(__dsub_rn(__dmul_rn(double(Bx), double(Ay)), __dmul_rn(double(By), double(Ax))));
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = __fadd_rn(__fadd_rn(U, V), W);
    if (det == 0.0f) return false;
    const float Az = __fmul_rn(r.sz, akz), Bz = __fmul_rn(r.sz, bkz), Cz = __fmul_rn(r.sz, ckz);
    const float T = fmaf(U, Az, fmaf(V, Bz, __fmul_rn(W, Cz)));
    if (T == 0.0f || ((T < 0.0f) != (det < 0.0f))) return false;
    const float t = __fdiv_rn(T, det);
    if (!(t > tmin)) return false;
    t_out = t;
    return true;
}

// Three-input min / max (one instruction on sm_100+; NaN inputs are
// ignored like fminf / fmaxf)
MRT_DEV float min3f(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
MRT_DEV float max3f(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

MRT_DEV float byte_to_float(uint32_t word, uint32_t k) {
    // 2^23 + byte as float bits, minus 2^23: exact
    return __fsub_rn(__int_as_float(__byte_perm(word, 0x4B000000u, k | 0x7440u)), 8388608.0f);
}

// Resumable traversal state of one ray.  The group (g_base, g_hits,
// g_imask) is the current internal-node group: base index of the children,
// hit keys (bit k: child slot k ^ oct), imask of the node the group came
// from.  Stack slot i of a thread lives at stk[i * stride].
struct Trav {
    RayPre r;
    float tmin, tmax, tbest;
    uint32_t best;
    uint32_t g_base, g_hits, g_imask;
    int sp;
    uint32_t iters;
};

// `root` is the index of the BVH8 root node: 0 for a single scene, the
// scene's first node in a concatenated multi-scene BVH.
MRT_DEV void trav_init(Trav& s, f3 o, f3 d, float tmin, float tmax, uint32_t root = 0u) {
    s.r = ray_pre(o, d);
    s.tmin = tmin;
    s.tmax = tmax;
    s.tbest = tmax;
    s.best = kMiss;
    s.g_base = root;
    s.g_hits = 1u << s.r.oct; // the root is child slot 0 of a virtual group
    s.g_imask = 1u;
    s.sp = 0;
    s.iters = 0u;
}

// Pops the next node of the ray's traversal into `node`.  Returns false
// when the traversal is finished (empty stack) or stopped with a status bit:
// stack overflow, or the iteration cap (node_count + 64 node visits) that
// ends a ray whose BVH links cycle, or a node index out of range.
template <int kStack>
MRT_DEV bool next_node(const DevScene& sc, Trav& s, uint2* stk, uint32_t stride, uint32_t& status, uint32_t& node) {
    if (s.g_hits == 0u) {
        if (s.sp == 0) return false;
        --s.sp;
        const uint2 e = stk[s.sp * stride];
        s.g_base = e.x;
        s.g_hits = e.y >> 8;
        s.g_imask = e.y & 0xFFu;
    }
    const uint32_t key = __ffs(s.g_hits) - 1u;
    s.g_hits &= s.g_hits - 1u;
    const uint32_t slot = key ^ s.r.oct;
    node = s.g_base + __popc(s.g_imask & ((1u << slot) - 1u));
    if (s.g_hits) {
        if (s.sp >= kStack) { status |= MRT_STATUS_STACK_OVF; return false; }
        stk[s.sp * stride] = make_uint2(s.g_base, (s.g_hits << 8) | s.g_imask);
        ++s.sp;
    }
    if (++s.iters > sc.node_count + 64u) { status |= MRT_STATUS_ITER_CAP; return false; }
    if (node >= sc.node_count) { status |= MRT_STATUS_BAD_NODE; return false; }
    return true;
}

// Box tests of the 8 children of one node against ray r with [tmin, tbest]:
// the hit interior children as bit keys (slot ^ oct, so that the lowest key
// is the nearest child for rays in octant oct), the triangles of the hit
// leaves as a bit mask relative to tri_base; child_base and imask describe
// the node's interior children.
MRT_DEV void node_test(const DevScene& sc, const RayPre& r, float tmin, float tbest, uint32_t oct, uint32_t node,
                       uint32_t& int_keys, uint32_t& tri_mask, uint32_t& child_base, uint32_t& tri_base,
                       uint32_t& imask_out) {
    const bool negx = r.ix < 0.0f, negy = r.iy < 0.0f, negz = r.iz < 0.0f;

    const uint4* np = sc.nodes + size_t(node) * 8u;
    const uint4 L0 = __ldg(np + 0), L1 = __ldg(np + 1), L2 = __ldg(np + 2), L3 = __ldg(np + 3),
                L4 = __ldg(np + 4);
    const int ex = int(int8_t(L0.w & 0xFFu)), ey = int(int8_t((L0.w >> 8) & 0xFFu)),
              ez = int(int8_t((L0.w >> 16) & 0xFFu));
    const uint32_t imask = L0.w >> 24;
    const float scx = __fmul_rn(__int_as_float((ex + 127) << 23), r.ix);
    const float scy = __fmul_rn(__int_as_float((ey + 127) << 23), r.iy);
    const float scz = __fmul_rn(__int_as_float((ez + 127) << 23), r.iz);
    const float adx = __fmul_rn(__fsub_rn(__uint_as_float(L0.x), r.o.x), r.ix);
    const float ady = __fmul_rn(__fsub_rn(__uint_as_float(L0.y), r.o.y), r.iy);
    const float adz = __fmul_rn(__fsub_rn(__uint_as_float(L0.z), r.o.z), r.iz);
    // near/far quantised planes per axis, chosen by the direction sign
    const uint32_t nx0 = negx ? L3.z : L2.x, nx1 = negx ? L3.w : L2.y;
    const uint32_t fx0 = negx ? L2.x : L3.z, fx1 = negx ? L2.y : L3.w;
    const uint32_t ny0 = negy ? L4.x : L2.z, ny1 = negy ? L4.y : L2.w;
    const uint32_t fy0 = negy ? L2.z : L4.x, fy1 = negy ? L2.w : L4.y;
    const uint32_t nz0 = negz ? L4.z : L3.x, nz1 = negz ? L4.w : L3.y;
    const uint32_t fz0 = negz ? L3.x : L4.z, fz1 = negz ? L3.y : L4.w;

    int_keys = 0u;
    tri_mask = 0u;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const uint32_t k = uint32_t(i & 3);
        const float tnx = fmaf(byte_to_float(i < 4 ? nx0 : nx1, k), scx, adx);
        const float tny = fmaf(byte_to_float(i < 4 ? ny0 : ny1, k), scy, ady);
        const float tnz = fmaf(byte_to_float(i < 4 ? nz0 : nz1, k), scz, adz);
        const float tfx = fmaf(byte_to_float(i < 4 ? fx0 : fx1, k), scx, adx);
        const float tfy = fmaf(byte_to_float(i < 4 ? fy0 : fy1, k), scy, ady);
        const float tfz = fmaf(byte_to_float(i < 4 ? fz0 : fz1, k), scz, adz);
        const float tn = max3f(tnx, tny, fmaxf(tnz, tmin));
        const float tf = min3f(tfx, tfy, fminf(tfz, tbest));
        if (tn <= __fmul_rn(tf, kRobustScale)) {
            const uint32_t meta = ((i < 4 ? L1.z : L1.w) >> (8 * k)) & 0xFFu;
            if ((imask >> i) & 1u) int_keys |= 1u << (uint32_t(i) ^ oct);
            else tri_mask |= (meta >> 5) << (meta & 31u);
        }
    }
    child_base = L1.x;
    tri_base = L1.y;
    imask_out = imask;
}

// Box tests of the 8 children of one node: the hit interior children become
// the ray's current group (s.g_*); the triangles of the hit leaves are
// returned as a bit mask relative to tri_base.
MRT_DEV uint32_t visit_node(const DevScene& sc, Trav& s, uint32_t node, uint32_t& tri_base) {
    uint32_t int_keys, tri_mask, child_base, imask;
    node_test(sc, s.r, s.tmin, s.tbest, s.r.oct, node, int_keys, tri_mask, child_base, tri_base, imask);
    s.g_base = child_base;
    s.g_hits = int_keys;
    s.g_imask = imask;
    return tri_mask;
}

// Watertight test of triangle ti against the ray.  Closest hit: keeps the
// nearest t, ties to the lower primitive id (the result does not depend on
// the order of the tests).  Any hit: returns true at the first t < tmax.
// A triangle index out of range sets a status bit and returns true.
template <bool kAnyHit>
MRT_DEV bool test_tri(const DevScene& sc, Trav& s, uint32_t ti, uint32_t& status) {
    if (ti >= sc.tri_count) { status |= MRT_STATUS_BAD_TRI; return true; }
    const float4* tp = sc.tris + size_t(ti) * 3u;
    const float4 a = __ldg(tp + 0), b = __ldg(tp + 1), c = __ldg(tp + 2);
    float t;
    if (intersect_tri(s.r, a, b, c, s.tmin, t)) {
        const uint32_t id = __float_as_uint(a.w);
        if (kAnyHit) {
            if (t < s.tmax) { s.best = id; s.tbest = t; return true; }
        } else if (t < s.tbest || (t == s.tbest && id < s.best)) {
            s.tbest = t;
            s.best = id;
        }
    }
    return false;
}

// One traversal step: visit the next node and test the triangles of its hit
// leaves.  Returns true when the ray is finished (s.best / s.tbest hold the
// result).  Every path through the step is bounded: one node and at most 24
// triangle tests.
template <bool kAnyHit, bool kCount, int kStack>
MRT_DEV bool trav_step(const DevScene& sc, Trav& s, uint2* stk, uint32_t stride, uint32_t& status,
                       uint32_t& cnt_nodes, uint32_t& cnt_tris) {
    uint32_t node;
    if (!next_node<kStack>(sc, s, stk, stride, status, node)) return true;
    if (kCount) ++cnt_nodes;
    uint32_t tri_base;
    uint32_t tri_mask = visit_node(sc, s, node, tri_base);
    while (tri_mask) {
        const uint32_t bit = __ffs(tri_mask) - 1u;
        tri_mask &= tri_mask - 1u;
        if (kCount) ++cnt_tris;
        if (test_tri<kAnyHit>(sc, s, tri_base + bit, status)) return true;
    }
    return s.g_hits == 0u && s.sp == 0;
}

// Unsigned key with the order of the floats (any non-NaN value).
MRT_DEV uint32_t float_key(float f) {
    const uint32_t u = __float_as_uint(f);
    return u ^ ((u >> 31) ? 0xFFFFFFFFu : 0x80000000u);
}
MRT_DEV float key_float(uint32_t k) { return __uint_as_float(k ^ ((k >> 31) ? 0x80000000u : 0xFFFFFFFFu)); }

// trav_step with the triangle tests of the step spread over the warp.  In
// the per-lane loop a step tests a leaf's triangles one per pass, and the
// warp runs as many passes as its busiest lane needs while the other lanes
// idle.  Here all 32 lanes call the step (`have` marks those holding a
// ray); each visits its next node as trav_step does, then the n_i triangles
// of lane i's hit leaves (T in all) become T (ray, triangle) pairs tested 32
// per pass: pair p goes to lane p mod 32, which finds the ray's owner by a
// binary search over the exclusive prefix sum of n_i and reads the owner's
// sheared ray with shuffles.  Hits meet in the owner's 64-bit shared slot
// (`slot`, 32 per warp) by atomicMin: (ordered t, id) for closest hit,
// which is test_tri's order-independent rule, so the result is identical;
// (leaf bit + 1, t) for any hit, which keeps the hit the per-lane loop
// would have met first.  Key 0 marks a triangle index out of range (no real key
// is 0), which ends the ray as test_tri does.  Returns true for a lane
// whose ray is finished.  Counting kernels keep the per-lane loop, whose
// per-ray counts are the oracle's.
template <bool kAnyHit, int kStack>
MRT_DEV bool trav_step_spread(const DevScene& sc, Trav& s, bool have, uint2* stk, uint32_t stride,
                              uint32_t& status, unsigned long long* slot) {
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t tri_mask = 0u, tri_base = 0u;
    bool done = false;
    if (have) {
        uint32_t node;
        if (next_node<kStack>(sc, s, stk, stride, status, node)) tri_mask = visit_node(sc, s, node, tri_base);
        else done = true;
    }
    const uint32_t cnt = __popc(tri_mask);
    uint32_t incl = cnt;
#pragma unroll
    for (uint32_t o = 1; o < 32u; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += v;
    }
    const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
    if (total) {
        const uint32_t excl = incl - cnt;
        if (cnt)
            slot[lane] = kAnyHit ? ~0ull
                                 : ((unsigned long long)float_key(s.tbest) << 32) | (unsigned long long)s.best;
        __syncwarp();
        const uint32_t kpack = uint32_t(s.r.kx) | (uint32_t(s.r.ky) << 2) | (uint32_t(s.r.kz) << 4);
        for (uint32_t c = 0; c < total; c += 32u) {
            const uint32_t p = c + lane;
            uint32_t own = 0u;  // the last lane whose exclusive sum is <= p
#pragma unroll
            for (uint32_t step = 16u; step >= 1u; step >>= 1) {
                const uint32_t e = __shfl_sync(0xFFFFFFFFu, excl, int(own + step));
                if (e <= p) own += step;
            }
            RayPre r;
            r.okx = __shfl_sync(0xFFFFFFFFu, s.r.okx, int(own));
            r.oky = __shfl_sync(0xFFFFFFFFu, s.r.oky, int(own));
            r.okz = __shfl_sync(0xFFFFFFFFu, s.r.okz, int(own));
            r.sx = __shfl_sync(0xFFFFFFFFu, s.r.sx, int(own));
            r.sy = __shfl_sync(0xFFFFFFFFu, s.r.sy, int(own));
            r.sz = __shfl_sync(0xFFFFFFFFu, s.r.sz, int(own));
            const uint32_t kp = __shfl_sync(0xFFFFFFFFu, kpack, int(own));
            r.kx = int(kp & 3u);
            r.ky = int((kp >> 2) & 3u);
            r.kz = int(kp >> 4);
            const float tmin = __shfl_sync(0xFFFFFFFFu, s.tmin, int(own));
            const float tmax = kAnyHit ? __shfl_sync(0xFFFFFFFFu, s.tmax, int(own)) : 0.0f;
            const uint32_t m = __shfl_sync(0xFFFFFFFFu, tri_mask, int(own));
            const uint32_t base = __shfl_sync(0xFFFFFFFFu, tri_base, int(own));
            const uint32_t e0 = __shfl_sync(0xFFFFFFFFu, excl, int(own));
            if (p < total) {
                const uint32_t bit = __fns(m, 0u, int(p - e0) + 1);
                const uint32_t ti = base + bit;
                if (ti >= sc.tri_count) {
                    status |= MRT_STATUS_BAD_TRI;
                    atomicMin(slot + own, 0ull);
                } else {
                    const float4* tp = sc.tris + size_t(ti) * 3u;
                    const float4 a = __ldg(tp + 0), b = __ldg(tp + 1), cc = __ldg(tp + 2);
                    float t;
                    if (intersect_tri(r, a, b, cc, tmin, t)) {
                        if (kAnyHit) {
                            if (t < tmax)
                                atomicMin(slot + own, ((unsigned long long)(bit + 1u) << 32) | __float_as_uint(t));
                        } else {
                            atomicMin(slot + own, ((unsigned long long)float_key(t) << 32) |
                                                      (unsigned long long)__float_as_uint(a.w));
                        }
                    }
                }
            }
        }
        __syncwarp();
        if (cnt) {
            const unsigned long long k = slot[lane];
            if (k == 0ull) {
                done = true;
            } else if (kAnyHit) {
                if (k != ~0ull) {
                    s.tbest = __uint_as_float(uint32_t(k));
                    s.best = __float_as_uint(__ldg(sc.tris + size_t(tri_base + uint32_t(k >> 32) - 1u) * 3u).w);
                    done = true;
                }
            } else {
                s.tbest = key_float(uint32_t(k >> 32));
                s.best = uint32_t(k);
            }
        }
    }
    if (have && !done) done = s.g_hits == 0u && s.sp == 0;
    return done;
}

// trav_step_spread for lanes that mix closest-hit and any-hit queries
// (any_hit per lane; the path tail's lanes are at different points of
// their paths).  The same steps, with the owner's kind read by a shuffle.
template <int kStack>
MRT_DEV bool trav_step_spread_mixed(const DevScene& sc, Trav& s, bool have, bool any_hit, uint2* stk,
                                    uint32_t stride, uint32_t& status, unsigned long long* slot) {
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t tri_mask = 0u, tri_base = 0u;
    bool done = false;
    if (have) {
        uint32_t node;
        if (next_node<kStack>(sc, s, stk, stride, status, node)) tri_mask = visit_node(sc, s, node, tri_base);
        else done = true;
    }
    const uint32_t cnt = __popc(tri_mask);
    uint32_t incl = cnt;
#pragma unroll
    for (uint32_t o = 1; o < 32u; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += v;
    }
    const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
    if (total) {
        const uint32_t excl = incl - cnt;
        if (cnt)
            slot[lane] = any_hit ? ~0ull
                                 : ((unsigned long long)float_key(s.tbest) << 32) | (unsigned long long)s.best;
        __syncwarp();
        const uint32_t kpack = uint32_t(s.r.kx) | (uint32_t(s.r.ky) << 2) | (uint32_t(s.r.kz) << 4);
        for (uint32_t c = 0; c < total; c += 32u) {
            const uint32_t p = c + lane;
            uint32_t own = 0u;  // the last lane whose exclusive sum is <= p
#pragma unroll
            for (uint32_t step = 16u; step >= 1u; step >>= 1) {
                const uint32_t e = __shfl_sync(0xFFFFFFFFu, excl, int(own + step));
                if (e <= p) own += step;
            }
            RayPre r;
            r.okx = __shfl_sync(0xFFFFFFFFu, s.r.okx, int(own));
            r.oky = __shfl_sync(0xFFFFFFFFu, s.r.oky, int(own));
            r.okz = __shfl_sync(0xFFFFFFFFu, s.r.okz, int(own));
            r.sx = __shfl_sync(0xFFFFFFFFu, s.r.sx, int(own));
            r.sy = __shfl_sync(0xFFFFFFFFu, s.r.sy, int(own));
            r.sz = __shfl_sync(0xFFFFFFFFu, s.r.sz, int(own));
            const uint32_t kp = __shfl_sync(0xFFFFFFFFu, kpack, int(own));
            r.kx = int(kp & 3u);
            r.ky = int((kp >> 2) & 3u);
            r.kz = int(kp >> 4);
            const float tmin = __shfl_sync(0xFFFFFFFFu, s.tmin, int(own));
            const bool own_any = __shfl_sync(0xFFFFFFFFu, uint32_t(any_hit), int(own)) != 0u;
            const float tmax = __shfl_sync(0xFFFFFFFFu, s.tmax, int(own));
            const uint32_t m = __shfl_sync(0xFFFFFFFFu, tri_mask, int(own));
            const uint32_t base = __shfl_sync(0xFFFFFFFFu, tri_base, int(own));
            const uint32_t e0 = __shfl_sync(0xFFFFFFFFu, excl, int(own));
            if (p < total) {
                const uint32_t bit = __fns(m, 0u, int(p - e0) + 1);
                const uint32_t ti = base + bit;
                if (ti >= sc.tri_count) {
                    status |= MRT_STATUS_BAD_TRI;
                    atomicMin(slot + own, 0ull);
                } else {
                    const float4* tp = sc.tris + size_t(ti) * 3u;
                    const float4 a = __ldg(tp + 0), b = __ldg(tp + 1), cc = __ldg(tp + 2);
                    float t;
                    if (intersect_tri(r, a, b, cc, tmin, t)) {
                        if (own_any) {
                            if (t < tmax)
                                atomicMin(slot + own, ((unsigned long long)(bit + 1u) << 32) | __float_as_uint(t));
                        } else {
                            atomicMin(slot + own, ((unsigned long long)float_key(t) << 32) |
                                                      (unsigned long long)__float_as_uint(a.w));
                        }
                    }
                }
            }
        }
        __syncwarp();
        if (cnt) {
            const unsigned long long k = slot[lane];
            if (k == 0ull) {
                done = true;
            } else if (any_hit) {
                if (k != ~0ull) {
                    s.tbest = __uint_as_float(uint32_t(k));
                    s.best = __float_as_uint(__ldg(sc.tris + size_t(tri_base + uint32_t(k >> 32) - 1u) * 3u).w);
                    done = true;
                }
            } else {
                s.tbest = key_float(uint32_t(k >> 32));
                s.best = uint32_t(k);
            }
        }
    }
    if (have && !done) done = s.g_hits == 0u && s.sp == 0;
    return done;
}

// Closest hit (kAnyHit = false) or first hit with t < tmax (kAnyHit = true)
// of one ray, run to completion.
template <bool kAnyHit, bool kCount, int kStack>
MRT_DEV void trace_bvh8(const DevScene& sc, f3 o, f3 d, float tmin, float tmax, uint32_t& hit_prim,
                        float& hit_t, uint2* stk, uint32_t stride, uint32_t& status,
                        uint32_t& cnt_nodes, uint32_t& cnt_tris) {
    Trav s;
    trav_init(s, o, d, tmin, tmax);
    while (!trav_step<kAnyHit, kCount, kStack>(sc, s, stk, stride, status, cnt_nodes, cnt_tris)) {
    }
    hit_prim = s.best;
    hit_t = s.best == kMiss ? s.tmax : s.tbest;
}

// Reference ray/sphere test (intersect.glsl:26-37): the nearer root of
// |o + t d - c|^2 = r^2, or -1 when the discriminant is negative.  It never
// returns the far root, so an origin inside a sphere reads as t < 0.
MRT_DEV float ray_sphere(f3 o, f3 d, f3 c, float radius) {
    const f3 oc = sub_rn(o, c);
    const float a = dot_rn(d, d);
    const float half_b = dot_rn(oc, d);
    const float cc = __fsub_rn(dot_rn(oc, oc), __fmul_rn(radius, radius));
    const float disc = __fsub_rn(__fmul_rn(half_b, half_b), __fmul_rn(a, cc));
    if (disc < 0.0f) return -1.0f;
    return __fdiv_rn(__fsub_rn(-half_b, __fsqrt_rn(disc)), a);
}

} // namespace mrt
