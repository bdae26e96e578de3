// Batched multi-scene tracing: many scenes of uneven triangle and ray
// counts in one persistent launch, and a closest-hit Lambertian bounce loop
// over all of them captured once into a CUDA graph.  The reference renders
// a single compiled-in scene; this is new.
//
// Layout: the scenes' BVH8 nodes, leaf-ordered triangles and materials are
// concatenated; child_base / tri_base of every node and every triangle id
// are rebased on the host, so traversal is unchanged except that each ray
// starts at its scene's root node (trav_init's `root`).
#include "internal.hpp"

#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

namespace mrt {
int set_error(mrt_ctx* ctx, int code, const char* msg);
int persistent_blocks(mrt_ctx* ctx);
TraceParams make_trace_params(const mrt_trace_params* p);
}

using namespace mrt;

constexpr uint32_t kMaxBatchScenes = 4096;
constexpr int kMaxBatchStack = 32;  // stack entries of the deepest kernel variant

// Stack entries the batched traversal uses: mrt_tuning.stack_depth (16, 24
// or 32; 0 = the default 24).  Returns 0 when it is below what the batch's
// deepest BVH needs (depth - 1 entries).
int batch_stack(const mrt_ctx* ctx, uint32_t max_depth) {
    const int want = ctx->tuning.stack_depth ? int(ctx->tuning.stack_depth) : kStackDepth;
    return uint32_t(want) + 1u >= max_depth ? want : 0;
}

struct mrt_batch {
    uint32_t scenes = 0;
    uint32_t max_depth = 0;          // deepest scene BVH (levels)
    DevScene dev{};
    void* d_nodes = nullptr;
    void* d_tris = nullptr;
    void* d_mats = nullptr;
    uint32_t* d_roots = nullptr;     // first node of each scene
    uint32_t* d_ray_off = nullptr;   // scenes + 1 ray offsets of the current call
    std::vector<uint32_t> h_ray_off;
    // path-trace state (sized for the largest call so far)
    size_t cap = 0;
    PathRay* q[2] = {nullptr, nullptr};
    ShadowRay* sq = nullptr;         // shadow rays of one vertex (next-event estimation)
    uint2* hits = nullptr;
    uint32_t* rng = nullptr;
    uint32_t* counters = nullptr;
    TraceParams* d_tp = nullptr;     // parameters read by the graph's kernels
    uint32_t* d_frame = nullptr;
    TraceParams* h_tp = nullptr;     // pinned staging for the per-call copy
    uint32_t* h_frame = nullptr;
    // captured bounce loop and what it was captured for
    cudaGraphExec_t exec = nullptr;
    cudaStream_t cap_stream = nullptr;
    const void* g_rays = nullptr;
    float* g_radiance = nullptr;
    uint32_t g_n = 0, g_bounces = 0, g_blocks = 0, g_dyn = 0;
    int g_stack = 0;
    bool g_spread = false, g_nee = false;
    uint32_t g_refill = 0;
};

namespace {

// scene of ray i: the last s with off[s] <= i (off in shared memory)
MRT_DEV uint32_t scene_of(const uint32_t* off, uint32_t scenes, uint32_t i) {
    uint32_t lo = 0, hi = scenes;  // invariant: off[lo] <= i < off[hi]
    while (hi - lo > 1u) {
        const uint32_t mid = (lo + hi) >> 1;
        if (off[mid] <= i) lo = mid;
        else hi = mid;
    }
    return lo;
}

// As warp_refill (kernels.cu), with the same min_idle rule.
__device__ __forceinline__ uint32_t refill(uint32_t* fetch, uint32_t n, bool need, bool& exhausted,
                                           uint32_t min_idle) {
    if (exhausted) return kMiss;
    const uint32_t mask = __ballot_sync(0xFFFFFFFFu, need);
    if (!mask) return kMiss;
    if (mask != 0xFFFFFFFFu && uint32_t(__popc(mask)) < min_idle) return kMiss;
    const uint32_t lane = lane_id(), leader = __ffs(mask) - 1u, cnt = __popc(mask);
    uint32_t base = 0u;
    if (lane == leader) base = atomicAdd(fetch, cnt);
    base = __shfl_sync(0xFFFFFFFFu, base, leader);
    if (base + cnt >= n) exhausted = true;
    if (!need) return kMiss;
    const uint32_t i = base + __popc(mask & ((1u << lane) - 1u));
    return i < n ? i : kMiss;
}

// One persistent launch over the rays of all scenes (per-lane refill);
// kStack: traversal stack entries per ray (a tuning choice: 16, 24 or 32);
// kSpread: the triangle tests of each step spread over the warp
// (trav_step_spread; same hits).
template <bool kAnyHit, int kStack, bool kSpread>
__global__ void __launch_bounds__(kTraceBlock, kTraceMinBlocks)
k_batch_trace(DevScene sc, const uint32_t* roots, const uint32_t* ray_off, uint32_t scenes, const mrt_ray* rays,
              uint32_t n, mrt_hit* hits, uint32_t* fetch, uint32_t* status, uint32_t refill_min) {
    __shared__ uint2 stk[kStack * kTraceBlock];
    __shared__ unsigned long long slots[kSpread ? kTraceBlock : 1];
    extern __shared__ uint32_t off[];  // scenes + 1 ray offsets
    for (uint32_t i = threadIdx.x; i <= scenes; i += blockDim.x) off[i] = ray_off[i];
    __syncthreads();
    uint2* my = stk + threadIdx.x;
    uint32_t st = 0u, cn = 0u, ct = 0u, ri = 0u;
    Trav s{};
    bool have = false, exhausted = false;
    while (true) {
        const uint32_t idx = refill(fetch, n, !have, exhausted, refill_min);
        if (idx != kMiss) {
            const float4* rp = reinterpret_cast<const float4*>(rays + idx);
            const float4 a = rp[0], b = rp[1];
            const uint32_t scn = scene_of(off, scenes, idx);
            trav_init(s, f3{a.x, a.y, a.z}, f3{b.x, b.y, b.z}, a.w, b.w, roots[scn]);
            ri = idx;
            have = true;
        }
        if (!__any_sync(0xFFFFFFFFu, have)) break;
        bool fin;
        if (kSpread)
            fin = trav_step_spread<kAnyHit, kStack>(sc, s, have, my, kTraceBlock, st, slots + (threadIdx.x & ~31u));
        else
            fin = have && trav_step<kAnyHit, false, kStack>(sc, s, my, kTraceBlock, st, cn, ct);
        if (have && fin) {
            hits[ri].prim = s.best;
            hits[ri].t = s.best == kMiss ? s.tmax : s.tbest;
            have = false;
        }
    }
    if (st) atomicOr(status, st);
}

// Bounce loop state: queue entry = origin | ray index, direction | scene,
// throughput | tmax.
__global__ void __launch_bounds__(kShadeBlock)
k_batch_init(const mrt_ray* rays, const uint32_t* ray_off, uint32_t scenes, uint32_t n, PathRay* q0, uint32_t* rng,
             float* radiance, uint32_t* counters, const uint32_t* frame) {
    extern __shared__ uint32_t off[];  // scenes + 1 ray offsets
    for (uint32_t i = threadIdx.x; i <= scenes; i += blockDim.x) off[i] = ray_off[i];
    __syncthreads();
    const uint32_t f = *frame;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4* rp = reinterpret_cast<const float4*>(rays + i);
        const float4 a = rp[0], b = rp[1];
        PathRay pr;
        pr.o_pix = make_float4(a.x, a.y, a.z, __uint_as_float(i));
        pr.d = make_float4(b.x, b.y, b.z, __uint_as_float(scene_of(off, scenes, i)));
        pr.beta = make_float4(1.0f, 1.0f, 1.0f, b.w);
        q0[i] = pr;
        uint32_t h = i * 0x9E3779B1u + ((f << 1u) | 1u);
        rng[i] = pcg(h) | 1u;
        radiance[3 * size_t(i) + 0] = 0.0f;
        radiance[3 * size_t(i) + 1] = 0.0f;
        radiance[3 * size_t(i) + 2] = 0.0f;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) counters[kCntExt] = n;
}

template <int kStack, bool kSpread>
__global__ void __launch_bounds__(kTraceBlock, kTraceMinBlocks)
k_batch_trace_queue(DevScene sc, const uint32_t* roots, const PathRay* q, uint2* hits, uint32_t* counters,
                    uint32_t bounce, uint32_t* status, uint32_t refill_min) {
    __shared__ uint2 stk[kStack * kTraceBlock];
    __shared__ unsigned long long slots[kSpread ? kTraceBlock : 1];
    const uint32_t n = counters[kCntExt + bounce];
    uint32_t* fetch = counters + kCntFetchExt + bounce;
    uint2* my = stk + threadIdx.x;
    uint32_t st = 0u, cn = 0u, ct = 0u, ri = 0u;
    Trav s{};
    bool have = false, exhausted = false;
    while (true) {
        const uint32_t idx = refill(fetch, n, !have, exhausted, refill_min);
        if (idx != kMiss) {
            const PathRay pr = q[idx];
            const float tmax = bounce == 0u ? pr.beta.w : INFINITY;
            trav_init(s, f3{pr.o_pix.x, pr.o_pix.y, pr.o_pix.z}, f3{pr.d.x, pr.d.y, pr.d.z}, 0.0f, tmax,
                      roots[__float_as_uint(pr.d.w)]);
            ri = idx;
            have = true;
        }
        if (!__any_sync(0xFFFFFFFFu, have)) break;
        bool fin;
        if (kSpread)
            fin = trav_step_spread<false, kStack>(sc, s, have, my, kTraceBlock, st, slots + (threadIdx.x & ~31u));
        else
            fin = have && trav_step<false, false, kStack>(sc, s, my, kTraceBlock, st, cn, ct);
        if (have && fin) {
            hits[ri] = make_uint2(s.best, __float_as_uint(s.best == kMiss ? s.tmax : s.tbest));
            have = false;
        }
    }
    if (st) atomicOr(status, st);
}

// Queue slot of this thread among the block's threads that `want` one:
// one global atomic per block (a warp-level atomic per warp makes the
// warps of a large bounce queue up on the counter).  All threads of the
// block must call it the same number of times.
__device__ __forceinline__ uint32_t block_append(uint32_t* counter, bool want) {
    constexpr int kWarps = kShadeBlock / 32;
    __shared__ uint32_t wsum[kWarps];
    __shared__ uint32_t base;
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    const uint32_t mask = __ballot_sync(0xFFFFFFFFu, want);
    if (lane == 0u) wsum[warp] = __popc(mask);
    __syncthreads();
    if (threadIdx.x == 0u) {  // exclusive scan of the warps' counts, one atomic
        uint32_t acc = 0u;
        for (int w = 0; w < kWarps; ++w) {
            const uint32_t c = wsum[w];
            wsum[w] = acc;
            acc += c;
        }
        base = acc ? atomicAdd(counter, acc) : 0u;
    }
    __syncthreads();
    const uint32_t slot = base + wsum[warp] + __popc(mask & ((1u << lane) - 1u));
    __syncthreads();  // wsum and base are reused by the next call
    return slot;
}

// Shade vertex `bounce`: escape adds throughput x sky; a hit (with
// next-event estimation) emits a shadow ray toward the directional light
// carrying throughput x albedo x irradiance x cos / pi, multiplies the
// albedo and, below the bounce limit, appends a cosine-weighted bounce ray
// (normalize(n + uniform sphere point), random.glsl:10-19 with per-ray PCG
// numbers) with Russian roulette past rr_start: the single-scene
// wavefront's estimator (shade_vertex) with per-ray random numbers.
// kNee: compiled per estimator (the escape-only form keeps its registers).
template <bool kNee>
__global__ void __launch_bounds__(kShadeBlock)
k_batch_shade(DevScene sc, const TraceParams* tpp, const PathRay* qin, PathRay* qout, ShadowRay* sq,
              const uint2* hits, uint32_t* rng, float* radiance, uint32_t* counters, uint32_t bounce,
              uint32_t* status) {
    const TraceParams tp = *tpp;
    const uint32_t n = counters[kCntExt + bounce];
    const uint32_t rounded = (n + kShadeBlock - 1u) / kShadeBlock * kShadeBlock;  // same trip count per block
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < rounded; i += gridDim.x * blockDim.x) {
        bool want = false, want_sh = false;
        PathRay out;
        ShadowRay sr;
        if (i < n) {
            const PathRay pr = qin[i];
            const uint2 h = hits[i];
            const uint32_t idx = __float_as_uint(pr.o_pix.w);
            f3 beta{pr.beta.x, pr.beta.y, pr.beta.z};
            if (h.x == kMiss) {
                // the path's only addition without next-event estimation
                // (radiance starts at zero); after its shadow rays' otherwise
                float* r = radiance + 3 * size_t(idx);
                const f3 e{__fmul_rn(beta.x, tp.sky[0]), __fmul_rn(beta.y, tp.sky[1]), __fmul_rn(beta.z, tp.sky[2])};
                r[0] = kNee ? __fadd_rn(r[0], e.x) : e.x;
                r[1] = kNee ? __fadd_rn(r[1], e.y) : e.y;
                r[2] = kNee ? __fadd_rn(r[2], e.z) : e.z;
            } else if (h.x < sc.mat_count) {
                const mrt_material m = sc.mats[h.x];
                const f3 d{pr.d.x, pr.d.y, pr.d.z};
                f3 nrm{m.normal[0], m.normal[1], m.normal[2]};
                if (dot_rn(nrm, d) > 0.0f) nrm = f3{-nrm.x, -nrm.y, -nrm.z};
                const f3 rho{__fdiv_rn(float(m.albedo_rgba8 & 0xFFu), 255.0f),
                             __fdiv_rn(float((m.albedo_rgba8 >> 8) & 0xFFu), 255.0f),
                             __fdiv_rn(float((m.albedo_rgba8 >> 16) & 0xFFu), 255.0f)};
                const f3 p = add_rn(f3{pr.o_pix.x, pr.o_pix.y, pr.o_pix.z}, scale_rn(d, __uint_as_float(h.y)));
                if (kNee) {
                    const f3 sun{tp.sun[0], tp.sun[1], tp.sun[2]};
                    const float cosl = dot_rn(nrm, sun);
                    if (cosl > 0.0f) {
                        const f3 os = offset_ray(p, nrm);
                        const f3 c = scale_rn(mul_rn(mul_rn(beta, rho), f3{tp.sun_e[0], tp.sun_e[1], tp.sun_e[2]}),
                                              __fmul_rn(cosl, kInvPi));
                        want_sh = true;
                        sr.o_pix = make_float4(os.x, os.y, os.z, pr.o_pix.w);
                        sr.contrib = make_float4(c.x, c.y, c.z, pr.d.w);  // w: the scene (bits)
                    }
                }
                beta = mul_rn(beta, rho);
                if (bounce < tp.max_bounces) {
                    uint32_t s = rng[idx];
                    const float u1 = random_float(s), u2 = random_float(s);
                    const f3 sp = random_sphere_point(__fsub_rn(__fmul_rn(u1, 2.0f), 1.0f),
                                                      __fsub_rn(__fmul_rn(u2, 2.0f), 1.0f), tp.exact_trig);
                    f3 nd = add_rn(nrm, sp);
                    if (dot_rn(nd, nd) == 0.0f) nd = nrm;
                    nd = normalize_rn(nd);
                    bool live = true;
                    if (tp.rr_start != 0u && bounce + 1u > tp.rr_start) {
                        float qv = fminf(fmaxf(fmaxf(fmaxf(beta.x, beta.y), beta.z), 0.05f), 1.0f);
                        if (random_float(s) >= qv) live = false;
                        else beta = f3{__fdiv_rn(beta.x, qv), __fdiv_rn(beta.y, qv), __fdiv_rn(beta.z, qv)};
                    }
                    rng[idx] = s;
                    if (live) {
                        const f3 o = offset_ray(p, nrm);
                        want = true;
                        out.o_pix = make_float4(o.x, o.y, o.z, pr.o_pix.w);
                        out.d = make_float4(nd.x, nd.y, nd.z, pr.d.w);
                        out.beta = make_float4(beta.x, beta.y, beta.z, INFINITY);
                    }
                }
            } else {
                atomicOr(status, MRT_STATUS_BAD_TRI);
            }
        }
        const uint32_t slot = block_append(counters + kCntExt + bounce + 1u, want);
        if (want) qout[slot] = out;
        if (kNee) {
            const uint32_t ss = block_append(counters + kCntShadow + bounce, want_sh);
            if (want_sh) sq[ss] = sr;
        }
    }
}

// Any-hit trace of the shadow rays of vertex `vertex` (each from its own
// scene's root toward the directional light); unoccluded rays add their
// contribution to their path's radiance (one shadow ray per path and
// vertex, so no two threads add to the same path).
template <int kStack>
__global__ void __launch_bounds__(kTraceBlock, kTraceMinBlocks)
k_batch_trace_shadow(DevScene sc, const uint32_t* roots, const TraceParams* tpp, const ShadowRay* sq,
                     float* radiance, uint32_t* counters, uint32_t vertex, uint32_t* status, uint32_t refill_min) {
    __shared__ uint2 stk[kStack * kTraceBlock];
    const uint32_t n = counters[kCntShadow + vertex];
    uint32_t* fetch = counters + kCntFetchShadow + vertex;
    const f3 sun{tpp->sun[0], tpp->sun[1], tpp->sun[2]};
    uint2* my = stk + threadIdx.x;
    uint32_t st = 0u, cn = 0u, ct = 0u, ri = 0u;
    Trav s{};
    bool have = false, exhausted = false;
    while (true) {
        const uint32_t idx = refill(fetch, n, !have, exhausted, refill_min);
        if (idx != kMiss) {
            const float4 a = sq[idx].o_pix;
            trav_init(s, f3{a.x, a.y, a.z}, sun, 0.0f, INFINITY, roots[__float_as_uint(sq[idx].contrib.w)]);
            ri = idx;
            have = true;
        }
        if (!__any_sync(0xFFFFFFFFu, have)) break;
        const bool fin = have && trav_step<true, false, kStack>(sc, s, my, kTraceBlock, st, cn, ct);
        if (have && fin) {
            if (s.best == kMiss) {
                const ShadowRay r = sq[ri];
                float* L = radiance + 3 * size_t(__float_as_uint(r.o_pix.w));
                L[0] = __fadd_rn(L[0], r.contrib.x);
                L[1] = __fadd_rn(L[1], r.contrib.y);
                L[2] = __fadd_rn(L[2], r.contrib.z);
            }
            have = false;
        }
    }
    if (st) atomicOr(status, st);
}

// ray counts of the bounce loop into the context's totals (frame stats)
__global__ void k_batch_tally(const uint32_t* counters, unsigned long long* totals, uint32_t bounces) {
    const uint32_t v = threadIdx.x;
    if (v >= 1u && v <= bounces) atomicAdd(totals + kCntExt + v, (unsigned long long)counters[kCntExt + v]);
}

int free_batch_state(mrt_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
    cudaFree(b->q[0]); cudaFree(b->q[1]); cudaFree(b->sq); cudaFree(b->hits); cudaFree(b->rng);
    cudaFree(b->counters);
    b->exec = nullptr;
    b->cap_stream = nullptr;
    b->q[0] = b->q[1] = nullptr;
    b->sq = nullptr;
    b->hits = nullptr;
    b->rng = nullptr;
    b->counters = nullptr;
    b->cap = 0;
    return MRT_OK;
}

int upload_offsets(mrt_ctx* ctx, mrt_batch* b, const uint32_t* ray_offsets, uint32_t& n, cudaStream_t s) {
    for (uint32_t i = 0; i < b->scenes; ++i)
        if (ray_offsets[i + 1] < ray_offsets[i]) return set_error(ctx, MRT_EINVAL, "ray_offsets must not decrease");
    if (ray_offsets[0] != 0) return set_error(ctx, MRT_EINVAL, "ray_offsets[0] must be 0");
    n = ray_offsets[b->scenes];
    bool same = b->h_ray_off.size() == b->scenes + 1u &&
                std::memcmp(b->h_ray_off.data(), ray_offsets, (b->scenes + 1u) * sizeof(uint32_t)) == 0;
    if (!same) {
        b->h_ray_off.assign(ray_offsets, ray_offsets + b->scenes + 1u);
        // a pageable H2D copy returns once the source is consumed
        if (cudaMemcpyAsync(b->d_ray_off, b->h_ray_off.data(), (b->scenes + 1u) * sizeof(uint32_t),
                            cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return set_error(ctx, MRT_ECUDA, "ray offset upload failed");
    }
    return MRT_OK;
}

// acc[g][i] += scale * sum_c x[g][c][i] (g < groups, c < copies, i < count),
// four floats per thread
__global__ void k_accumulate_copies(float* acc, const float* x, uint32_t groups, uint32_t copies, size_t count,
                                    float scale) {
    const size_t q = count / 4, total = size_t(groups) * q;
    for (size_t k = blockIdx.x * size_t(blockDim.x) + threadIdx.x; k < total; k += size_t(gridDim.x) * blockDim.x) {
        const size_t g = k / q, i = k - g * q;
        const float4* src = reinterpret_cast<const float4*>(x) + g * copies * q + i;
        float4 s = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        for (uint32_t c = 0; c < copies; ++c) {
            const float4 v = src[size_t(c) * q];
            s.x += v.x; s.y += v.y; s.z += v.z; s.w += v.w;
        }
        float4* d = reinterpret_cast<float4*>(acc) + g * q + i;
        float4 a = *d;
        a.x = fmaf(scale, s.x, a.x);
        a.y = fmaf(scale, s.y, a.y);
        a.z = fmaf(scale, s.z, a.z);
        a.w = fmaf(scale, s.w, a.w);
        *d = a;
    }
}

} // namespace

extern "C" {

int mrt_cuda_accumulate_copies(mrt_ctx* ctx, float* acc, const float* x, uint32_t groups, uint32_t copies,
                               size_t count, float scale, void* stream) {
    if (!ctx || !acc || !x || groups == 0 || copies == 0 || count % 4 ||
        (reinterpret_cast<uintptr_t>(acc) | reinterpret_cast<uintptr_t>(x)) % 16)
        return set_error(ctx, MRT_EINVAL, "accumulate_copies: bad arguments");
    cudaSetDevice(ctx->device);
    const size_t total = size_t(groups) * (count / 4);
    const int blocks = int(std::min<size_t>((total + 255) / 256, size_t(ctx->sm_count) * 16));
    k_accumulate_copies<<<std::max(blocks, 1), 256, 0, static_cast<cudaStream_t>(stream)>>>(acc, x, groups, copies,
                                                                                            count, scale);
    if (cudaGetLastError() != cudaSuccess) return set_error(ctx, MRT_ECUDA, "accumulate_copies: launch");
    ctx->launches++;
    return MRT_OK;
}

int mrt_cuda_batch_create(mrt_ctx* ctx, uint32_t count, const mrt_bvh8_node* const* nodes,
                          const uint32_t* node_counts, const mrt_tri* const* tris, const uint32_t* tri_counts,
                          const mrt_material* const* materials, mrt_batch** out) {
    if (!ctx || !out || !nodes || !node_counts || !tris || !tri_counts || !materials || count == 0)
        return set_error(ctx, MRT_EINVAL, "batch_create: null argument or no scenes");
    if (count > kMaxBatchScenes) return set_error(ctx, MRT_ERANGE, "batch_create: more than 4096 scenes");
    *out = nullptr;
    uint64_t nn = 0, nt = 0;
    uint32_t max_depth = 0;
    for (uint32_t s = 0; s < count; ++s) {
        if (!nodes[s] || !tris[s] || !materials[s] || node_counts[s] == 0 || tri_counts[s] == 0)
            return set_error(ctx, MRT_EINVAL, "batch_create: empty scene");
        nn += node_counts[s];
        nt += tri_counts[s];
        max_depth = std::max(max_depth, bvh8_depth(nodes[s], node_counts[s]));
    }
    if (max_depth > uint32_t(kMaxBatchStack) + 1u)
        return set_error(ctx, MRT_ERANGE, "batch_create: a BVH8 deeper than the largest traversal stack (33 levels)");
    if (nn >= 0xFFFFFFFFull || nt >= 0xFFFFFFFFull) return set_error(ctx, MRT_ERANGE, "batch_create: too large");
    std::vector<mrt_bvh8_node> an;
    std::vector<mrt_tri> at;
    std::vector<mrt_material> am;
    std::vector<uint32_t> roots(count);
    an.reserve(nn);
    at.reserve(nt);
    am.reserve(nt);
    for (uint32_t s = 0; s < count; ++s) {
        const uint32_t nb = uint32_t(an.size()), tb = uint32_t(at.size());
        roots[s] = nb;
        for (uint32_t i = 0; i < node_counts[s]; ++i) {
            mrt_bvh8_node n = nodes[s][i];
            n.child_base += nb;
            n.tri_base += tb;
            an.push_back(n);
        }
        for (uint32_t i = 0; i < tri_counts[s]; ++i) {
            mrt_tri t = tris[s][i];
            t.id += tb;
            at.push_back(t);
        }
        // materials are indexed by the scene's original triangle id
        am.insert(am.end(), materials[s], materials[s] + tri_counts[s]);
    }
    mrt_batch* b = new (std::nothrow) mrt_batch;
    if (!b) return MRT_ENOMEM;
    b->scenes = count;
    bool ok = cudaMalloc(&b->d_nodes, an.size() * sizeof(mrt_bvh8_node)) == cudaSuccess &&
              cudaMalloc(&b->d_tris, at.size() * sizeof(mrt_tri)) == cudaSuccess &&
              cudaMalloc(&b->d_mats, am.size() * sizeof(mrt_material)) == cudaSuccess &&
              cudaMalloc(&b->d_roots, count * sizeof(uint32_t)) == cudaSuccess &&
              cudaMalloc(&b->d_ray_off, (count + 1) * sizeof(uint32_t)) == cudaSuccess &&
              cudaMalloc(&b->d_tp, sizeof(TraceParams)) == cudaSuccess &&
              cudaMalloc(&b->d_frame, sizeof(uint32_t)) == cudaSuccess &&
              cudaMallocHost(&b->h_tp, sizeof(TraceParams)) == cudaSuccess &&
              cudaMallocHost(&b->h_frame, sizeof(uint32_t)) == cudaSuccess;
    ok = ok && cudaMemcpy(b->d_nodes, an.data(), an.size() * sizeof(mrt_bvh8_node), cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(b->d_tris, at.data(), at.size() * sizeof(mrt_tri), cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(b->d_mats, am.data(), am.size() * sizeof(mrt_material), cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(b->d_roots, roots.data(), count * sizeof(uint32_t), cudaMemcpyHostToDevice) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        mrt_cuda_batch_destroy(ctx, b);
        return set_error(ctx, MRT_ENOMEM, "batch_create: device allocation or copy failed");
    }
    b->dev.nodes = static_cast<const uint4*>(b->d_nodes);
    b->dev.tris = static_cast<const float4*>(b->d_tris);
    b->dev.mats = static_cast<const mrt_material*>(b->d_mats);
    b->max_depth = max_depth;
    b->dev.node_count = uint32_t(an.size());
    b->dev.tri_count = uint32_t(at.size());
    b->dev.mat_count = uint32_t(am.size());
    *out = b;
    return MRT_OK;
}

int mrt_cuda_batch_destroy(mrt_ctx* ctx, mrt_batch* b) {
    if (!ctx || !b) return MRT_EINVAL;
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();
    free_batch_state(b);
    cudaFree(b->d_nodes); cudaFree(b->d_tris); cudaFree(b->d_mats); cudaFree(b->d_roots); cudaFree(b->d_ray_off);
    cudaFree(b->d_tp); cudaFree(b->d_frame);
    if (b->h_tp) cudaFreeHost(b->h_tp);
    if (b->h_frame) cudaFreeHost(b->h_frame);
    delete b;
    return MRT_OK;
}

int mrt_cuda_batch_trace(mrt_ctx* ctx, mrt_batch* b, const mrt_ray* rays, const uint32_t* ray_offsets, mrt_hit* hits,
                         uint32_t flags, void* stream) {
    if (!ctx || !b || !ray_offsets) return set_error(ctx, MRT_EINVAL, "batch_trace: null argument");
    cudaSetDevice(ctx->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    uint32_t n = 0;
    int rc = upload_offsets(ctx, b, ray_offsets, n, s);
    if (rc) return rc;
    if (n == 0) return MRT_OK;
    if (!rays || !hits) return set_error(ctx, MRT_EINVAL, "batch_trace: null rays or hits");
    // the context's primary-ray work counter doubles as this launch's counter
    if (cudaMemsetAsync(ctx->d_prim_fetch, 0, sizeof(uint32_t), s) != cudaSuccess)
        return set_error(ctx, MRT_ECUDA, "batch_trace: memset failed");
    const int blocks = persistent_blocks(ctx);
    const size_t dsm = (b->scenes + 1u) * sizeof(uint32_t);
    const int stack = batch_stack(ctx, b->max_depth);
    if (!stack) return set_error(ctx, MRT_ERANGE, "batch_trace: stack_depth below the batch's BVH depth");
    const bool any = (flags & MRT_TRACE_ANY_HIT) != 0u;
    const bool spread = ((ctx->tuning.tri_spread >> (any ? 1u : 0u)) & 1u) != 0u;
    const uint32_t rmin = ctx->tuning.refill_min ? ctx->tuning.refill_min : 1u;
#define MRT_BT(K, S, P)                                                                                   \
    k_batch_trace<K, S, P><<<blocks, kTraceBlock, dsm, s>>>(b->dev, b->d_roots, b->d_ray_off, b->scenes, rays, \
                                                            n, hits, ctx->d_prim_fetch, ctx->d_status, rmin)
#define MRT_BT2(K, S) \
    do { if (spread) MRT_BT(K, S, true); else MRT_BT(K, S, false); } while (0)
    if (stack == 16) { if (any) MRT_BT2(true, 16); else MRT_BT2(false, 16); }
    else if (stack == 32) { if (any) MRT_BT2(true, 32); else MRT_BT2(false, 32); }
    else { if (any) MRT_BT2(true, 24); else MRT_BT2(false, 24); }
#undef MRT_BT2
#undef MRT_BT
    if (cudaGetLastError() != cudaSuccess) return set_error(ctx, MRT_ECUDA, "batch_trace: launch failed");
    ctx->launches++;
    return MRT_OK;
}

int mrt_cuda_batch_pathtrace(mrt_ctx* ctx, mrt_batch* b, const mrt_ray* rays, const uint32_t* ray_offsets,
                             const mrt_trace_params* params, uint32_t frame, float* radiance, int use_graph,
                             void* stream) {
    if (!ctx || !b || !ray_offsets || !params) return set_error(ctx, MRT_EINVAL, "batch_pathtrace: null argument");
    if (params->max_bounces > MRT_MAX_BOUNCES) return set_error(ctx, MRT_ERANGE, "batch_pathtrace: max_bounces > 16");
    cudaSetDevice(ctx->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    uint32_t n = 0;
    int rc = upload_offsets(ctx, b, ray_offsets, n, s);
    if (rc) return rc;
    if (n == 0) return MRT_OK;
    if (!rays || !radiance) return set_error(ctx, MRT_EINVAL, "batch_pathtrace: null rays or radiance");
    if (b->cap < n) {
        free_batch_state(b);
        bool ok = cudaMalloc(&b->q[0], n * sizeof(PathRay)) == cudaSuccess &&
                  cudaMalloc(&b->q[1], n * sizeof(PathRay)) == cudaSuccess &&
                  cudaMalloc(&b->sq, n * sizeof(ShadowRay)) == cudaSuccess &&
                  cudaMalloc(&b->hits, n * sizeof(uint2)) == cudaSuccess &&
                  cudaMalloc(&b->rng, n * sizeof(uint32_t)) == cudaSuccess &&
                  cudaMalloc(&b->counters, kCntSlots * sizeof(uint32_t)) == cudaSuccess;
        if (!ok) {
            cudaGetLastError();
            free_batch_state(b);
            return set_error(ctx, MRT_ENOMEM, "batch_pathtrace: out of device memory for the path queues");
        }
        b->cap = n;
    }
    // per-call parameters go through device memory so a captured graph
    // replays with new values
    *b->h_tp = make_trace_params(params);
    *b->h_frame = frame;
    if (cudaMemcpyAsync(b->d_tp, b->h_tp, sizeof(TraceParams), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(b->d_frame, b->h_frame, sizeof(uint32_t), cudaMemcpyHostToDevice, s) != cudaSuccess)
        return set_error(ctx, MRT_ECUDA, "batch_pathtrace: parameter upload failed");

    const int blocks = persistent_blocks(ctx);
    const int stack = batch_stack(ctx, b->max_depth);
    if (!stack) return set_error(ctx, MRT_ERANGE, "batch_pathtrace: stack_depth below the batch's BVH depth");
    const uint32_t bounces = params->max_bounces;
    const bool spread = (ctx->tuning.tri_spread & 1u) != 0u;
    const uint32_t rmin = ctx->tuning.refill_min ? ctx->tuning.refill_min : 1u;
    const bool nee = params->estimator == MRT_EST_NEE;
    const int sblocks = int(std::min<size_t>((n + kShadeBlock - 1) / kShadeBlock, 8192));
    auto enqueue = [&](cudaStream_t st) -> bool {
        if (cudaMemsetAsync(b->counters, 0, kCntSlots * sizeof(uint32_t), st) != cudaSuccess) return false;
        k_batch_init<<<sblocks, kShadeBlock, (b->scenes + 1u) * sizeof(uint32_t), st>>>(
            rays, b->d_ray_off, b->scenes, n, b->q[0], b->rng, radiance, b->counters, b->d_frame);
        for (uint32_t v = 0; v <= bounces; ++v) {
#define MRT_BQ(S, P)                                                                                       \
    k_batch_trace_queue<S, P><<<blocks, kTraceBlock, 0, st>>>(b->dev, b->d_roots, b->q[v & 1u], b->hits, \
                                                              b->counters, v, ctx->d_status, rmin)
            if (stack == 16) { if (spread) MRT_BQ(16, true); else MRT_BQ(16, false); }
            else if (stack == 32) { if (spread) MRT_BQ(32, true); else MRT_BQ(32, false); }
            else { if (spread) MRT_BQ(24, true); else MRT_BQ(24, false); }
#undef MRT_BQ
            if (nee)
                k_batch_shade<true><<<sblocks, kShadeBlock, 0, st>>>(b->dev, b->d_tp, b->q[v & 1u],
                                                                     b->q[(v + 1u) & 1u], b->sq, b->hits, b->rng,
                                                                     radiance, b->counters, v, ctx->d_status);
            else
                k_batch_shade<false><<<sblocks, kShadeBlock, 0, st>>>(b->dev, b->d_tp, b->q[v & 1u],
                                                                      b->q[(v + 1u) & 1u], b->sq, b->hits, b->rng,
                                                                      radiance, b->counters, v, ctx->d_status);
            if (nee) {
#define MRT_BS(S)                                                                                          \
    k_batch_trace_shadow<S><<<blocks, kTraceBlock, 0, st>>>(b->dev, b->d_roots, b->d_tp, b->sq, radiance, \
                                                            b->counters, v, ctx->d_status, rmin)
                if (stack == 16) MRT_BS(16);
                else if (stack == 32) MRT_BS(32);
                else MRT_BS(24);
#undef MRT_BS
            }
        }
        k_batch_tally<<<1, 32, 0, st>>>(b->counters, ctx->d_totals, bounces);
        return cudaGetLastError() == cudaSuccess;
    };
    ctx->acc.primary_rays += n;
    if (!use_graph) {
        if (!enqueue(s)) return set_error(ctx, MRT_ECUDA, "batch_pathtrace: launch failed");
        ctx->launches += 2 + (nee ? 3 : 2) * (bounces + 1);
        return MRT_OK;
    }
    const bool same = b->exec && b->g_rays == rays && b->g_radiance == radiance && b->g_n == n &&
                      b->g_bounces == bounces && b->g_blocks == uint32_t(blocks) && b->g_stack == stack &&
                      b->g_spread == spread && b->g_refill == rmin && b->g_nee == nee;
    if (!same) {
        if (b->exec) cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
        if (!b->cap_stream && cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking) != cudaSuccess)
            return set_error(ctx, MRT_ECUDA, "batch_pathtrace: capture stream");
        cudaGraph_t g = nullptr;
        if (cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
            return set_error(ctx, MRT_ECUDA, "batch_pathtrace: begin capture failed");
        const bool ok = enqueue(b->cap_stream);
        cudaError_t e = cudaStreamEndCapture(b->cap_stream, &g);
        if (!ok || e != cudaSuccess || !g) {
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            return set_error(ctx, MRT_ECUDA, "batch_pathtrace: graph capture failed");
        }
        e = cudaGraphInstantiate(&b->exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            b->exec = nullptr;
            return set_error(ctx, MRT_ECUDA, "batch_pathtrace: graph instantiation failed");
        }
        b->g_rays = rays;
        b->g_radiance = radiance;
        b->g_n = n;
        b->g_bounces = bounces;
        b->g_blocks = uint32_t(blocks);
        b->g_stack = stack;
        b->g_spread = spread;
        b->g_refill = rmin;
        b->g_nee = nee;
    }
    if (cudaGraphLaunch(b->exec, s) != cudaSuccess) return set_error(ctx, MRT_ECUDA, "batch_pathtrace: graph launch");
    ctx->launches += 2 + (nee ? 3 : 2) * (bounces + 1);
    return MRT_OK;
}

} // extern "C"
