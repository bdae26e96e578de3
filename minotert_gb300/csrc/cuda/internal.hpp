// Private declarations shared by the C-ABI layer (api.cu) and the kernels.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "mrt_cuda.h"
#include "sky.cuh"
#include "traverse.cuh"

namespace mrt {

// Traversal stack entries per thread (shared memory) and the residency
// target of the traversal kernels: 24 entries x 8 B x 128 threads = 24 KB
// and <= 64 registers give 8 blocks (32 warps) per SM on GB300, the
// fastest schedule measured (6 blocks: +10% frame time, 5: +20%).
#ifndef MRT_TRACE_STACK
#define MRT_TRACE_STACK 24
#endif
#ifndef MRT_TRACE_MIN_BLOCKS
#define MRT_TRACE_MIN_BLOCKS 8
#endif
constexpr int kTraceBlock = 128;   // threads per traversal block
constexpr int kStackDepth = MRT_TRACE_STACK;
constexpr int kTraceMinBlocks = MRT_TRACE_MIN_BLOCKS;
constexpr int kShadeBlock = 256;
// The shading kernels wait on scattered loads (materials, RNG state, blue
// noise): 4 blocks per SM (<= 64 registers) keep more of them in flight.
constexpr int kShadeMinBlocks = 4;
constexpr uint32_t kSortNever = 0xFFFFFFFFu;  // mrt_tuning.sort_min_rays: never sort

// Wavefront records
struct PathRay {     // 48 bytes
    float4 o_pix;    // origin xyz, pixel index (bits)
    float4 d;        // direction xyz, unused
    float4 beta;     // throughput rgb, unused
};
struct ShadowRay {   // 32 bytes
    float4 o_pix;    // origin xyz, pixel index (bits)
    float4 contrib;  // radiance added when unoccluded
};

// Device counters (uint32 slots)
enum : uint32_t {
    kCntExt = 0,                       // [b]: rays in the extension queue of bounce b
    kCntShadow = kCntExt + 17,         // [b]: shadow rays emitted at vertex b
    kCntFetchExt = kCntShadow + 17,    // [b]: work fetch of extension trace b
    kCntFetchShadow = kCntFetchExt + 17,
    kCntSorted = kCntFetchShadow + 17,  // [b]: 1 when the queue of bounce b was sorted into qsort
    kCntSlots = kCntSorted + 17,
};

// Accumulated totals (uint64 slots): ray counts copied from the counters
// above (slots 0..33), then traversal work in counting mode.
enum : uint32_t {
    kTotNodesExt = 64,     // [b]
    kTotTrisExt = 82,      // [b]
    kTotNodesShadow = 100,
    kTotTrisShadow = 101,
    kTotNodesPrim = 102,
    kTotTrisPrim = 103,
    kTotSlots = 128,
};

struct WaveBuffers {
    size_t cap = 0;        // rays per queue
    size_t npix = 0;
    PathRay* q[2] = {nullptr, nullptr};
    uint2* hits = nullptr;
    ShadowRay* sq = nullptr;
    float4* L = nullptr;
    uint32_t* rng = nullptr;
    uint32_t* counters = nullptr;
    unsigned long long* totals = nullptr; // accumulated ray counts
    uint32_t* keys = nullptr;             // sort scratch
    uint32_t* perm = nullptr;
    PathRay* qsort = nullptr;
    uint32_t* hist = nullptr;
};

// The extension queue of bounce b as the trace and shade kernels read it.
__device__ __forceinline__ const PathRay* ext_queue(const WaveBuffers& wb, uint32_t bounce) {
    if (wb.counters[kCntSorted + bounce]) return wb.qsort;
    return (bounce & 1u) ? wb.q[1] : wb.q[0];
}

struct FrameParams {
    mrt_camera_consts c;
    float pv[16];       // projection * view
    float ppv[16];      // projection * prev_view
    uint32_t width, height;
    float pitch_x, pitch_y;
};

// Pinhole ray of pixel (x, y) (primaryRay.comp:46-51): uv at the pixel
// centre with v flipped, origin = invView * (0,0,0,1),
// dir = normalize(invView * vec4((invProj * vec4(2uv-1, 1, 1)).xyz, 0)).
MRT_DEV void primary_ray(const FrameParams& fp, uint32_t x, uint32_t y, f3& o, f3& d) {
    const float uvx = __fmul_rn(__fadd_rn(float(x), 0.5f), fp.pitch_x);
    const float uvy = __fsub_rn(1.0f, __fmul_rn(__fadd_rn(float(y), 0.5f), fp.pitch_y));
    float org[4], vd[4], wd[4];
    matvec_rn(fp.c.inv_view, 0.0f, 0.0f, 0.0f, 1.0f, org);
    matvec_rn(fp.c.inv_projection, __fsub_rn(__fmul_rn(uvx, 2.0f), 1.0f),
              __fsub_rn(__fmul_rn(uvy, 2.0f), 1.0f), 1.0f, 1.0f, vd);
    matvec_rn(fp.c.inv_view, vd[0], vd[1], vd[2], 0.0f, wd);
    o = f3{org[0], org[1], org[2]};
    d = normalize_rn(f3{wd[0], wd[1], wd[2]});
}

MRT_DEV f3 ray_at(f3 o, f3 d, float t) { return add_rn(o, scale_rn(d, t)); } // intersect.glsl:22-24

struct TraceParams {
    uint32_t samples, max_bounces, rr_start, rng_mode, estimator;
    uint32_t exact_trig;  // mrt_trace_params.exact_trig
    float sun[3], sun_e[3], sky[3];
    SkyDev atmo;  // atmosphere miss shader; atmo.view == nullptr: constant sky
};

// Radiance of a path escaping in direction d: the bound sky, else the
// constant sky radiance.
MRT_DEV f3 escape_radiance(const TraceParams& tp, f3 d) {
    if (tp.atmo.view) return sky_color(tp.atmo, d);
    return f3{tp.sky[0], tp.sky[1], tp.sky[2]};
}

// Miss-shader state of a bound sky (sky.cu)
SkyDev sky_dev(const mrt_sky* s, const float cam[3]);

struct BlueNoise {
    const float2* rot;
    uint32_t w, h;
};

// Launchers (kernels.cu).  All return cudaError_t of the launch.
// Depth of a BVH8 (levels along in-range child links, each node counted
// once); the traversal stack holds at most depth - 1 entries.
uint32_t bvh8_depth(const mrt_bvh8_node* nodes, uint32_t n);

// fetch != nullptr selects the persistent dynamic-fetch kernel (`blocks`
// blocks); otherwise one thread per pixel, with the triangle tests spread
// over each warp when `spread` is set (not while counting).
cudaError_t launch_primary_tri(const DevScene& sc, const FrameParams& fp, const mrt_gbuffer& g,
                               uint32_t* status, unsigned long long* totals, uint32_t* fetch, int blocks,
                               bool spread, uint32_t refill_min, cudaStream_t s);
cudaError_t launch_primary_sphere(const DevScene& sc, const FrameParams& fp, const mrt_gbuffer& g,
                                  cudaStream_t s);
cudaError_t launch_secondary_sphere(const DevScene& sc, const FrameParams& fp, const mrt_gbuffer& g,
                                    const TraceParams& tp, BlueNoise bn, float* color,
                                    uint32_t accumulate, uint32_t frame_index, cudaStream_t s);
cudaError_t launch_trace_rays(const DevScene& sc, const mrt_ray* rays, uint32_t n, mrt_hit* hits,
                              bool any_hit, uint32_t* nodes_v, uint32_t* tris_v, uint32_t* status,
                              cudaStream_t s);

// wavefront pieces
cudaError_t launch_shade_primary(const DevScene& sc, const FrameParams& fp, const mrt_gbuffer& g,
                                 const TraceParams& tp, BlueNoise bn, const WaveBuffers& wb,
                                 uint32_t sample, uint32_t* status, cudaStream_t s);
// Work schedule of the persistent trace kernels: each warp fetches 32 rays
// and runs them to completion (batch); idle lanes refill after every step
// (dynamic); each of the two with the step's triangle tests spread over the
// warp (trav_step_spread).
enum : int { kFetchBatch = 0, kFetchDynamic = 1, kFetchSpread = 2, kFetchBatchSpread = 3 };
// refill_min (dynamic fetch): idle lanes a warp waits for before it fetches
// new rays (1: refill whenever a lane is idle)
cudaError_t launch_trace_ext(const DevScene& sc, const WaveBuffers& wb, uint32_t bounce, int blocks,
                             uint32_t* status, bool count, int mode, uint32_t refill_min, cudaStream_t s);
cudaError_t launch_trace_shadow(const DevScene& sc, const WaveBuffers& wb, const TraceParams& tp,
                                uint32_t vertex, int blocks, uint32_t* status, bool count, int mode,
                                uint32_t refill_min, cudaStream_t s);
cudaError_t launch_trace_merged(const DevScene& sc, const WaveBuffers& wb, const TraceParams& tp, uint32_t bounce,
                                int blocks, uint32_t* status, uint32_t refill_min, cudaStream_t s);
cudaError_t launch_shade(const DevScene& sc, const TraceParams& tp, BlueNoise bn, const WaveBuffers& wb,
                         uint32_t width, uint32_t bounce, uint32_t* status, cudaStream_t s);
// every path of the bounce-`first` extension queue to its end (k_tail);
// from_hits: that queue's hits are already in wb.hits (traced by k_trace_ext)
cudaError_t launch_tail(const DevScene& sc, const TraceParams& tp, BlueNoise bn, const WaveBuffers& wb,
                        uint32_t width, uint32_t first, bool from_hits, bool spread, int blocks, uint32_t* status,
                        cudaStream_t s);
cudaError_t launch_tally(const WaveBuffers& wb, cudaStream_t s);
cudaError_t launch_sort_ext(const DevScene& sc, const WaveBuffers& wb, uint32_t bounce, uint32_t min_rays,
                            cudaStream_t s);
cudaError_t launch_finalize(const WaveBuffers& wb, float* color, uint32_t samples, uint32_t accumulate,
                            uint32_t frame_index, cudaStream_t s);

// learned radiance cache (kernels.cu)
cudaError_t launch_cache_train_paths(const DevScene& sc, const FrameParams& fp, const TraceParams& tp,
                                     uint32_t bounces, uint32_t n_paths, uint32_t frame, float* q, float* t,
                                     uint32_t* count, uint32_t cap, uint32_t* status, cudaStream_t s);
cudaError_t launch_cache_query(const DevScene& sc, const TraceParams& tp, const WaveBuffers& wb, float* q,
                               float4* pb, uint32_t* status, cudaStream_t s);
cudaError_t launch_cache_query_primary(const DevScene& sc, const FrameParams& fp, const mrt_gbuffer& g, float* q,
                                       float4* pb, uint32_t* status, cudaStream_t s);
cudaError_t launch_cache_apply(const WaveBuffers& wb, const uint32_t* n_dev, uint32_t n_max, const float* pred,
                               const float4* pb, cudaStream_t s);
uint32_t cache_query_vertex(const mrt_cache* c);  // nrc.cu
bool cache_overlap_training(const mrt_cache* c);  // nrc.cu

int trace_blocks_per_sm();  // occupancy of the traversal kernels

} // namespace mrt

struct mrt_scene {
    int kind = 0; // 0 triangles, 1 spheres
    mrt::DevScene dev{};
    void* d_nodes = nullptr;
    void* d_tris = nullptr;
    void* d_mats = nullptr;
    void* d_spheres = nullptr;
};

struct mrt_timing_rec {
    int kind;      // 0 primary, 1 extend, 2 shadow, 3 shade, 4 sort, 5 total
    int bounce;
    cudaEvent_t a, b;
};

struct mrt_ctx {
    int device = 0;
    int sm_count = 0;
    std::string err;
    uint32_t* d_status = nullptr;
    float2* d_bn = nullptr;
    uint32_t bn_w = 0, bn_h = 0;
    mrt::WaveBuffers wb;
    // render_frame_host buffers
    uint32_t* d_vis = nullptr;
    void* d_aux = nullptr;   // normal (8 B/px) then depth (2 B/px)
    float* d_t = nullptr;
    float* d_color = nullptr;
    size_t frame_pixels = 0;
    // render_frame_host_async: two colour buffers in flight, read back on a
    // copy stream; ev_rendered[b] / ev_copied[b]: buffer b's frame is
    // rendered / read back
    float* d_color_async[2] = {nullptr, nullptr};
    size_t async_pixels = 0;
    uint32_t async_next = 0;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_rendered[2] = {nullptr, nullptr}, ev_copied[2] = {nullptr, nullptr};
    // timing
    bool timing = false;
    bool counters = false;
    mrt_tuning tuning{0u, 3u, 0u, mrt::kSortNever, 3u, 0u, 11u, 8u, 1u, 1u};  // autotuned on GB300 (icosphere field, 1080p)
    uint32_t* d_prim_fetch = nullptr;  // work counter of the persistent primary kernel
    int occ_blocks = 0;                // traversal blocks per SM at full occupancy
    unsigned long long* d_totals = nullptr;  // kTotSlots accumulated totals
    std::vector<mrt_timing_rec> recs;
    std::vector<cudaEvent_t> ev_pool;
    mrt_frame_stats acc{};
    uint32_t launches = 0;
    const mrt_sky* sky = nullptr;  // miss shader bound by mrt_cuda_set_sky
    // second stream for the shadow rays that overlap the next extension
    // trace (mrt_tuning.overlap_shadow), with its fork / join events
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
};
