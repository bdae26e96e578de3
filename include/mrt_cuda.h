/*
 * mrt_cuda.h -- the C ABI of the GB300 (sm_103a) ray-tracing device layer.
 *
 * This replaces the Vulkan device layer of MinoteRT (src/sys/vulkan.ixx plus
 * the vuk render graph) on the ray-tracing hot path.  The renderer keeps the
 * pass structure of src/gfx/modules/pathtracer.ixx:
 *
 *   Pathtracer::primaryRays   (pathtracer.ixx:29-116)  -> mrt_cuda_primary_rays
 *   Pathtracer::secondaryRays (pathtracer.ixx:118-195) -> mrt_cuda_secondary_rays
 *
 * and the device work those passes dispatched (src/gpu/primaryRay.comp,
 * src/gpu/secondaryRays.comp) runs as hand-written CUDA kernels.
 *
 * Conventions
 *   - Every entry point returns MRT_OK (0) or a negative MRT_E* code; nothing
 *     throws across the ABI.  mrt_cuda_last_error() gives a message.
 *   - Device pointers are plain pointers obtained from mrt_cuda_alloc (or any
 *     other CUDA allocation on the context's device).  Streams are passed as
 *     `void*` holding a cudaStream_t (NULL = the legacy default stream).
 *   - All work is stream-ordered; only mrt_cuda_sync / mrt_cuda_status /
 *     the *_host entry points synchronise.
 *   - A context is used from one host thread at a time; many contexts may
 *     coexist.
 *   - Matrices are column-major float[16] (GLSL / minote.math layout,
 *     src/stx/math.ixx): m[col*4 + row].
 */
#ifndef MRT_CUDA_H
#define MRT_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MRT_ABI_VERSION 1

/* ---- return codes ------------------------------------------------------ */
enum {
    MRT_OK       = 0,
    MRT_EINVAL   = -1, /* bad argument (null pointer, size, enum)            */
    MRT_ECUDA    = -2, /* a CUDA runtime call failed                          */
    MRT_ENOMEM   = -3, /* device or host allocation failed                   */
    MRT_ETIMEOUT = -4, /* mrt_cuda_sync wall-clock limit expired             */
    MRT_EDEVICE  = -5, /* a kernel raised a device status flag (see below)   */
    MRT_ESTATE   = -6, /* call made in the wrong state (e.g. no blue noise)  */
    MRT_ERANGE   = -7  /* size beyond a documented maximum                   */
};

/* ---- device status flags (mrt_cuda_status) ----------------------------- */
#define MRT_STATUS_ITER_CAP  0x01u /* a traversal hit its iteration cap      */
#define MRT_STATUS_STACK_OVF 0x02u /* traversal stack overflow               */
#define MRT_STATUS_BAD_NODE  0x04u /* child node index out of range          */
#define MRT_STATUS_BAD_TRI   0x08u /* triangle index out of range            */
#define MRT_STATUS_QUEUE_OVF 0x10u /* a wavefront queue overflowed           */
#define MRT_STATUS_BAD_SCENE 0x20u /* batched launch: scene index invalid    */
#define MRT_STATUS_PIPE_TIMEOUT 0x40u /* a tensor-core pipeline wait ran out */

/* ---- scene data formats ------------------------------------------------ */

/* One node of the compressed 8-wide BVH (quantised child boxes), 128 bytes,
 * 128-byte aligned so a node is exactly one L2 line; the first 80 bytes are
 * read by traversal.  Child slot i covers the box
 *     lo = origin + q_lo[i] * 2^exp,  hi = origin + q_hi[i] * 2^exp
 * per axis.  meta[i] == 0: empty slot.  imask bit i: slot i is an internal
 * node; its index is child_base + popcount(imask & ((1<<i)-1)).  Otherwise
 * slot i is a leaf: meta[i] >> 5 is a unary triangle count (1, 3 or 7 for
 * 1..3 triangles) and meta[i] & 31 the first triangle's offset from
 * tri_base.  Internal slots carry meta = 0x20 | (24 + i).
 * The reference has no BVH (it loops over 5 spheres, primaryRay.comp:26-32);
 * this format is new. */
typedef struct mrt_bvh8_node {
    float    origin[3];
    int8_t   exp[3];
    uint8_t  imask;
    uint32_t child_base;
    uint32_t tri_base;
    uint8_t  meta[8];
    uint8_t  q_lo_x[8], q_lo_y[8], q_lo_z[8];
    uint8_t  q_hi_x[8], q_hi_y[8], q_hi_z[8];
    uint32_t reserved[12];
} mrt_bvh8_node;

/* A triangle in BVH leaf order, 48 bytes: three vertices, each padded to
 * 16 bytes; `id` is the triangle's index in the caller's original mesh. */
typedef struct mrt_tri {
    float v0[3]; uint32_t id;
    float v1[3]; uint32_t pad1;
    float v2[3]; uint32_t pad2;
} mrt_tri;

/* Per-original-triangle shading record, 16 bytes: unit geometric normal
 * (winding v0,v1,v2) and albedo as RGBA8 UNORM (albedo = byte / 255). */
typedef struct mrt_material {
    float    normal[3];
    uint32_t albedo_rgba8;
} mrt_material;

/* Analytic sphere, the primitive of the reference's scene
 * (intersect.glsl:9-13, scene.glsl:4-11). */
typedef struct mrt_sphere {
    float center[3];
    float radius;
    float albedo[3];
    float pad;
} mrt_sphere;

/* Generic ray, 32 bytes: a hit is accepted for tmin < t < tmax. */
typedef struct mrt_ray {
    float org[3]; float tmin;
    float dir[3]; float tmax;
} mrt_ray;

/* Closest/any hit, 8 bytes.  prim = original triangle id (or sphere index),
 * 0xFFFFFFFF on a miss.  Ties at equal t resolve to the lower prim id. */
typedef struct mrt_hit {
    uint32_t prim;
    float    t;
} mrt_hit;

#define MRT_MISS 0xFFFFFFFFu

/* Per-dispatch camera constants: the union of the two reference UBOs
 * (primaryRay.comp:14-21 and secondaryRays.comp:25-32).  Host fill as in
 * pathtracer.ixx:86-105 / 171-184. */
typedef struct mrt_camera_consts {
    float    view[16];
    float    projection[16];
    float    inv_view[16];
    float    inv_projection[16];
    float    prev_view[16];
    float    camera_pos[3];
    uint32_t frame_counter;
} mrt_camera_consts;

/* The g-buffer of Pathtracer::GBuffer (pathtracer.ixx:22-27).  Device
 * pointers to width*height texels, row-major, row 0 = top of the image
 * (the shader's gl_GlobalInvocationID.y = 0).  Formats follow the reference
 * (pathtracer.ixx:42-69): visibility R32_UINT, depth R16F (NDC z of the
 * inverted infinite projection), normal RGBA16F (w = 0), motion RG16F.
 * hit_t (FP32 closest-hit distance) is new; the triangle path reads it
 * instead of reconstructing the hit from FP16 depth.  Any pointer but
 * visibility may be NULL to skip that output. */
typedef struct mrt_gbuffer {
    uint32_t* visibility;
    float*    hit_t;
    uint16_t* depth;
    uint16_t* normal;
    uint16_t* motion;
    uint32_t  width;
    uint32_t  height;
} mrt_gbuffer;

/* RNG modes */
#define MRT_RNG_REFERENCE 0u /* seed=(frame<<1)|1 for every pixel, decorrelated
                                only by the blue-noise Cranley-Patterson
                                rotation (secondaryRays.comp:124-125)        */
#define MRT_RNG_PER_PIXEL 1u /* seed also hashed with the pixel index        */

/* Estimators */
#define MRT_EST_ESCAPE 0u /* reference: light only from the sky on escape,
                             zero if the path runs out of bounces
                             (secondaryRays.comp:64-100)                     */
#define MRT_EST_NEE    1u /* plus one shadow ray per vertex toward a
                             directional light (new; no reference code)     */

typedef struct mrt_trace_params {
    uint32_t samples;      /* paths per pixel in this call (reference: 8)   */
    uint32_t max_bounces;  /* diffuse bounces after the primary hit
                              (reference: 8)                                 */
    uint32_t rr_start;     /* Russian roulette for bounces > rr_start;
                              0 = off                                        */
    uint32_t rng_mode;     /* MRT_RNG_*                                      */
    uint32_t estimator;    /* MRT_EST_*                                      */
    uint32_t accumulate;   /* 0: write this call's mean; 1: fold it into the
                              running mean with weight 1/(frame_index+1)
                              (frame_index 0 overwrites: the buffer's old
                              contents are never read)                       */
    uint32_t frame_index;  /* frames already in the running mean             */
    uint32_t sort_rays;    /* 1: sort extension rays between bounces         */
    float    sun_dir[3];   /* unit vector toward the directional light       */
    uint32_t exact_trig;   /* 1: the sphere-point sampler's sine and cosine
                              (random.glsl:10-19) are evaluated in binary64
                              and rounded once to binary32, as the CPU
                              oracle does, so path-traced colour matches it
                              bit for bit (up to a binary64 result lying
                              within a few binary64 ulps of a binary32
                              rounding boundary, about 1e-8 of calls);
                              0: CUDA sincosf (default, faster)             */
    float    sun_irradiance[3];
    float    pad1;
    float    sky_radiance[3]; /* constant radiance of escaping rays          */
    float    pad2;
} mrt_trace_params;

/* Per-frame statistics of the last mrt_cuda_secondary_rays call, filled when
 * timing is enabled (mrt_cuda_set_timing). */
#define MRT_MAX_BOUNCES 16
typedef struct mrt_frame_stats {
    uint64_t primary_rays;
    uint64_t extension_rays[MRT_MAX_BOUNCES]; /* rays traced at bounce b+1   */
    uint64_t shadow_rays;
    /* traversal work, filled when counters are enabled
     * (mrt_cuda_set_counters): BVH8 nodes and triangles visited */
    uint64_t nodes_primary, tris_primary;
    uint64_t nodes_extension[MRT_MAX_BOUNCES], tris_extension[MRT_MAX_BOUNCES];
    uint64_t nodes_shadow, tris_shadow;
    float    ms_primary;     /* primary closest-hit kernel                   */
    float    ms_extend;      /* all extension (closest-hit) kernels          */
    float    ms_extend_b[MRT_MAX_BOUNCES];
    float    ms_shadow;      /* all shadow (any-hit) kernels                 */
    float    ms_shade;       /* shade + ray generation kernels               */
    float    ms_sort;        /* ray sort kernels                             */
    float    ms_total;       /* whole secondary pass                         */
    float    ms_cache_train; /* radiance cache: training paths + steps       */
    float    ms_cache_infer; /* radiance cache: queries                      */
    uint32_t launches;       /* kernels launched by the pass                 */
    uint32_t pad;
} mrt_frame_stats;

typedef struct mrt_ctx   mrt_ctx;
typedef struct mrt_scene mrt_scene;

/* ---- context ----------------------------------------------------------- */
/* Replaces the Vulkan service (src/sys/vulkan.ixx:426, Vulkan_impl ctor
 * :106-115): selects `device` and creates the per-context device state.
 * A context (with its scenes, caches and denoisers) is used by one host
 * thread at a time: its work buffers, second stream and fork / join events
 * are shared by the passes it runs. */
int         mrt_cuda_create(mrt_ctx** out, int device);
int         mrt_cuda_destroy(mrt_ctx* ctx);
const char* mrt_cuda_last_error(const mrt_ctx* ctx);
int         mrt_cuda_abi_version(void);
/* Reads (and with clear != 0 resets) the device status word; synchronises
 * the context.  Returns MRT_OK; *flags holds MRT_STATUS_* bits. */
int mrt_cuda_status(mrt_ctx* ctx, uint32_t* flags, int clear);
/* Waits for `stream` with a wall-clock limit (polling cudaStreamQuery);
 * MRT_ETIMEOUT when it expires.  timeout_s <= 0: no limit. */
int mrt_cuda_sync(mrt_ctx* ctx, void* stream, double timeout_s);
/* Enables per-kernel CUDA-event timing into mrt_frame_stats. */
int mrt_cuda_set_timing(mrt_ctx* ctx, int enable);
/* Runs the traversal kernels in their counting form (nodes / triangles
 * visited per ray, summed into mrt_frame_stats).  Slower; for profiling. */
int mrt_cuda_set_counters(mrt_ctx* ctx, int enable);
/* Returns the statistics accumulated since the previous call and resets
 * them; synchronises the context. */
int mrt_cuda_frame_stats(mrt_ctx* ctx, mrt_frame_stats* out);

/* Launch-schedule knobs of the traversal kernels (new; the reference
 * dispatches fixed 8x8 groups, pathtracer.ixx:106,190).  Picked by the
 * autotuner; defaults are the tuned values for GB300. */
typedef struct mrt_tuning {
    uint32_t trace_blocks_per_sm; /* persistent blocks per SM; 0 = occupancy max */
    uint32_t dynamic_fetch;       /* bit 0: extension rays, bit 1: shadow rays
                                     refill idle lanes after every node step
                                     (clear: each warp fetches 32 rays and
                                     runs them to completion)                */
    uint32_t primary_persistent;  /* 1: primary rays through the persistent
                                     dynamic-fetch kernel (0: one thread per
                                     pixel, 8x4-pixel warps)                 */
    uint32_t sort_min_rays;       /* sort extension queues holding at least
                                     this many rays (direction octant + origin
                                     Morton key); 0xFFFFFFFF = never.  A call
                                     with mrt_trace_params.sort_rays = 1 sorts
                                     every queue                             */
    uint32_t tail_bounce;         /* 0: every bounce as separate wavefront
                                     passes; b >= 1: the paths still alive
                                     at bounce b finish in one persistent
                                     launch (trace, shade, shadow ray and
                                     the later bounces per lane; same image) */
    uint32_t stack_depth;         /* traversal stack entries of the batched
                                     kernels (mrt_cuda_batch_*): 16, 24 or
                                     32; 0 = 24.  Must cover the batch's
                                     deepest BVH (depth - 1 entries)         */
    uint32_t tri_spread;          /* bit 0: extension rays, bit 1: shadow rays
                                     (with dynamic_fetch set for them), bit 2:
                                     primary rays (one thread per pixel), bit
                                     3: the path tail: the triangle tests of
                                     a traversal step are spread over the
                                     warp's lanes instead of each lane
                                     testing its own leaves' (same hits)     */
    uint32_t refill_min;          /* kernels with dynamic fetch (and the
                                     batched ones): a warp fetches new rays
                                     once at least this many of its lanes
                                     are idle (or all are); 0 or 1 =
                                     whenever one is (up to 32)              */
    uint32_t overlap_shadow;      /* 1: the shadow rays of vertex b - 1 and
                                     the extension rays of bounce b trace on
                                     two streams at once (a stream of the
                                     context joined before shading; same
                                     image); 2: both queues in one
                                     persistent launch (warps refill from
                                     the extension queue, then the shadow
                                     queue; same image)                      */
    uint32_t tail_from_hits;      /* 1: bounce tail_bounce is traced by the
                                     wavefront kernel and the path tail
                                     starts from its hits (shading that
                                     bounce, its shadow rays and the rest)   */
} mrt_tuning;
int mrt_cuda_set_tuning(mrt_ctx* ctx, const mrt_tuning* tuning);
int mrt_cuda_get_tuning(mrt_ctx* ctx, mrt_tuning* tuning);

typedef struct mrt_device_info {
    char     name[96];
    int32_t  sm_count;
    int32_t  cc_major, cc_minor;
    uint32_t trace_blocks_per_sm_max; /* occupancy limit of the traversal kernels */
    uint64_t total_mem;
    uint64_t l2_bytes;
} mrt_device_info;
int mrt_cuda_device_info(mrt_ctx* ctx, mrt_device_info* out);

/* Read-bandwidth sweep (new; a measurement aid with no counterpart in the
 * reference): `passes` sweeps of 16-byte loads that bypass L1 over `bytes`
 * of the device buffer `buf` (16-byte aligned), by min(sink_words, 8 x SMs)
 * blocks, each XOR-folding what it read into sink[block].  On a buffer that
 * fits in L2, time it with events to get the L2 read bandwidth that bounds
 * the traversal kernels, whose scene stays L2-resident. */
int mrt_cuda_read_sweep(mrt_ctx* ctx, const void* buf, size_t bytes, uint32_t passes,
                        uint32_t* sink, uint32_t sink_words, void* stream);

/* ---- memory and streams (the reference's vuk allocator role,
 *      renderer.ixx:42-43) --------------------------------------------- */
int mrt_cuda_alloc(mrt_ctx* ctx, size_t bytes, void** dptr);
int mrt_cuda_free(mrt_ctx* ctx, void* dptr);
int mrt_cuda_host_alloc(mrt_ctx* ctx, size_t bytes, void** hptr); /* pinned */
int mrt_cuda_host_free(mrt_ctx* ctx, void* hptr);
int mrt_cuda_copy_h2d(mrt_ctx* ctx, void* dst, const void* src, size_t bytes, void* stream);
int mrt_cuda_copy_d2h(mrt_ctx* ctx, void* dst, const void* src, size_t bytes, void* stream);
int mrt_cuda_copy_d2d(mrt_ctx* ctx, void* dst, const void* src, size_t bytes, void* stream);
int mrt_cuda_memset(mrt_ctx* ctx, void* dst, int value, size_t bytes, void* stream);
int mrt_cuda_stream_create(mrt_ctx* ctx, void** stream);
int mrt_cuda_stream_destroy(mrt_ctx* ctx, void* stream);
int mrt_cuda_event_create(mrt_ctx* ctx, void** event);
int mrt_cuda_event_destroy(mrt_ctx* ctx, void* event);
int mrt_cuda_event_record(mrt_ctx* ctx, void* event, void* stream);
int mrt_cuda_event_elapsed(mrt_ctx* ctx, void* start, void* stop, float* ms);

/* ---- scenes ------------------------------------------------------------ */
/* Uploads a host-built BVH8 (see mrt_host.h, mrt_bvh8_build) with its
 * leaf-ordered triangles and per-original-triangle materials; the library
 * owns the device copy.  Replaces the reference's compile-time scene
 * constant (scene.glsl:4-11). */
int mrt_cuda_scene_upload_triangles(mrt_ctx* ctx,
                                    const mrt_bvh8_node* nodes, uint32_t node_count,
                                    const mrt_tri* tris, uint32_t tri_count,
                                    const mrt_material* materials, uint32_t material_count,
                                    mrt_scene** out);
/* Uploads an analytic sphere list (the reference's own scene 0 form). */
int mrt_cuda_scene_upload_spheres(mrt_ctx* ctx, const mrt_sphere* spheres,
                                  uint32_t count, mrt_scene** out);
int mrt_cuda_scene_destroy(mrt_ctx* ctx, mrt_scene* scene);

/* Blue-noise texture upload (renderer.ixx:101-110 decodes an RGBA8 PNG and
 * creates an R8G8B8A8_UNORM texture).  Channels R,G become the per-pixel
 * Cranley-Patterson rotation, fetched at (x % w, y % h)
 * (secondaryRays.comp:125).  w, h <= 1024. */
int mrt_cuda_blue_noise_upload(mrt_ctx* ctx, const uint8_t* rgba, uint32_t w, uint32_t h);

/* ---- passes ------------------------------------------------------------ */
/* Primary rays: one pinhole ray per pixel from inv_view/inv_projection
 * (primaryRay.comp:46-51), closest hit, g-buffer stores (primaryRay.comp:
 * 60-75).  Replaces Pathtracer::primaryRays (pathtracer.ixx:29-116). */
int mrt_cuda_primary_rays(mrt_ctx* ctx, const mrt_scene* scene,
                          const mrt_camera_consts* consts,
                          const mrt_gbuffer* gbuffer, void* stream);

/* Secondary rays: per pixel, `samples` paths of up to `max_bounces`
 * cosine-weighted diffuse bounces from the primary hit in the g-buffer,
 * throughput times albedo, sky (and for MRT_EST_NEE the directional light)
 * as light, mean written or accumulated to `color` (device, float RGB,
 * width*height*3).  Replaces Pathtracer::secondaryRays
 * (pathtracer.ixx:118-195) and secondaryRays.comp:102-135.  Triangle scenes
 * run as a wavefront (extend / shade / shadow kernels with compaction
 * between bounces); sphere scenes run the reference's per-pixel loop. */
int mrt_cuda_secondary_rays(mrt_ctx* ctx, const mrt_scene* scene,
                            const mrt_gbuffer* gbuffer,
                            const mrt_camera_consts* consts,
                            const mrt_trace_params* params,
                            float* color, void* stream);

/* Generic closest-hit (flags = 0) or any-hit (MRT_TRACE_ANY_HIT) query for
 * `count` rays in device memory; hits written to device memory. */
#define MRT_TRACE_ANY_HIT 0x1u
int mrt_cuda_trace_rays(mrt_ctx* ctx, const mrt_scene* scene,
                        const mrt_ray* rays, uint32_t count, mrt_hit* hits,
                        uint32_t flags, void* stream);

/* Per-ray traversal counters for the roofline (nodes and triangles visited,
 * closest-hit): device arrays of `count` uint32 each. */
int mrt_cuda_trace_rays_counted(mrt_ctx* ctx, const mrt_scene* scene,
                                const mrt_ray* rays, uint32_t count, mrt_hit* hits,
                                uint32_t* nodes_visited, uint32_t* tris_visited,
                                void* stream);

/* ---- batched scenes (new: the reference renders one scene) ----------- */
/* Concatenates `count` BVH8 scenes into one device BVH: child and triangle
 * indices are rebased and triangle ids are offset by the triangle counts of
 * the preceding scenes, so hits report batch-wide ids (scene s's local id =
 * prim - sum of tri_counts[0..s-1]).  Rays of any scene then trace in one
 * persistent launch, each starting at its own scene's root node. */
typedef struct mrt_batch mrt_batch;
int mrt_cuda_batch_create(mrt_ctx* ctx, uint32_t scene_count,
                          const mrt_bvh8_node* const* nodes, const uint32_t* node_counts,
                          const mrt_tri* const* tris, const uint32_t* tri_counts,
                          const mrt_material* const* materials, mrt_batch** out);
int mrt_cuda_batch_destroy(mrt_ctx* ctx, mrt_batch* batch);
/* Closest hit (flags = 0) or any hit of `rays` (device), grouped by scene:
 * scene s owns rays [ray_offsets[s], ray_offsets[s+1]) (host array of
 * scene_count + 1 entries). */
int mrt_cuda_batch_trace(mrt_ctx* ctx, mrt_batch* batch, const mrt_ray* rays,
                         const uint32_t* ray_offsets, mrt_hit* hits, uint32_t flags,
                         void* stream);
/* Closest-hit Lambertian path trace of the given primary rays over
 * params->max_bounces diffuse bounces: throughput x albedo, sky radiance on
 * escape and, with params->estimator = MRT_EST_NEE, a shadow ray toward the
 * directional light at every vertex (the single-scene tracer's estimator),
 * a per-ray PCG stream seeded by (ray index, frame), compaction of live
 * paths after every bounce.  radiance: device float RGB per ray.
 * use_graph != 0: the first call captures the whole bounce loop into a
 * CUDA graph (kept in the batch for these buffers and sizes) and later
 * calls replay it with one launch; make that first call outside any
 * caller's stream capture. */
int mrt_cuda_batch_pathtrace(mrt_ctx* ctx, mrt_batch* batch, const mrt_ray* rays,
                             const uint32_t* ray_offsets, const mrt_trace_params* params,
                             uint32_t frame, float* radiance, int use_graph, void* stream);
/* Running sums over copies of the same rays: acc[g][i] += scale *
 * sum_c x[g][c][i] for g < groups, c < copies, i < count floats (device
 * pointers, 16-byte aligned, count a multiple of 4).  With the rays of a
 * batched path trace laid out [scene][copy][pixel] and scale = 1 / (copies x
 * calls) this accumulates per-pixel sample means. */
int mrt_cuda_accumulate_copies(mrt_ctx* ctx, float* acc, const float* x, uint32_t groups,
                               uint32_t copies, size_t count, float scale, void* stream);

/* ---- learned radiance cache (new: the reference has no learned part) -- */
/* A multiresolution hash grid over position (16 levels x 2 FP16 features,
 * 2^log2_table entries per level, resolutions base_res .. max_res per unit
 * of the scene box) plus normal and direction, into an MLP of 4 hidden
 * layers of width 64 (ReLU, no biases, FP16 weights, FP32 accumulation on
 * the tensor cores) predicting outgoing RGB radiance.  Trained online with
 * Adam on the relative L2 loss against path-traced suffix radiance. */
typedef struct mrt_cache_config {
    uint32_t log2_table;    /* 19                                          */
    float    base_res;      /* 16                                          */
    float    max_res;       /* 2048                                        */
    float    lr_grid;       /* Adam learning rate of the grid features     */
    float    lr_mlp;        /* Adam learning rate of the MLP weights       */
    uint32_t seed;
    uint32_t train_paths;   /* training paths per frame (65536)            */
    uint32_t train_steps;   /* optimiser steps per frame (4)               */
    uint32_t train_bounces; /* bounce limit of the training paths (8)      */
    uint32_t query_vertex;  /* where paths end in the cache: 1 = at the hit
                               of the first diffuse bounce (default), 0 = at
                               the primary hit.  The cache learns indirect
                               outgoing radiance; every vertex's direct
                               light comes from its shadow ray            */
} mrt_cache_config;
typedef struct mrt_cache mrt_cache;
int mrt_cuda_cache_create(mrt_ctx* ctx, const mrt_cache_config* cfg, mrt_cache** out);
int mrt_cuda_cache_destroy(mrt_ctx* ctx, mrt_cache* cache);
/* Scene box the positions are normalised by (queries use [0,1]^3). */
int mrt_cuda_cache_set_bounds(mrt_ctx* ctx, mrt_cache* cache, const float lo[3], const float hi[3]);
/* Queries: device rows of 9 floats (position in [0,1]^3, unit normal,
 * unit outgoing direction); out: device rows of 3 floats.  Inference runs
 * on tcgen05 (128-query tiles, FP32 accumulators in tensor memory); a
 * tensor-core wait that runs out sets MRT_STATUS_PIPE_TIMEOUT. */
int mrt_cuda_cache_infer(mrt_ctx* ctx, mrt_cache* cache, const float* queries, uint32_t n,
                         float* out, void* stream);
/* enable = 0: inference and training on mma.sync instead (the earlier
 * kernels, kept for comparison); 1 (default): tcgen05 (training: the
 * forward writes each 128-row tile's activations, the backward accumulates
 * the weight gradients of its tiles in tensor memory and scatters the hash
 * grid's gradients from its last epilogue). */
int mrt_cuda_cache_set_tcgen05(mrt_cache* cache, int enable);
/* enable = 1 (default): mrt_cuda_cache_frame trains on the context's
 * second stream while the frame's rays are traced, joined before the cache
 * is queried (same image); 0: training first, on the caller's stream. */
int mrt_cuda_cache_set_overlap(mrt_cache* cache, int enable);
/* One training step on n device samples (queries + 3-float targets; n is
 * rounded down to a multiple of 16): forward, loss, backward; with
 * apply_update an Adam step (gradients are cleared), otherwise gradients
 * accumulate.  loss_out (host, may be NULL) receives the mean loss and
 * synchronises the stream. */
int mrt_cuda_cache_train_step(mrt_ctx* ctx, mrt_cache* cache, const float* queries,
                              const float* targets, uint32_t n, int apply_update,
                              float* loss_out, void* stream);
/* Host copies of parameters and gradients: which = 0 MLP weights (17408
 * FP32: 4 layers of 64x64 [out][in], then 16x64 output rows), 1 their
 * gradients, 2 grid features (16 * 2^log2_table * 2 FP32), 3 their
 * gradients.  set != 0 writes host -> device (and refreshes FP16 copies;
 * setting the grid gradients also marks their nonzero entries for the
 * grid's next Adam step, which updates only entries with a gradient). */
int mrt_cuda_cache_params(mrt_ctx* ctx, mrt_cache* cache, int which, float* host,
                          size_t count, int set);
/* One frame of cache-terminated path tracing (replaces the secondary pass):
 * trains the cache on cfg.train_paths fresh paths from this frame's camera
 * (cfg.train_steps Adam steps), then per pixel traces the primary hit's
 * shadow ray and, with query_vertex = 1, one diffuse bounce and that hit's
 * shadow ray, and ends the path in the cache:
 *   query_vertex 1: color = direct(x0) + throughput x (direct(x1) + cache(x1, n1, -d1))
 *   query_vertex 0: color = direct(x0) + cache(x0, n0, -d0)
 * where cache() is the learned indirect outgoing radiance.  Same g-buffer,
 * parameters and output as mrt_cuda_secondary_rays (max_bounces is
 * ignored). */
int mrt_cuda_cache_frame(mrt_ctx* ctx, mrt_cache* cache, const mrt_scene* scene,
                         const mrt_gbuffer* gbuffer, const mrt_camera_consts* consts,
                         const mrt_trace_params* params, float* color, int train, void* stream);

/* ---- learned denoiser (new; the reference's denoiser is the joint
 *      bilateral filter of src/gpu/denoise/bilateral.comp) --------------
 * A 3-level U-Net (3x3 convolutions, 32/64/128 channels, skip
 * connections) over 16-channel BF16 NHWC features: log(1 + radiance /
 * albedo), albedo, normal, depth, zero padding.  Forward on the tensor cores (BF16,
 * FP32 accumulate); training backward on the tensor cores with BF16
 * gradients (or in FP32, see the modes below); Adam on FP32 master weights.  The network predicts
 * a correction to the input's log(1 + radiance), with an L1 loss.  Width and height must be multiples
 * of 4. */
typedef struct mrt_denoiser mrt_denoiser;
int mrt_cuda_denoiser_create(mrt_ctx* ctx, uint32_t seed, mrt_denoiser** out);
int mrt_cuda_denoiser_destroy(mrt_ctx* ctx, mrt_denoiser* den);
int mrt_cuda_denoiser_param_count(mrt_denoiser* den, size_t* weights, size_t* biases);
/* Forward convolutions: mode 2 (default) on the tcgen05 tensor cores with
 * persistent, warp-specialised CTAs for the layers without upsampling (a
 * producer warp streaming tensor copies, an MMA warp, four epilogue warps,
 * two tensor-memory accumulators), mode 1 tcgen05 with one CTA per output
 * tile, mode 0 mma.sync (the earliest kernels, kept for comparison).  In
 * mode 2 the two upsampling layers gather their halo with four cp.async
 * producer warps; in mode 1 they run the per-tile cp.async kernel.
 * The training step's backward follows the mode too: mode 2 runs it on the
 * tensor cores (BF16 gradients at each layer's pre-activation, data
 * gradients as convolutions with the mirrored, transposed weights on the
 * persistent kernel, weight and bias gradients as tcgen05 GEMMs reducing
 * over the pixels), modes 1 and 0 on FP32 CUDA-core kernels.
 * Returns MRT_EINVAL for another mode. */
int mrt_cuda_denoiser_set_tcgen05(mrt_denoiser* den, int mode);
/* Features of one frame from its g-buffer (visibility + hit_t) and colour
 * (float RGB); scene_diagonal normalises depth.  features: device,
 * width*height*16 BF16. */
int mrt_cuda_denoiser_features(mrt_ctx* ctx, const mrt_scene* scene, const mrt_gbuffer* gbuffer,
                               const float* color, float scene_diagonal, uint16_t* features,
                               void* stream);
/* Denoised colour (float RGB) of `batch` feature images. */
int mrt_cuda_denoiser_infer(mrt_ctx* ctx, mrt_denoiser* den, const uint16_t* features, uint32_t batch,
                            uint32_t width, uint32_t height, float* out, void* stream);
/* One step on a batch of feature images and float RGB targets; lr is the
 * Adam learning rate; apply_update = 0 only accumulates gradients.
 * loss_out (host, may be NULL) receives the mean L1 loss and synchronises. */
int mrt_cuda_denoiser_train_step(mrt_ctx* ctx, mrt_denoiser* den, const uint16_t* features,
                                 const float* targets, uint32_t batch, uint32_t width, uint32_t height,
                                 float lr, int apply_update, float* loss_out, void* stream);
/* which = 0 weights then biases (FP32 masters; layer l's weights are
 * [cout][3x3 tap][cin]), 1 their gradients; set != 0 writes host -> device. */
int mrt_cuda_denoiser_params(mrt_ctx* ctx, mrt_denoiser* den, int which, float* host, size_t count,
                             int set);

/* ---- sky / atmosphere ---------------------------------------------------
 * Replaces Atmosphere and Sky (src/gfx/modules/sky.ixx:18-262) and their
 * shaders (src/gpu/sky/genTransmittance.comp, genMultiScattering.comp,
 * genView.comp).  Distances in kilometres; the planet centre is at
 * (0, 0, -bottom_radius) in world space (+Z up).  LUTs are float RGBA:
 * transmittance 256x64, multiple scattering 32x32, sky view 192x108. */
typedef struct mrt_atmosphere_params {  /* sky.ixx Atmosphere::Params :29-56 */
    float bottom_radius;               /* planet radius                      */
    float top_radius;                  /* radius of the atmosphere's top     */
    float rayleigh_density_exp_scale;  /* density = exp(scale * height)      */
    float rayleigh_scattering[3];
    float mie_density_exp_scale;
    float mie_scattering[3];
    float mie_extinction[3];
    float mie_absorption[3];
    float mie_phase_g;                 /* Cornette-Shanks asymmetry          */
    float absorption_density0_layer_width;   /* ozone tent: below the width */
    float absorption_density0_constant_term; /* linear*h + constant, above  */
    float absorption_density0_linear_term;   /* the second line, clamped to */
    float absorption_density1_constant_term; /* [0, 1]                      */
    float absorption_density1_linear_term;
    float absorption_extinction[3];
    float ground_albedo[3];
} mrt_atmosphere_params;
/* Earth's atmosphere (Atmosphere::Params::earth, sky.ixx:59-83). */
void mrt_atmosphere_earth(mrt_atmosphere_params* out);

typedef struct mrt_sky mrt_sky;
int mrt_cuda_sky_create(mrt_ctx* ctx, mrt_sky** out);
int mrt_cuda_sky_destroy(mrt_ctx* ctx, mrt_sky* sky);
/* Transmittance and multiple-scattering LUTs (Atmosphere ctor,
 * sky.ixx:84-174); the reference rebuilds them every frame. */
int mrt_cuda_sky_atmosphere(mrt_ctx* ctx, mrt_sky* sky, const mrt_atmosphere_params* params,
                            void* stream);
/* Sky-view LUT around probe_pos (Sky::createView, sky.ixx:199-262).  The
 * sun direction and illuminance also drive the sun disc of the miss
 * shader (the reference hard-codes the same defaults in
 * secondaryRays.comp:43-44 and sky.ixx:187-188). */
int mrt_cuda_sky_view(mrt_ctx* ctx, mrt_sky* sky, const float probe_pos[3], const float sun_dir[3],
                      const float sun_illuminance[3], void* stream);
/* Copies LUT `which` (0 transmittance, 1 multiple scattering, 2 sky view)
 * to host RGBA floats; count = floats available.  Synchronises. */
int mrt_cuda_sky_lut(mrt_ctx* ctx, const mrt_sky* sky, int which, float* host_rgba, size_t count);
/* skyColor(dir) (secondaryRays.comp:36-58) for n device directions ->
 * n device RGB floats, seen from camera_pos. */
int mrt_cuda_sky_eval(mrt_ctx* ctx, const mrt_sky* sky, const float camera_pos[3], const float* dirs,
                      uint32_t n, float* out_rgb, void* stream);
/* Binds `sky` (NULL: unbind) as the radiance of escaping paths in
 * mrt_cuda_secondary_rays and mrt_cuda_cache_frame, seen from the
 * camera's position; unbound, they use mrt_trace_params.sky_radiance.
 * The sky must outlive the binding and its view must be built. */
int mrt_cuda_set_sky(mrt_ctx* ctx, const mrt_sky* sky);

/* ---- joint bilateral filter ------------------------------------------------
 * Replaces Denoiser::bilateral (src/gfx/modules/denoiser.ixx:34-97) and
 * src/gpu/denoise/bilateral.comp: a circular Gaussian of radius
 * round(k_sigma * sigma) over the colour, each tap weighted by how well its
 * normal and linear depth agree with the centre's, plus the reference's
 * 0.005 x random dither.  Taps sit on whole columns and fractional rows
 * (the reference's d.y loop), read bilinearly with clamp-to-edge.  The
 * output stays float RGB (the reference writes RGBA8 UNORM, clamping HDR). */
#define MRT_BILATERAL_MAX_RADIUS 24
typedef struct mrt_bilateral_params {  /* BilateralParams, denoiser.ixx:20-31 */
    float    sigma;          /* 5.0                                          */
    float    k_sigma;        /* 2.0                                          */
    float    threshold;      /* 0.12                                         */
    float    near_plane;     /* camera near plane: linear depth = near / z  */
    uint32_t frame_counter;  /* dither seed (bilateral.comp:68)              */
    uint32_t dither;         /* 1: add the dither                            */
} mrt_bilateral_params;
void mrt_bilateral_defaults(mrt_bilateral_params* out);
/* color, out: device float RGB, width*height*3; gbuffer supplies depth
 * (R16F) and normal (RGBA16F).  out must not alias color. */
int mrt_cuda_bilateral(mrt_ctx* ctx, const mrt_gbuffer* gbuffer, const float* color,
                       const mrt_bilateral_params* params, float* out, void* stream);

/* ---- tonemappers ----------------------------------------------------------
 * Replaces Tonemapper (src/gfx/modules/tonemapper.ixx) and
 * src/gpu/tonemap/*.comp: exposure, one of six curves, sRGB encode, RGBA8
 * UNORM (round to nearest even, alpha 255). */
#define MRT_TONEMAP_LINEAR   0u
#define MRT_TONEMAP_REINHARD 1u
#define MRT_TONEMAP_HABLE    2u
#define MRT_TONEMAP_ACES     3u
#define MRT_TONEMAP_UCHIMURA 4u
#define MRT_TONEMAP_AMD      5u
typedef struct mrt_tonemap_params {
    uint32_t mode;             /* MRT_TONEMAP_*; the renderer's default: AMD  */
    float    exposure;         /* 1.0                                         */
    float    reinhard_max;     /* 8.0 (renderer.ixx)                          */
    float    uchimura[6];      /* max brightness 1, contrast 1, linear start
                                  0.22, linear length 0.4, black tightness
                                  1.33, pedestal 0 (tonemapper.ixx:20-40)     */
    float    amd[5];           /* hdr max 16, contrast 2, shoulder 1, mid in
                                  0.18, mid out 0.18 (tonemapper.ixx:42-57)   */
} mrt_tonemap_params;
void mrt_tonemap_defaults(mrt_tonemap_params* out);
/* color: device float RGB (width*height*3); out: device RGBA8. */
int mrt_cuda_tonemap(mrt_ctx* ctx, const float* color, uint32_t width, uint32_t height,
                     const mrt_tonemap_params* params, uint8_t* out, void* stream);

/* ---- temporal reprojection (new; the reference writes motion vectors in
 *      primaryRay.comp:73-75 and never reads them) --------------------------
 * Folds this frame's estimate into a history reprojected with the motion
 * vectors: the history is read bilinearly at the previous-frame position,
 * each of the four taps kept only when the previous frame saw a surface
 * there whose normal and linear depth agree with this pixel's reprojected
 * surface; the result is history + (sample - history) / n with the history
 * length n = min(previous n + 1, max_history), and n = 1 where no tap
 * survives (disocclusion) or the pixel sees the sky.  Both g-buffers need
 * visibility, hit_t, depth, normal and motion; `consts` are this frame's
 * (prev_view = the previous camera). */
typedef struct mrt_reproject_params {
    float max_history;  /* cap of n (frames)                                */
    float normal_cos;   /* minimum cosine between the normals (0.9)         */
    float depth_rel;    /* maximum |linear depth difference| / depth (0.05) */
    float pad;
} mrt_reproject_params;
/* sample, hist, out: device float RGB; hist_len, out_len: device float.
 * out / out_len must not alias hist / hist_len. */
int mrt_cuda_reproject(mrt_ctx* ctx, const mrt_gbuffer* cur, const mrt_gbuffer* prev,
                       const mrt_camera_consts* consts, const float* sample, const float* hist,
                       const float* hist_len, const mrt_reproject_params* params, float* out,
                       float* out_len, void* stream);

/* Primary rays for callers that cannot allocate device memory.
 *
 * No counterpart in the reference.  Some callers of this library may not
 * call cudaMalloc: a renderer whose host engine owns every device byte
 * through its own pool or budget, code running while a stream is being
 * captured into a CUDA graph (where a cudaMalloc is not recorded), or a
 * plug-in whose host forbids allocations on its render thread.  They pass
 * their own device buffers for the scene (BVH8 nodes, leaf-ordered
 * triangles, materials, as built by mrt_bvh8_build) and for the g-buffer,
 * and this entry point allocates nothing: no context, no cudaMalloc or
 * cudaFree, no allocating library call.
 *
 * It runs the persistent dynamic-fetch primary-ray kernel, whose work
 * counter lives in a file-scope device array of 256 bytes that every GPU
 * loading the library holds until the process exits.  The results equal
 * mrt_cuda_primary_rays.
 *
 *   - Works in the calling thread's current CUDA context (the runtime's
 *     primary context of the current device when none is current).  The
 *     first call in a context looks up that context's copy of the array and
 *     the launch size; make that first call before any stream capture.  A
 *     context created later (after cudaDeviceReset, or a caller's own
 *     driver-API context) gets its own look-up on its first call.
 *   - width * height must be at most MRT_NOALLOC_MAX_PIXELS; larger images
 *     return MRT_ERANGE and launch nothing.
 *   - All calls in a context share the one array, which keeps the previous
 *     call's contents; each call clears what must start at zero on
 *     `stream`.  Calls whose work overlaps on the GPU (other streams, other
 *     threads) race on the array: serialise them.
 *   - `status` (device, required) receives MRT_STATUS_* bits ORed in; the
 *     caller clears it and reads it back.  BVH depth is not checked on the
 *     host here: a BVH deeper than the traversal stack reports
 *     MRT_STATUS_STACK_OVF in `status`, and out-of-range node or triangle
 *     indices report MRT_STATUS_BAD_NODE / MRT_STATUS_BAD_TRI; the g-buffer
 *     is not to be trusted when any bit is set.
 * Returns MRT_OK, MRT_EINVAL (null pointer, including `status`, or zero
 * size), MRT_ERANGE (too large) or MRT_ECUDA. */
#define MRT_NOALLOC_MAX_PIXELS (1u << 26)
int mrt_cuda_primary_rays_noalloc(const mrt_bvh8_node* nodes, uint32_t node_count,
                                  const mrt_tri* tris, uint32_t tri_count,
                                  const mrt_material* materials, uint32_t material_count,
                                  const mrt_camera_consts* consts, const mrt_gbuffer* gbuffer,
                                  uint32_t* status, void* stream);

/* One whole frame through HOST buffers: primary + secondary passes on
 * library-owned device buffers, then copies of visibility, hit_t (may be
 * NULL) and color (float RGB) back to the host.  Synchronises `stream`. */
int mrt_cuda_render_frame_host(mrt_ctx* ctx, const mrt_scene* scene,
                               const mrt_camera_consts* consts,
                               const mrt_trace_params* params,
                               uint32_t width, uint32_t height,
                               uint32_t* visibility, float* hit_t, float* color,
                               void* stream);

/* The same frame with the read-back in flight: primary + secondary passes on
 * `stream` into one of two library-owned colour buffers (alternating per
 * call), then the colour copied to `color` (host, pinned for an
 * asynchronous copy) on a stream of the context; returns without
 * synchronising, so the next frame's passes overlap this frame's copy.
 * `color` must not be read, and a buffer passed here not reused, before
 * mrt_cuda_frames_wait returns.  Frames in flight do not accumulate:
 * params->accumulate must be 0 (MRT_EINVAL otherwise).  Same image as
 * mrt_cuda_render_frame_host. */
int mrt_cuda_render_frame_host_async(mrt_ctx* ctx, const mrt_scene* scene,
                                     const mrt_camera_consts* consts,
                                     const mrt_trace_params* params,
                                     uint32_t width, uint32_t height, float* color,
                                     void* stream);
/* Waits until every colour read-back of mrt_cuda_render_frame_host_async
 * has reached the host. */
int mrt_cuda_frames_wait(mrt_ctx* ctx);

#ifdef __cplusplus
}
#endif

#endif /* MRT_CUDA_H */
