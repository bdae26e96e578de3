/*
 * mrt_host.h -- host-side C++ modules of the renderer, exported as C.
 *
 * These are the CPU parts that stay on the host in MinoteRT and that the
 * device layer (mrt_cuda.h) consumes:
 *   - camera math: Camera::view / Camera::projection (src/gfx/camera.ixx:
 *     26-44) over look / perspective / inverse (src/stx/math.ixx:739-861),
 *     and the per-dispatch constant fill of pathtracer.ixx:86-105, 171-184;
 *   - the acceleration structure: an SAH BVH2 collapsed to the quantised
 *     BVH8 of mrt_cuda.h (new: the reference has no BVH);
 *   - procedural scenes from a seed (new: the reference's scene is a
 *     5-sphere constant, scene.glsl:4-11, returned by mrt_scene_reference);
 *   - the blue-noise asset loader (a PNG decoder, renderer.ixx:101-110)
 *     and a blue-noise tile generator (void-and-cluster).
 * All entry points return MRT_OK or a negative MRT_E* code.
 */
#ifndef MRT_HOST_H
#define MRT_HOST_H

#include "mrt_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

/* The reference's Camera (camera.ixx:10-26), without the movement speeds. */
typedef struct mrt_camera {
    uint32_t viewport[2];  /* width, height                                  */
    float    vertical_fov; /* radians                                        */
    float    near_plane;
    float    position[3];
    float    yaw;          /* radians; direction = (cp*cy, cp*sy, sp)        */
    float    pitch;
} mrt_camera;

/* view = look(position, direction(), +Z)        (camera.ixx:32-35)
 * projection = perspective(fov, h/w, near)      (camera.ixx:38-41) */
void mrt_camera_view(const mrt_camera* cam, float out[16]);
void mrt_camera_projection(const mrt_camera* cam, float out[16]);
/* 4x4 inverse by cofactors (math.ixx:739-820). */
void mrt_mat4_inverse(const float m[16], float out[16]);
/* Fills mrt_camera_consts as pathtracer.ixx:86-105 and :171-184 do. */
void mrt_camera_consts_make(const mrt_camera* cam, const mrt_camera* prev_cam,
                            uint32_t frame_counter, mrt_camera_consts* out);

/* ---- triangle meshes ------------------------------------------------- */
typedef struct mrt_mesh {
    float*        verts;     /* tri_count * 9 floats: v0 v1 v2 per triangle  */
    mrt_material* materials; /* tri_count records                            */
    uint32_t      tri_count;
    uint32_t      pad;
    float         bounds_lo[3];
    float         bounds_hi[3];
} mrt_mesh;

void mrt_mesh_free(mrt_mesh* mesh);

/* Heightfield + boxes: a grid x grid cell heightfield (z = sum of 4 sine
 * octaves with seeded phases and frequencies; 2*grid^2 triangles) plus
 * `boxes` axis-aligned boxes with edge lengths U[0.5, 3] (12 triangles
 * each) resting on it; albedo U[0.2, 0.8] per object. */
int mrt_scene_heightfield_boxes(uint64_t seed, uint32_t grid, uint32_t boxes,
                                mrt_mesh* out);

/* Icosphere field: `spheres` icospheres subdivided `levels` times
 * (20*4^levels triangles each), radius log-uniform[rmin, rmax], vertices
 * displaced along the normal by seeded Perlin noise of amplitude
 * 0.05 * radius, over a ground plane of >= ground_tris triangles. */
int mrt_scene_icospheres(uint64_t seed, uint32_t spheres, uint32_t levels,
                         float rmin, float rmax, uint32_t ground_tris,
                         mrt_mesh* out);

/* Number of triangles of a heightfield whose triangle count is close to
 * `target` (used by the batched scene mix). */
uint32_t mrt_heightfield_grid_for(uint32_t target_tris);

/* ---- BVH ------------------------------------------------------------- */
typedef struct mrt_bvh_build_params {
    uint32_t sah_bins;       /* binned SAH bins (0 = 64)                     */
    uint32_t max_leaf_tris;  /* <= 3                                         */
    uint32_t threads;        /* 0 = hardware concurrency                     */
    uint32_t trav_cost_pct;  /* SAH cost of a BVH2 node step relative to a
                                triangle test, percent (0 = 50: splitting
                                small leaves is cheap, the collapse packs
                                the pieces into the same 8-wide node)        */
    uint32_t collapse;       /* BVH2 -> BVH8: 0 = greedy (open the child of
                                largest area until 8 slots are used), 1 =
                                SAH-optimal (dynamic programming over how
                                many child slots each subtree gets)          */
    uint32_t prim_cost_pct;  /* SAH-optimal collapse: cost of a triangle
                                test relative to visiting an 8-wide node,
                                percent (0 = 30)                             */
} mrt_bvh_build_params;

typedef struct mrt_bvh8 {
    mrt_bvh8_node* nodes;
    mrt_tri*       tris;
    uint32_t       node_count;
    uint32_t       tri_count;
    uint32_t       depth;       /* BVH8 levels, root = 1                     */
    uint32_t       leaf_count;
    double         build_ms;
    double         sah_cost;
} mrt_bvh8;

/* Binned SAH BVH2 over the triangles, collapsed into 8-wide nodes with
 * octant-ordered child slots and conservative 8-bit quantised boxes. */
int  mrt_bvh8_build(const float* verts, uint32_t tri_count,
                    const mrt_bvh_build_params* params, mrt_bvh8* out);
void mrt_bvh8_free(mrt_bvh8* bvh);

/* ---- reference scene 0 ---------------------------------------------- */
/* The 5 spheres of src/gpu/scene.glsl:4-11 (km units). */
uint32_t mrt_scene_reference(mrt_sphere* out /* [5] */);
/* The reference's default camera (app.ixx:20-32) at a given viewport. */
void mrt_camera_reference(uint32_t width, uint32_t height, mrt_camera* out);

/* ---- headless renderer ------------------------------------------------
 * Replaces Renderer_impl::draw (src/gfx/renderer.ixx:39-68) without the
 * window, ImGui and swapchain: per frame it (re)builds the atmosphere and
 * the sky view at the camera (:55-57), runs primaryRays with the previous
 * camera (:58), secondaryRays (:59), optionally folds the frame into a
 * reprojected history (new), denoises (:60, renderer.ixx:128-160) and
 * tonemaps (:61, :162-230) into RGBA8, all on device buffers owned by the
 * renderer; the previous camera is kept for the motion vectors (:66). */
#define MRT_ACCUM_NONE      0u /* each frame stands alone (the reference)    */
#define MRT_ACCUM_REPROJECT 1u /* mrt_cuda_reproject into a history          */
#define MRT_DENOISE_NONE      0u
#define MRT_DENOISE_BILATERAL 1u /* the reference's default                  */
#define MRT_SKY_CONSTANT   0u /* trace.sky_radiance                          */
#define MRT_SKY_ATMOSPHERE 1u /* the reference: LUTs rebuilt every frame     */
typedef struct mrt_render_settings {
    mrt_trace_params      trace;      /* samples, bounces, estimator, light   */
    uint32_t              sky_mode;   /* MRT_SKY_*                            */
    uint32_t              accumulation; /* MRT_ACCUM_*                        */
    uint32_t              denoise;    /* MRT_DENOISE_*                        */
    uint32_t              pad;
    mrt_atmosphere_params atmosphere; /* MRT_SKY_ATMOSPHERE                   */
    float                 sun_dir[3]; /* sky view sun (Sky, sky.ixx:186-187)  */
    float                 sun_illuminance[3];
    mrt_bilateral_params  bilateral;  /* near_plane / frame_counter are
                                         taken from the camera and frame     */
    mrt_reproject_params  reproject;
    mrt_tonemap_params    tonemap;
} mrt_render_settings;
/* The reference's defaults: 8 samples x 8 bounces, escape-only estimator,
 * reference RNG, Earth atmosphere, no accumulation, bilateral denoiser
 * (sigma 5, kSigma 2, threshold 0.12), AMD tonemapper at exposure 1. */
void mrt_render_settings_defaults(mrt_render_settings* out);

typedef struct mrt_renderer mrt_renderer;
int mrt_renderer_create(mrt_ctx* ctx, const mrt_scene* scene, uint32_t width, uint32_t height,
                        mrt_renderer** out);
int mrt_renderer_destroy(mrt_renderer* r);
/* Draws one frame on `stream` (stream-ordered; returns before the GPU
 * finishes).  The first frame's previous camera is the camera itself. */
int mrt_renderer_draw(mrt_renderer* r, const mrt_camera* camera, const mrt_render_settings* settings,
                      void* stream);
/* Device pointers of the last frame's planes: 0 RGBA8 output, 1 float RGB
 * before tonemapping, 2 float RGB path-traced estimate, 3 the g-buffer
 * (mrt_gbuffer*).  Valid until the next draw. */
const void* mrt_renderer_plane(const mrt_renderer* r, int which);
/* Copies the last frame to host memory (either pointer may be NULL):
 * rgba8 = width*height*4 bytes, hdr = width*height*3 floats.  Syncs. */
int mrt_renderer_read(mrt_renderer* r, uint8_t* rgba8, float* hdr, void* stream);
/* Binary PPM (P6, RGB from RGBA8) and PFM (PF, float RGB, bottom-up rows
 * as the format stores them).  Return 0 or MRT_EINVAL on an I/O error. */
int mrt_write_ppm(const char* path, const uint8_t* rgba8, uint32_t width, uint32_t height);
int mrt_write_pfm(const char* path, const float* rgb, uint32_t width, uint32_t height);

/* ---- blue noise ------------------------------------------------------ */
/* size x size RGBA8 blue-noise tile by void-and-cluster (Ulichney 1993),
 * one independent rank map per channel, seeded. size <= 256. */
int mrt_blue_noise_generate(uint32_t seed, uint32_t size, uint8_t* rgba_out);

/* The reference's blue-noise asset loader (renderer.ixx:101-110, which
 * calls lodepng::decode(..., LCT_RGBA, 8) on assets/blue_noise.png):
 * decodes an 8-bit, non-interlaced PNG -- greyscale, greyscale + alpha,
 * RGB or RGBA -- to RGBA8 rows, top row first, widening grey to (g, g, g)
 * and a missing alpha to 255.  With rgba == NULL only *width / *height
 * are set; otherwise rgba must hold 4 * width * height bytes.  Returns
 * MRT_OK, MRT_EINVAL (not a PNG this decoder reads, or corrupt: chunk
 * CRC-32 and zlib Adler-32 are checked; a missing file for _load) or
 * MRT_ERANGE (rgba_bytes too small). */
int mrt_png_decode_rgba8(const uint8_t* data, size_t size, uint8_t* rgba, size_t rgba_bytes,
                         uint32_t* width, uint32_t* height);
int mrt_png_load_rgba8(const char* path, uint8_t* rgba, size_t rgba_bytes,
                       uint32_t* width, uint32_t* height);

#ifdef __cplusplus
}
#endif

#endif /* MRT_HOST_H */
