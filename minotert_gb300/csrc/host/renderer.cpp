// Headless renderer over the C ABI: Renderer_impl::draw
// (src/gfx/renderer.ixx:39-68) minus the window, ImGui and swapchain.
//
// Per frame: atmosphere LUTs and the sky view at the camera (renderer.ixx
// :55-57, rebuilt every frame as there), primaryRays(camera, prevCamera)
// (:58), secondaryRays (:59), an optional reprojected history (new), the
// denoiser (:60; bilateral by default, :139) and the tonemapper (:61; AMD by
// default, :180) into RGBA8.  The previous camera is kept for the motion
// vectors (:50-51, :66).  Everything is stream-ordered on device buffers the
// renderer owns; mrt_renderer_read copies the result out.
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "mrt_host.h"

struct mrt_renderer {
    mrt_ctx* ctx = nullptr;
    const mrt_scene* scene = nullptr;
    uint32_t w = 0, h = 0;
    uint64_t frame = 0;
    mrt_camera prev{};
    mrt_sky* sky = nullptr;
    // two g-buffers (this frame / previous frame) and two histories
    mrt_gbuffer g[2]{};
    float* hist[2] = {nullptr, nullptr};
    float* hist_len[2] = {nullptr, nullptr};
    int cur = 0;
    bool have_history = false;
    float* sample = nullptr;   // this frame's path-traced estimate
    float* filtered = nullptr; // denoiser output
    uint8_t* rgba = nullptr;
    const float* hdr = nullptr;  // plane tonemapped last frame
    std::vector<void*> allocs;
};

namespace {

int alloc(mrt_renderer* r, size_t bytes, void** p) {
    int rc = mrt_cuda_alloc(r->ctx, bytes, p);
    if (rc == MRT_OK) r->allocs.push_back(*p);
    return rc;
}

}  // namespace

extern "C" {

void mrt_render_settings_defaults(mrt_render_settings* s) {
    if (!s) return;
    std::memset(s, 0, sizeof(*s));
    s->trace.samples = 8;  // secondaryRays.comp:128-129
    s->trace.max_bounces = 8;
    s->trace.rng_mode = MRT_RNG_REFERENCE;
    s->trace.estimator = MRT_EST_ESCAPE;
    s->trace.sun_dir[2] = 1.0f;
    s->sky_mode = MRT_SKY_ATMOSPHERE;
    s->accumulation = MRT_ACCUM_NONE;
    s->denoise = MRT_DENOISE_BILATERAL;
    mrt_atmosphere_earth(&s->atmosphere);
    const float sun[3] = {-0.435286462f, 0.818654716f, 0.374606609f};  // sky.ixx:186
    for (int k = 0; k < 3; ++k) {
        s->sun_dir[k] = sun[k];
        s->sun_illuminance[k] = 8.0f;
    }
    mrt_bilateral_defaults(&s->bilateral);
    s->reproject.max_history = 32.0f;
    s->reproject.normal_cos = 0.9f;
    s->reproject.depth_rel = 0.05f;
    mrt_tonemap_defaults(&s->tonemap);
}

int mrt_renderer_create(mrt_ctx* ctx, const mrt_scene* scene, uint32_t width, uint32_t height, mrt_renderer** out) {
    if (!ctx || !scene || !out || width == 0 || height == 0) return MRT_EINVAL;
    *out = nullptr;
    mrt_renderer* r = new (std::nothrow) mrt_renderer;
    if (!r) return MRT_ENOMEM;
    r->ctx = ctx;
    r->scene = scene;
    r->w = width;
    r->h = height;
    const size_t n = size_t(width) * height;
    int rc = MRT_OK;
    for (int k = 0; k < 2 && rc == MRT_OK; ++k) {
        void *vis, *t, *dep, *nrm, *mot, *hs, *hl;
        rc = alloc(r, n * 4, &vis);
        if (rc == MRT_OK) rc = alloc(r, n * 4, &t);
        if (rc == MRT_OK) rc = alloc(r, n * 2, &dep);
        if (rc == MRT_OK) rc = alloc(r, n * 8, &nrm);
        if (rc == MRT_OK) rc = alloc(r, n * 4, &mot);
        if (rc == MRT_OK) rc = alloc(r, n * 12, &hs);
        if (rc == MRT_OK) rc = alloc(r, n * 4, &hl);
        if (rc != MRT_OK) break;
        r->g[k].visibility = static_cast<uint32_t*>(vis);
        r->g[k].hit_t = static_cast<float*>(t);
        r->g[k].depth = static_cast<uint16_t*>(dep);
        r->g[k].normal = static_cast<uint16_t*>(nrm);
        r->g[k].motion = static_cast<uint16_t*>(mot);
        r->g[k].width = width;
        r->g[k].height = height;
        r->hist[k] = static_cast<float*>(hs);
        r->hist_len[k] = static_cast<float*>(hl);
    }
    void *smp = nullptr, *flt = nullptr, *rgba = nullptr;
    if (rc == MRT_OK) rc = alloc(r, n * 12, &smp);
    if (rc == MRT_OK) rc = alloc(r, n * 12, &flt);
    if (rc == MRT_OK) rc = alloc(r, n * 4, &rgba);
    if (rc == MRT_OK) rc = mrt_cuda_sky_create(ctx, &r->sky);
    if (rc == MRT_OK) {
        // the configs' 64x64 blue-noise tile; a caller may upload another
        uint8_t bn[64 * 64 * 4];
        rc = mrt_blue_noise_generate(1, 64, bn);
        if (rc == MRT_OK) rc = mrt_cuda_blue_noise_upload(ctx, bn, 64, 64);
    }
    if (rc != MRT_OK) {
        mrt_renderer_destroy(r);
        return rc;
    }
    r->sample = static_cast<float*>(smp);
    r->filtered = static_cast<float*>(flt);
    r->rgba = static_cast<uint8_t*>(rgba);
    *out = r;
    return MRT_OK;
}

int mrt_renderer_destroy(mrt_renderer* r) {
    if (!r) return MRT_OK;
    if (r->sky) mrt_cuda_sky_destroy(r->ctx, r->sky);
    for (void* p : r->allocs) mrt_cuda_free(r->ctx, p);
    delete r;
    return MRT_OK;
}

int mrt_renderer_draw(mrt_renderer* r, const mrt_camera* camera, const mrt_render_settings* s, void* stream) {
    if (!r || !camera || !s) return MRT_EINVAL;
    if (camera->viewport[0] != r->w || camera->viewport[1] != r->h) return MRT_EINVAL;
    if (r->frame == 0) r->prev = *camera;  // renderer.ixx:50-51
    const uint32_t fc = uint32_t(r->frame);
    mrt_camera_consts consts;
    mrt_camera_consts_make(camera, &r->prev, fc, &consts);
    // sky (renderer.ixx:55-57)
    const bool atmo = s->sky_mode == MRT_SKY_ATMOSPHERE;
    int rc = MRT_OK;
    if (atmo) {
        rc = mrt_cuda_sky_atmosphere(r->ctx, r->sky, &s->atmosphere, stream);
        if (rc == MRT_OK) rc = mrt_cuda_sky_view(r->ctx, r->sky, camera->position, s->sun_dir, s->sun_illuminance, stream);
        if (rc != MRT_OK) return rc;
    }
    // primaryRays (:58) into this frame's g-buffer
    const int cur = r->cur, prv = 1 - r->cur;
    rc = mrt_cuda_primary_rays(r->ctx, r->scene, &consts, &r->g[cur], stream);
    if (rc != MRT_OK) return rc;
    // secondaryRays (:59): this frame's estimate
    mrt_trace_params tp = s->trace;
    tp.accumulate = 0;
    rc = mrt_cuda_set_sky(r->ctx, atmo ? r->sky : nullptr);
    if (rc == MRT_OK) rc = mrt_cuda_secondary_rays(r->ctx, r->scene, &r->g[cur], &consts, &tp, r->sample, stream);
    mrt_cuda_set_sky(r->ctx, nullptr);
    if (rc != MRT_OK) return rc;
    const float* color = r->sample;
    // reprojected history (new)
    if (s->accumulation == MRT_ACCUM_REPROJECT) {
        const size_t n = size_t(r->w) * r->h;
        const mrt_gbuffer* pg = &r->g[prv];
        if (!r->have_history) {
            // no history yet: an empty one (length 0) over this frame's own
            // g-buffer, so the result is this frame's estimate with length 1
            rc = mrt_cuda_copy_d2d(r->ctx, r->hist[prv], r->sample, n * 12, stream);
            if (rc == MRT_OK) rc = mrt_cuda_memset(r->ctx, r->hist_len[prv], 0, n * 4, stream);
            if (rc != MRT_OK) return rc;
            pg = &r->g[cur];
        }
        rc = mrt_cuda_reproject(r->ctx, &r->g[cur], pg, &consts, r->sample, r->hist[prv], r->hist_len[prv],
                                &s->reproject, r->hist[cur], r->hist_len[cur], stream);
        if (rc != MRT_OK) return rc;
        r->have_history = true;
        color = r->hist[cur];
    } else {
        r->have_history = false;
    }
    // denoise (:60)
    if (s->denoise == MRT_DENOISE_BILATERAL) {
        mrt_bilateral_params bp = s->bilateral;
        bp.near_plane = camera->near_plane;
        bp.frame_counter = fc;
        rc = mrt_cuda_bilateral(r->ctx, &r->g[cur], color, &bp, r->filtered, stream);
        if (rc != MRT_OK) return rc;
        color = r->filtered;
    }
    // tonemap (:61)
    rc = mrt_cuda_tonemap(r->ctx, color, r->w, r->h, &s->tonemap, r->rgba, stream);
    if (rc != MRT_OK) return rc;
    r->hdr = color;
    r->prev = *camera;  // :66
    r->cur = prv;
    r->frame++;
    return MRT_OK;
}

const void* mrt_renderer_plane(const mrt_renderer* r, int which) {
    if (!r || r->frame == 0) return nullptr;
    switch (which) {
    case 0: return r->rgba;
    case 1: return r->hdr;
    case 2: return r->sample;
    case 3: return &r->g[1 - r->cur];
    default: return nullptr;
    }
}

int mrt_renderer_read(mrt_renderer* r, uint8_t* rgba8, float* hdr, void* stream) {
    if (!r || r->frame == 0) return MRT_EINVAL;
    const size_t n = size_t(r->w) * r->h;
    int rc = MRT_OK;
    if (rgba8) rc = mrt_cuda_copy_d2h(r->ctx, rgba8, r->rgba, n * 4, stream);
    if (rc == MRT_OK && hdr) rc = mrt_cuda_copy_d2h(r->ctx, hdr, r->hdr, n * 12, stream);
    if (rc == MRT_OK) rc = mrt_cuda_sync(r->ctx, stream, 0.0);
    return rc;
}

int mrt_write_ppm(const char* path, const uint8_t* rgba8, uint32_t width, uint32_t height) {
    if (!path || !rgba8) return MRT_EINVAL;
    FILE* f = std::fopen(path, "wb");
    if (!f) return MRT_EINVAL;
    std::fprintf(f, "P6\n%u %u\n255\n", width, height);
    bool ok = true;
    for (size_t i = 0; i < size_t(width) * height && ok; ++i) ok = std::fwrite(rgba8 + 4 * i, 1, 3, f) == 3;
    ok = std::fclose(f) == 0 && ok;
    return ok ? MRT_OK : MRT_EINVAL;
}

int mrt_write_pfm(const char* path, const float* rgb, uint32_t width, uint32_t height) {
    if (!path || !rgb) return MRT_EINVAL;
    FILE* f = std::fopen(path, "wb");
    if (!f) return MRT_EINVAL;
    std::fprintf(f, "PF\n%u %u\n-1.0\n", width, height);  // negative scale: little-endian
    bool ok = true;
    for (uint32_t y = 0; y < height && ok; ++y) {
        const float* row = rgb + size_t(height - 1 - y) * width * 3;
        ok = std::fwrite(row, sizeof(float), size_t(width) * 3, f) == size_t(width) * 3;
    }
    ok = std::fclose(f) == 0 && ok;
    return ok ? MRT_OK : MRT_EINVAL;
}

}  // extern "C"
