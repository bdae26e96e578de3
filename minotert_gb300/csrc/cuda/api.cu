// The mrt_cuda_* C ABI: context, memory, scene upload and the two renderer
// passes.  Replaces the Vulkan device layer (src/sys/vulkan.ixx) and the vuk
// dispatches of src/gfx/modules/pathtracer.ixx on the ray-tracing path.
#include "internal.hpp"

#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <thread>

using namespace mrt;

namespace {

int fail(mrt_ctx* ctx, int code, const char* fmt, ...) {
    if (ctx) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        std::vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        ctx->err = buf;
    }
    return code;
}

#define MRT_CK(call)                                                                                   \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess) return fail(ctx, MRT_ECUDA, "%s: %s", #call, cudaGetErrorString(e_));  \
    } while (0)

inline cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }

// minote.math mat * mat (math.ixx:680-697): column c of the result is
// ((L0*R[c][0] + L1*R[c][1]) + L2*R[c][2]) + L3*R[c][3], no contraction.
void matmul4(const float* l, const float* r, float* out) {
    for (int c = 0; c < 4; ++c)
        for (int row = 0; row < 4; ++row) {
            float acc = l[0 * 4 + row] * r[c * 4 + 0];
            acc = acc + l[1 * 4 + row] * r[c * 4 + 1];
            acc = acc + l[2 * 4 + row] * r[c * 4 + 2];
            acc = acc + l[3 * 4 + row] * r[c * 4 + 3];
            out[c * 4 + row] = acc;
        }
}

FrameParams frame_params(const mrt_camera_consts* c, uint32_t w, uint32_t h) {
    FrameParams fp;
    std::memset(&fp, 0, sizeof(fp));
    fp.c = *c;
    matmul4(c->projection, c->view, fp.pv);
    matmul4(c->projection, c->prev_view, fp.ppv);
    fp.width = w;
    fp.height = h;
    fp.pitch_x = 1.0f / float(w); // OutPitch = vec2(1) / vec2(OutBounds)
    fp.pitch_y = 1.0f / float(h);
    return fp;
}

TraceParams trace_params(const mrt_trace_params* p) {
    TraceParams t{};
    t.samples = p->samples;
    t.max_bounces = p->max_bounces;
    t.rr_start = p->rr_start;
    t.rng_mode = p->rng_mode;
    t.estimator = p->estimator;
    t.exact_trig = p->exact_trig;
    for (int k = 0; k < 3; ++k) {
        t.sun[k] = p->sun_dir[k];
        t.sun_e[k] = p->sun_irradiance[k];
        t.sky[k] = p->sky_radiance[k];
    }
    return t;
}

cudaEvent_t get_event(mrt_ctx* ctx) {
    if (!ctx->ev_pool.empty()) {
        cudaEvent_t e = ctx->ev_pool.back();
        ctx->ev_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

struct Scope {
    mrt_ctx* ctx;
    cudaStream_t s;
    int kind, bounce;
    cudaEvent_t a = nullptr;
    Scope(mrt_ctx* c, cudaStream_t st, int k, int b) : ctx(c), s(st), kind(k), bounce(b) {
        if (ctx->timing) {
            a = get_event(ctx);
            cudaEventRecord(a, s);
        }
    }
    ~Scope() {
        if (ctx->timing && a) {
            cudaEvent_t b = get_event(ctx);
            cudaEventRecord(b, s);
            ctx->recs.push_back(mrt_timing_rec{kind, bounce, a, b});
        }
    }
};

void free_wave(WaveBuffers& wb) {
    cudaFree(wb.q[0]); cudaFree(wb.q[1]); cudaFree(wb.hits); cudaFree(wb.sq); cudaFree(wb.L);
    cudaFree(wb.rng); cudaFree(wb.counters); cudaFree(wb.keys); cudaFree(wb.perm);
    cudaFree(wb.qsort); cudaFree(wb.hist);
    wb = WaveBuffers();
}

int ensure_wave(mrt_ctx* ctx, size_t npix) {
    WaveBuffers& wb = ctx->wb;
    if (wb.cap >= npix && wb.counters) {
        wb.npix = npix;
        return MRT_OK;
    }
    free_wave(wb);
    size_t cap = npix;
    bool ok = cudaMalloc(&wb.q[0], cap * sizeof(PathRay)) == cudaSuccess &&
              cudaMalloc(&wb.q[1], cap * sizeof(PathRay)) == cudaSuccess &&
              cudaMalloc(&wb.hits, cap * sizeof(uint2)) == cudaSuccess &&
              cudaMalloc(&wb.sq, cap * sizeof(ShadowRay)) == cudaSuccess &&
              cudaMalloc(&wb.L, npix * sizeof(float4)) == cudaSuccess &&
              cudaMalloc(&wb.rng, npix * sizeof(uint32_t)) == cudaSuccess &&
              cudaMalloc(&wb.counters, kCntSlots * sizeof(uint32_t)) == cudaSuccess &&
              cudaMalloc(&wb.keys, cap * sizeof(uint32_t)) == cudaSuccess &&
              cudaMalloc(&wb.qsort, cap * sizeof(PathRay)) == cudaSuccess &&
              cudaMalloc(&wb.hist, 4096 * sizeof(uint32_t)) == cudaSuccess;
    wb.totals = ctx->d_totals;
    if (!ok) {
        free_wave(wb);
        return fail(ctx, MRT_ENOMEM, "wavefront buffers for %zu rays: out of device memory", npix);
    }
    wb.cap = cap;
    wb.npix = npix;
    return MRT_OK;
}

// Persistent traversal grid: blocks per SM from the tuning (0 = the
// occupancy maximum, computed once per context) times the SM count.
int trace_blocks(mrt_ctx* ctx) {
    if (ctx->occ_blocks == 0) ctx->occ_blocks = trace_blocks_per_sm();
    int per_sm = ctx->tuning.trace_blocks_per_sm ? int(ctx->tuning.trace_blocks_per_sm) : ctx->occ_blocks;
    if (per_sm > ctx->occ_blocks) per_sm = ctx->occ_blocks;
    return per_sm * ctx->sm_count;
}


int check_gbuffer(mrt_ctx* ctx, const mrt_gbuffer* g) {
    if (!g || !g->visibility) return fail(ctx, MRT_EINVAL, "gbuffer.visibility is NULL");
    if (g->width == 0 || g->height == 0) return fail(ctx, MRT_EINVAL, "gbuffer has zero size");
    if (uint64_t(g->width) * g->height > (1ull << 28)) return fail(ctx, MRT_ERANGE, "gbuffer larger than 2^28 pixels");
    return MRT_OK;
}

} // namespace

namespace mrt {
// Depth of a BVH8 along in-range child links, each node counted once (a
// corrupt blob with cycles still terminates; traversal bounds-checks the
// rest at run time).  The traversal stack holds at most depth - 1 entries.
uint32_t bvh8_depth(const mrt_bvh8_node* nodes, uint32_t n) {
    std::vector<uint8_t> seen(n, 0);
    std::vector<std::pair<uint32_t, uint32_t>> st{{0u, 1u}};
    uint32_t depth = 0;
    seen[0] = 1;
    while (!st.empty()) {
        auto [ni, d] = st.back();
        st.pop_back();
        depth = d > depth ? d : depth;
        const mrt_bvh8_node& nd = nodes[ni];
        uint32_t k = 0;
        for (int s = 0; s < 8; ++s) {
            if (!((nd.imask >> s) & 1u)) continue;
            uint64_t c = uint64_t(nd.child_base) + k++;
            if (c < n && !seen[c]) {
                seen[c] = 1;
                st.push_back({uint32_t(c), d + 1});
            }
        }
    }
    return depth;
}

// learned radiance cache (nrc.cu)
cudaError_t cache_infer(const mrt_cache* c, const float* q, uint32_t n, const uint32_t* n_dev, float* out,
                        uint32_t* status, cudaStream_t s);
int cache_frame_buffers(mrt_ctx* ctx, mrt_cache* c, size_t n, float** q, float4** pb, float** pred);
int cache_train_frame(mrt_ctx* ctx, mrt_cache* c, const DevScene& sc, const FrameParams& fp, const TraceParams& tp,
                      uint32_t* status, cudaStream_t s);
// Frame constants for entry points outside this file (noalloc.cu).
FrameParams make_frame_params(const mrt_camera_consts* c, uint32_t w, uint32_t h) { return frame_params(c, w, h); }
// Error reporting, persistent grid size and trace-parameter conversion for
// the other C-ABI files (batch.cu).
int set_error(mrt_ctx* ctx, int code, const char* msg) { return fail(ctx, code, "%s", msg); }
int persistent_blocks(mrt_ctx* ctx) { return trace_blocks(ctx); }
TraceParams make_trace_params(const mrt_trace_params* p) { return trace_params(p); }
} // namespace mrt

extern "C" {

int mrt_cuda_abi_version(void) { return MRT_ABI_VERSION; }

const char* mrt_cuda_last_error(const mrt_ctx* ctx) {
    if (!ctx) return "null context";
    return ctx->err.c_str();
}

int mrt_cuda_create(mrt_ctx** out, int device) {
    if (!out) return MRT_EINVAL;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return MRT_ECUDA;
    if (device < 0 || device >= n) return MRT_EINVAL;
    if (cudaSetDevice(device) != cudaSuccess) return MRT_ECUDA;
    mrt_ctx* ctx = new (std::nothrow) mrt_ctx;
    if (!ctx) return MRT_ENOMEM;
    ctx->device = device;
    cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (cudaMalloc(&ctx->d_status, sizeof(uint32_t)) != cudaSuccess ||
        cudaMemset(ctx->d_status, 0, sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc(&ctx->d_totals, kTotSlots * sizeof(unsigned long long)) != cudaSuccess ||
        cudaMemset(ctx->d_totals, 0, kTotSlots * sizeof(unsigned long long)) != cudaSuccess ||
        cudaMalloc(&ctx->d_prim_fetch, sizeof(uint32_t)) != cudaSuccess) {
        cudaFree(ctx->d_status);
        cudaFree(ctx->d_totals);
        cudaFree(ctx->d_prim_fetch);
        delete ctx;
        return MRT_ENOMEM;
    }
    // the side stream of overlap_shadow exists from the start, so that a
    // frame captured into a graph by the caller never creates it
    if (cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming) != cudaSuccess) {
        mrt_cuda_destroy(ctx);
        return MRT_ECUDA;
    }
    *out = ctx;
    return MRT_OK;
}

int mrt_cuda_destroy(mrt_ctx* ctx) {
    if (!ctx) return MRT_EINVAL;
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();
    free_wave(ctx->wb);
    cudaFree(ctx->d_status);
    cudaFree(ctx->d_totals);
    cudaFree(ctx->d_prim_fetch);
    cudaFree(ctx->d_bn);
    cudaFree(ctx->d_vis);
    cudaFree(ctx->d_aux);
    cudaFree(ctx->d_t);
    cudaFree(ctx->d_color);
    for (int b = 0; b < 2; ++b) {
        cudaFree(ctx->d_color_async[b]);
        if (ctx->ev_rendered[b]) cudaEventDestroy(ctx->ev_rendered[b]);
        if (ctx->ev_copied[b]) cudaEventDestroy(ctx->ev_copied[b]);
    }
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    for (auto& r : ctx->recs) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
    for (auto e : ctx->ev_pool) cudaEventDestroy(e);
    if (ctx->side) cudaStreamDestroy(ctx->side);
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    delete ctx;
    return MRT_OK;
}

int mrt_cuda_status(mrt_ctx* ctx, uint32_t* flags, int clear) {
    if (!ctx || !flags) return MRT_EINVAL;
    cudaSetDevice(ctx->device);
    MRT_CK(cudaDeviceSynchronize());
    MRT_CK(cudaMemcpy(flags, ctx->d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    if (clear) MRT_CK(cudaMemset(ctx->d_status, 0, sizeof(uint32_t)));
    return MRT_OK;
}

int mrt_cuda_sync(mrt_ctx* ctx, void* stream, double timeout_s) {
    if (!ctx) return MRT_EINVAL;
    cudaSetDevice(ctx->device);
    auto t0 = std::chrono::steady_clock::now();
    while (true) {
        cudaError_t e = cudaStreamQuery(as_stream(stream));
        if (e == cudaSuccess) return MRT_OK;
        if (e != cudaErrorNotReady) return fail(ctx, MRT_ECUDA, "stream query: %s", cudaGetErrorString(e));
        double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (timeout_s > 0.0 && el > timeout_s)
            return fail(ctx, MRT_ETIMEOUT, "stream not finished after %.3f s", timeout_s);
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
}

int mrt_cuda_set_timing(mrt_ctx* ctx, int enable) {
    if (!ctx) return MRT_EINVAL;
    ctx->timing = enable != 0;
    return MRT_OK;
}

// Work schedule of the extension (which = 0) or shadow (which = 1) trace
// kernels from mrt_tuning.dynamic_fetch and tri_spread.
static int fetch_mode(const mrt_ctx* ctx, uint32_t which) {
    const bool spread = ((ctx->tuning.tri_spread >> which) & 1u) != 0u;
    if (!((ctx->tuning.dynamic_fetch >> which) & 1u)) return spread ? mrt::kFetchBatchSpread : mrt::kFetchBatch;
    return spread ? mrt::kFetchSpread : mrt::kFetchDynamic;
}

static uint32_t refill_min(const mrt_ctx* ctx) { return ctx->tuning.refill_min ? ctx->tuning.refill_min : 1u; }



int mrt_cuda_set_tuning(mrt_ctx* ctx, const mrt_tuning* tuning) {
    if (!ctx || !tuning) return fail(ctx, MRT_EINVAL, "set_tuning: null argument");
    if (tuning->trace_blocks_per_sm > 64 || tuning->dynamic_fetch > 3 || tuning->primary_persistent > 1 ||
        tuning->tail_bounce > MRT_MAX_BOUNCES || tuning->tri_spread > 15 || tuning->refill_min > 32 || tuning->overlap_shadow > 2 ||
        tuning->tail_from_hits > 1 ||
        (tuning->stack_depth != 0u && tuning->stack_depth != 16u && tuning->stack_depth != 24u &&
         tuning->stack_depth != 32u))
        return fail(ctx, MRT_EINVAL, "set_tuning: value out of range");
    ctx->tuning = *tuning;
    return MRT_OK;
}

int mrt_cuda_get_tuning(mrt_ctx* ctx, mrt_tuning* tuning) {
    if (!ctx || !tuning) return fail(ctx, MRT_EINVAL, "get_tuning: null argument");
    *tuning = ctx->tuning;
    return MRT_OK;
}

int mrt_cuda_device_info(mrt_ctx* ctx, mrt_device_info* out) {
    if (!ctx || !out) return fail(ctx, MRT_EINVAL, "device_info: null argument");
    cudaSetDevice(ctx->device);
    cudaDeviceProp p;
    MRT_CK(cudaGetDeviceProperties(&p, ctx->device));
    std::memset(out, 0, sizeof(*out));
    std::snprintf(out->name, sizeof(out->name), "%s", p.name);
    out->sm_count = p.multiProcessorCount;
    out->cc_major = p.major;
    out->cc_minor = p.minor;
    if (ctx->occ_blocks == 0) ctx->occ_blocks = trace_blocks_per_sm();
    out->trace_blocks_per_sm_max = uint32_t(ctx->occ_blocks);
    out->total_mem = p.totalGlobalMem;
    out->l2_bytes = uint64_t(p.l2CacheSize);
    return MRT_OK;
}

int mrt_cuda_set_counters(mrt_ctx* ctx, int enable) {
    if (!ctx) return MRT_EINVAL;
    ctx->counters = enable != 0;
    return MRT_OK;
}

int mrt_cuda_frame_stats(mrt_ctx* ctx, mrt_frame_stats* out) {
    if (!ctx || !out) return MRT_EINVAL;
    cudaSetDevice(ctx->device);
    MRT_CK(cudaDeviceSynchronize());
    mrt_frame_stats st = ctx->acc;
    for (auto& r : ctx->recs) {
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, r.a, r.b);
        switch (r.kind) {
        case 0: st.ms_primary += ms; break;
        case 1:
            st.ms_extend += ms;
            if (r.bounce >= 1 && r.bounce <= MRT_MAX_BOUNCES) st.ms_extend_b[r.bounce - 1] += ms;
            break;
        case 2: st.ms_shadow += ms; break;
        case 3: st.ms_shade += ms; break;
        case 4: st.ms_sort += ms; break;
        case 5: st.ms_total += ms; break;
        case 6: st.ms_cache_train += ms; break;
        case 7: st.ms_cache_infer += ms; break;
        default: break;
        }
        ctx->ev_pool.push_back(r.a);
        ctx->ev_pool.push_back(r.b);
    }
    ctx->recs.clear();
    {
        unsigned long long tot[kTotSlots];
        MRT_CK(cudaMemcpy(tot, ctx->d_totals, sizeof(tot), cudaMemcpyDeviceToHost));
        MRT_CK(cudaMemset(ctx->d_totals, 0, sizeof(tot)));
        for (int b = 1; b <= MRT_MAX_BOUNCES; ++b) {
            st.extension_rays[b - 1] += tot[kCntExt + b];
            st.nodes_extension[b - 1] += tot[kTotNodesExt + b];
            st.tris_extension[b - 1] += tot[kTotTrisExt + b];
        }
        for (int v = 0; v <= MRT_MAX_BOUNCES; ++v) st.shadow_rays += tot[kCntShadow + v];
        st.nodes_shadow += tot[kTotNodesShadow];
        st.tris_shadow += tot[kTotTrisShadow];
        st.nodes_primary += tot[kTotNodesPrim];
        st.tris_primary += tot[kTotTrisPrim];
    }
    st.launches = ctx->launches;
    *out = st;
    ctx->acc = mrt_frame_stats{};
    ctx->launches = 0;
    return MRT_OK;
}

// ---- memory ---------------------------------------------------------------

int mrt_cuda_alloc(mrt_ctx* ctx, size_t bytes, void** dptr) {
    if (!ctx || !dptr) return MRT_EINVAL;
    cudaSetDevice(ctx->device);
    *dptr = nullptr;
    if (bytes == 0) return MRT_OK;
    if (cudaMalloc(dptr, bytes) != cudaSuccess) {
        cudaGetLastError();
        return fail(ctx, MRT_ENOMEM, "cudaMalloc(%zu) failed", bytes);
    }
    return MRT_OK;
}

int mrt_cuda_free(mrt_ctx* ctx, void* dptr) {
    if (!ctx) return MRT_EINVAL;
    cudaSetDevice(ctx->device);
    MRT_CK(cudaFree(dptr));
    return MRT_OK;
}

int mrt_cuda_host_alloc(mrt_ctx* ctx, size_t bytes, void** hptr) {
    if (!ctx || !hptr) return MRT_EINVAL;
    cudaSetDevice(ctx->device);
    if (cudaMallocHost(hptr, bytes ? bytes : 1) != cudaSuccess) {
        cudaGetLastError();
        return fail(ctx, MRT_ENOMEM, "cudaMallocHost(%zu) failed", bytes);
    }
    return MRT_OK;
}

int mrt_cuda_host_free(mrt_ctx* ctx, void* hptr) {
    if (!ctx) return MRT_EINVAL;
    MRT_CK(cudaFreeHost(hptr));
    return MRT_OK;
}

int mrt_cuda_copy_h2d(mrt_ctx* ctx, void* dst, const void* src, size_t bytes, void* stream) {
    if (!ctx || (bytes && (!dst || !src))) return MRT_EINVAL;
    cudaSetDevice(ctx->device);
    MRT_CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, as_stream(stream)));
    return MRT_OK;
}

int mrt_cuda_copy_d2h(mrt_ctx* ctx, void* dst, const void* src, size_t bytes, void* stream) {
    if (!ctx || (bytes && (!dst || !src))) return MRT_EINVAL;
    cudaSetDevice(ctx->device);
    MRT_CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, as_stream(stream)));
    return MRT_OK;
}

int mrt_cuda_copy_d2d(mrt_ctx* ctx, void* dst, const void* src, size_t bytes, void* stream) {
    if (!ctx || (bytes && (!dst || !src))) return MRT_EINVAL;
    cudaSetDevice(ctx->device);
    MRT_CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, as_stream(stream)));
    return MRT_OK;
}

int mrt_cuda_memset(mrt_ctx* ctx, void* dst, int value, size_t bytes, void* stream) {
    if (!ctx || (bytes && !dst)) return MRT_EINVAL;
    cudaSetDevice(ctx->device);
    MRT_CK(cudaMemsetAsync(dst, value, bytes, as_stream(stream)));
    return MRT_OK;
}

int mrt_cuda_stream_create(mrt_ctx* ctx, void** stream) {
    if (!ctx || !stream) return MRT_EINVAL;
    cudaSetDevice(ctx->device);
    cudaStream_t s;
    MRT_CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    *stream = s;
    return MRT_OK;
}

int mrt_cuda_stream_destroy(mrt_ctx* ctx, void* stream) {
    if (!ctx) return MRT_EINVAL;
    MRT_CK(cudaStreamDestroy(as_stream(stream)));
    return MRT_OK;
}

int mrt_cuda_event_create(mrt_ctx* ctx, void** event) {
    if (!ctx || !event) return MRT_EINVAL;
    cudaSetDevice(ctx->device);
    cudaEvent_t e;
    MRT_CK(cudaEventCreate(&e));
    *event = e;
    return MRT_OK;
}

int mrt_cuda_event_destroy(mrt_ctx* ctx, void* event) {
    if (!ctx) return MRT_EINVAL;
    MRT_CK(cudaEventDestroy(static_cast<cudaEvent_t>(event)));
    return MRT_OK;
}

int mrt_cuda_event_record(mrt_ctx* ctx, void* event, void* stream) {
    if (!ctx || !event) return MRT_EINVAL;
    MRT_CK(cudaEventRecord(static_cast<cudaEvent_t>(event), as_stream(stream)));
    return MRT_OK;
}

int mrt_cuda_event_elapsed(mrt_ctx* ctx, void* start, void* stop, float* ms) {
    if (!ctx || !start || !stop || !ms) return MRT_EINVAL;
    MRT_CK(cudaEventSynchronize(static_cast<cudaEvent_t>(stop)));
    MRT_CK(cudaEventElapsedTime(ms, static_cast<cudaEvent_t>(start), static_cast<cudaEvent_t>(stop)));
    return MRT_OK;
}

// ---- scenes ---------------------------------------------------------------

int mrt_cuda_scene_upload_triangles(mrt_ctx* ctx, const mrt_bvh8_node* nodes, uint32_t node_count,
                                    const mrt_tri* tris, uint32_t tri_count, const mrt_material* materials,
                                    uint32_t material_count, mrt_scene** out) {
    if (!ctx || !out || !nodes || !tris || !materials || node_count == 0 || tri_count == 0 || material_count == 0)
        return fail(ctx, MRT_EINVAL, "scene_upload_triangles: null pointer or empty scene");
    cudaSetDevice(ctx->device);
    *out = nullptr;
    const uint32_t depth = bvh8_depth(nodes, node_count);
    if (depth > uint32_t(kStackDepth))
        return fail(ctx, MRT_ERANGE, "BVH8 depth %u exceeds the traversal stack (%d levels)", depth, kStackDepth);
    mrt_scene* sc = new (std::nothrow) mrt_scene;
    if (!sc) return MRT_ENOMEM;
    size_t nb = size_t(node_count) * sizeof(mrt_bvh8_node), tb = size_t(tri_count) * sizeof(mrt_tri),
           mb = size_t(material_count) * sizeof(mrt_material);
    if (cudaMalloc(&sc->d_nodes, nb) != cudaSuccess || cudaMalloc(&sc->d_tris, tb) != cudaSuccess ||
        cudaMalloc(&sc->d_mats, mb) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(sc->d_nodes); cudaFree(sc->d_tris); cudaFree(sc->d_mats);
        delete sc;
        return fail(ctx, MRT_ENOMEM, "scene upload: out of device memory (%zu bytes)", nb + tb + mb);
    }
    if (cudaMemcpy(sc->d_nodes, nodes, nb, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(sc->d_tris, tris, tb, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(sc->d_mats, materials, mb, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(sc->d_nodes); cudaFree(sc->d_tris); cudaFree(sc->d_mats);
        delete sc;
        return fail(ctx, MRT_ECUDA, "scene upload: copy failed");
    }
    sc->kind = 0;
    sc->dev.nodes = static_cast<const uint4*>(sc->d_nodes);
    sc->dev.tris = static_cast<const float4*>(sc->d_tris);
    sc->dev.mats = static_cast<const mrt_material*>(sc->d_mats);
    sc->dev.spheres = nullptr;
    sc->dev.node_count = node_count;
    sc->dev.tri_count = tri_count;
    sc->dev.mat_count = material_count;
    sc->dev.sphere_count = 0;
    // scene bounds from the root's quantised child boxes (conservative)
    {
        const mrt_bvh8_node& r = nodes[0];
        const uint8_t* ql[3] = {r.q_lo_x, r.q_lo_y, r.q_lo_z};
        const uint8_t* qh[3] = {r.q_hi_x, r.q_hi_y, r.q_hi_z};
        for (int a = 0; a < 3; ++a) {
            int lo = 255, hi = 0;
            for (int s = 0; s < 8; ++s)
                if (r.meta[s]) { lo = ql[a][s] < lo ? ql[a][s] : lo; hi = qh[a][s] > hi ? qh[a][s] : hi; }
            const float sc_e = std::ldexp(1.0f, r.exp[a]);
            const float l = r.origin[a] + float(lo) * sc_e, h = r.origin[a] + float(hi) * sc_e;
            sc->dev.lo[a] = l;
            sc->dev.inv_ext[a] = h > l ? 1.0f / (h - l) : 0.0f;
        }
    }
    *out = sc;
    return MRT_OK;
}

int mrt_cuda_scene_upload_spheres(mrt_ctx* ctx, const mrt_sphere* spheres, uint32_t count, mrt_scene** out) {
    if (!ctx || !out || !spheres || count == 0 || count > 4096)
        return fail(ctx, MRT_EINVAL, "scene_upload_spheres: bad arguments");
    cudaSetDevice(ctx->device);
    mrt_scene* sc = new (std::nothrow) mrt_scene;
    if (!sc) return MRT_ENOMEM;
    if (cudaMalloc(&sc->d_spheres, count * sizeof(mrt_sphere)) != cudaSuccess) {
        cudaGetLastError();
        delete sc;
        return fail(ctx, MRT_ENOMEM, "sphere upload failed");
    }
    if (cudaMemcpy(sc->d_spheres, spheres, count * sizeof(mrt_sphere), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(sc->d_spheres);
        delete sc;
        return fail(ctx, MRT_ECUDA, "sphere upload copy failed");
    }
    sc->kind = 1;
    sc->dev.spheres = static_cast<const float4*>(sc->d_spheres);
    sc->dev.sphere_count = count;
    *out = sc;
    return MRT_OK;
}

int mrt_cuda_scene_destroy(mrt_ctx* ctx, mrt_scene* scene) {
    if (!ctx || !scene) return MRT_EINVAL;
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();
    cudaFree(scene->d_nodes);
    cudaFree(scene->d_tris);
    cudaFree(scene->d_mats);
    cudaFree(scene->d_spheres);
    delete scene;
    return MRT_OK;
}

int mrt_cuda_blue_noise_upload(mrt_ctx* ctx, const uint8_t* rgba, uint32_t w, uint32_t h) {
    if (!ctx || !rgba || w == 0 || h == 0 || w > 1024 || h > 1024)
        return fail(ctx, MRT_EINVAL, "blue_noise_upload: bad arguments");
    cudaSetDevice(ctx->device);
    std::vector<float2> rot(size_t(w) * h);
    for (size_t i = 0; i < rot.size(); ++i) {
        // R8G8B8A8_UNORM: channel byte / 255 (renderer.ixx:104-105)
        rot[i].x = float(rgba[4 * i + 0]) / 255.0f;
        rot[i].y = float(rgba[4 * i + 1]) / 255.0f;
    }
    cudaFree(ctx->d_bn);
    ctx->d_bn = nullptr;
    MRT_CK(cudaMalloc(&ctx->d_bn, rot.size() * sizeof(float2)));
    MRT_CK(cudaMemcpy(ctx->d_bn, rot.data(), rot.size() * sizeof(float2), cudaMemcpyHostToDevice));
    ctx->bn_w = w;
    ctx->bn_h = h;
    return MRT_OK;
}

// ---- passes ---------------------------------------------------------------

int mrt_cuda_primary_rays(mrt_ctx* ctx, const mrt_scene* scene, const mrt_camera_consts* consts,
                          const mrt_gbuffer* gbuffer, void* stream) {
    if (!ctx || !scene || !consts) return fail(ctx, MRT_EINVAL, "primary_rays: null argument");
    int rc = check_gbuffer(ctx, gbuffer);
    if (rc) return rc;
    cudaSetDevice(ctx->device);
    FrameParams fp = frame_params(consts, gbuffer->width, gbuffer->height);
    cudaStream_t s = as_stream(stream);
    {
        Scope sc(ctx, s, 0, 0);
        cudaError_t e = scene->kind == 0
                            ? launch_primary_tri(scene->dev, fp, *gbuffer, ctx->d_status,
                                                 ctx->counters ? ctx->d_totals : nullptr,
                                                 ctx->tuning.primary_persistent ? ctx->d_prim_fetch : nullptr,
                                                 trace_blocks(ctx), (ctx->tuning.tri_spread & 4u) != 0u,
                                                 refill_min(ctx), s)
                            : launch_primary_sphere(scene->dev, fp, *gbuffer, s);
        if (e != cudaSuccess) return fail(ctx, MRT_ECUDA, "primary rays launch: %s", cudaGetErrorString(e));
    }
    ctx->launches++;
    ctx->acc.primary_rays += uint64_t(gbuffer->width) * gbuffer->height;
    return MRT_OK;
}

int mrt_cuda_secondary_rays(mrt_ctx* ctx, const mrt_scene* scene, const mrt_gbuffer* gbuffer,
                            const mrt_camera_consts* consts, const mrt_trace_params* params, float* color,
                            void* stream) {
    if (!ctx || !scene || !consts || !params || !color) return fail(ctx, MRT_EINVAL, "secondary_rays: null argument");
    int rc = check_gbuffer(ctx, gbuffer);
    if (rc) return rc;
    if (params->samples == 0 || params->samples > 65536) return fail(ctx, MRT_EINVAL, "samples must be 1..65536");
    if (params->max_bounces > MRT_MAX_BOUNCES) return fail(ctx, MRT_ERANGE, "max_bounces > %d", MRT_MAX_BOUNCES);
    if (params->rng_mode > MRT_RNG_PER_PIXEL || params->estimator > MRT_EST_NEE)
        return fail(ctx, MRT_EINVAL, "bad rng_mode or estimator");
    if (!ctx->d_bn) return fail(ctx, MRT_ESTATE, "no blue-noise texture uploaded");
    cudaSetDevice(ctx->device);
    cudaStream_t s = as_stream(stream);
    const uint32_t W = gbuffer->width, H = gbuffer->height;
    FrameParams fp = frame_params(consts, W, H);
    TraceParams tp = trace_params(params);
    tp.atmo = sky_dev(ctx->sky, consts->camera_pos);
    BlueNoise bn{ctx->d_bn, ctx->bn_w, ctx->bn_h};
    Scope total(ctx, s, 5, 0);
    if (scene->kind == 1) {
        if (!gbuffer->depth || !gbuffer->normal)
            return fail(ctx, MRT_EINVAL, "sphere scenes need gbuffer depth and normal");
        Scope sc(ctx, s, 3, 0);
        cudaError_t e = launch_secondary_sphere(scene->dev, fp, *gbuffer, tp, bn, color, params->accumulate,
                                                params->frame_index, s);
        if (e != cudaSuccess) return fail(ctx, MRT_ECUDA, "secondary launch: %s", cudaGetErrorString(e));
        ctx->launches++;
        return MRT_OK;
    }
    if (!gbuffer->hit_t) return fail(ctx, MRT_EINVAL, "triangle scenes need gbuffer hit_t");
    rc = ensure_wave(ctx, size_t(W) * H);
    if (rc) return rc;
    WaveBuffers& wb = ctx->wb;
    const int tblocks = trace_blocks(ctx);
    const bool nee = tp.estimator == MRT_EST_NEE;
    const int dyn = fetch_mode(ctx, 0u), dyn_sh = fetch_mode(ctx, 1u);
    const bool overlap_sh = ctx->tuning.overlap_shadow != 0u && !ctx->counters;
#define MRT_LAUNCH_ON(st_, kind, bounce, expr)                                                           \
    do {                                                                                                 \
        Scope sc_(ctx, st_, kind, bounce);                                                               \
        cudaError_t e_ = (expr);                                                                         \
        if (e_ != cudaSuccess) return fail(ctx, MRT_ECUDA, "%s: %s", #expr, cudaGetErrorString(e_));    \
        ctx->launches++;                                                                                 \
    } while (0)
#define MRT_LAUNCH(kind, bounce, expr) MRT_LAUNCH_ON(s, kind, bounce, expr)
    for (uint32_t smp = 0; smp < tp.samples; ++smp) {
        MRT_CK(cudaMemsetAsync(wb.counters, 0, kCntSlots * sizeof(uint32_t), s));
        MRT_LAUNCH(3, 0, launch_shade_primary(scene->dev, fp, *gbuffer, tp, bn, wb, smp, ctx->d_status, s));
        // bounces from tail_bounce on go through one persistent launch (not
        // while counting nodes: the counting kernels are the wavefront's)
        const uint32_t tail = ctx->counters ? 0u : ctx->tuning.tail_bounce;
        bool tail_done = false;
        for (uint32_t b = 1; b <= tp.max_bounces; ++b) {
            // The shadow rays of vertex b - 1 and the extension rays of
            // bounce b are independent (different queues; only the shadow
            // rays add radiance, and shade(b) after the join adds the next):
            // with overlap_shadow they run on two streams, so each fills the
            // GPU while the other drains.  Not before the path tail, whose
            // radiance additions must follow the shadow rays'.
            // tail_from_hits: bounce b is still traced by the wavefront
            // kernel and the tail starts from its hits (shading b onwards)
            const bool tail_from_hits = ctx->tuning.tail_from_hits != 0u;
            const bool tail_now = tail != 0u && b >= tail && !tail_from_hits;
            const bool overlap = nee && overlap_sh && !tail_now;
            // overlap_shadow 2: both queues in one persistent launch instead
            const bool merged = overlap && ctx->tuning.overlap_shadow == 2u;
            if (overlap && !merged) {
                MRT_CK(cudaEventRecord(ctx->ev_fork, s));
                MRT_CK(cudaStreamWaitEvent(ctx->side, ctx->ev_fork, 0));
                MRT_LAUNCH_ON(ctx->side, 2, int(b - 1),
                              launch_trace_shadow(scene->dev, wb, tp, b - 1, tblocks, ctx->d_status, ctx->counters,
                                                  dyn_sh, refill_min(ctx), ctx->side));
                MRT_CK(cudaEventRecord(ctx->ev_join, ctx->side));
            } else if (nee && !overlap) {
                MRT_LAUNCH(2, int(b - 1), launch_trace_shadow(scene->dev, wb, tp, b - 1, tblocks, ctx->d_status,
                                                              ctx->counters, dyn_sh, refill_min(ctx), s));
            }
            if (tail_now) {
                MRT_LAUNCH(1, int(b), launch_tail(scene->dev, tp, bn, wb, W, b, false, (ctx->tuning.tri_spread & 8u) != 0u,
                                                  tblocks, ctx->d_status, s));
                tail_done = true;
                break;
            }
            if (params->sort_rays || ctx->tuning.sort_min_rays != kSortNever) {
                MRT_LAUNCH(4, int(b), launch_sort_ext(scene->dev, wb, b,
                                                      params->sort_rays ? 0u : ctx->tuning.sort_min_rays, s));
                ctx->launches += 2;  // histogram, scan, scatter
            }
            if (merged)
                MRT_LAUNCH(1, int(b), launch_trace_merged(scene->dev, wb, tp, b, tblocks, ctx->d_status,
                                                          refill_min(ctx), s));
            else
                MRT_LAUNCH(1, int(b), launch_trace_ext(scene->dev, wb, b, tblocks, ctx->d_status, ctx->counters, dyn,
                                                       refill_min(ctx), s));
            if (overlap && !merged) MRT_CK(cudaStreamWaitEvent(s, ctx->ev_join, 0));
            if (tail != 0u && b >= tail) {  // (tail_from_hits)
                MRT_LAUNCH(1, int(b), launch_tail(scene->dev, tp, bn, wb, W, b, true, (ctx->tuning.tri_spread & 8u) != 0u,
                                                  tblocks, ctx->d_status, s));
                tail_done = true;
                break;
            }
            MRT_LAUNCH(3, int(b), launch_shade(scene->dev, tp, bn, wb, W, b, ctx->d_status, s));
        }
        if (nee && !tail_done)
            MRT_LAUNCH(2, int(tp.max_bounces),
                       launch_trace_shadow(scene->dev, wb, tp, tp.max_bounces, tblocks, ctx->d_status, ctx->counters,
                                           dyn_sh, refill_min(ctx), s));
        MRT_LAUNCH(3, 0, launch_tally(wb, s));
    }
    MRT_LAUNCH(3, 0, launch_finalize(wb, color, tp.samples, params->accumulate, params->frame_index, s));
#undef MRT_LAUNCH
#undef MRT_LAUNCH_ON
    return MRT_OK;
}

int mrt_cuda_cache_frame(mrt_ctx* ctx, mrt_cache* cache, const mrt_scene* scene, const mrt_gbuffer* gbuffer,
                         const mrt_camera_consts* consts, const mrt_trace_params* params, float* color, int train,
                         void* stream) {
    if (!ctx || !cache || !scene || !consts || !params || !color)
        return fail(ctx, MRT_EINVAL, "cache_frame: null argument");
    if (scene->kind != 0) return fail(ctx, MRT_EINVAL, "cache_frame: triangle scenes only");
    int rc = check_gbuffer(ctx, gbuffer);
    if (rc) return rc;
    if (!gbuffer->hit_t) return fail(ctx, MRT_EINVAL, "cache_frame: gbuffer hit_t required");
    if (!ctx->d_bn) return fail(ctx, MRT_ESTATE, "no blue-noise texture uploaded");
    if (params->rng_mode > MRT_RNG_PER_PIXEL || params->estimator > MRT_EST_NEE)
        return fail(ctx, MRT_EINVAL, "bad rng_mode or estimator");
    cudaSetDevice(ctx->device);
    cudaStream_t s = as_stream(stream);
    const uint32_t W = gbuffer->width, H = gbuffer->height;
    const FrameParams fp = frame_params(consts, W, H);
    TraceParams tp = trace_params(params);
    tp.atmo = sky_dev(ctx->sky, consts->camera_pos);
    const BlueNoise bn{ctx->d_bn, ctx->bn_w, ctx->bn_h};
    Scope total(ctx, s, 5, 0);
    // Training (its own paths, then the Adam steps) needs nothing of this
    // frame's rays and the rays need nothing of the cache until it is
    // queried: with overlap the training goes to the context's side stream
    // and the main stream waits for it just before the query is answered,
    // so the latency-bound training kernels and the ray tracing fill each
    // other's idle SMs.  Same image.
    const bool overlap_train = train && cache_overlap_training(cache);
    if (train) {
        cudaStream_t ts = s;
        if (overlap_train) {
            MRT_CK(cudaEventRecord(ctx->ev_fork, s));
            MRT_CK(cudaStreamWaitEvent(ctx->side, ctx->ev_fork, 0));
            ts = ctx->side;
        }
        Scope sc(ctx, ts, 6, 0);
        rc = cache_train_frame(ctx, cache, scene->dev, fp, tp, ctx->d_status, ts);
        if (rc) return rc;
    }
    if (overlap_train) MRT_CK(cudaEventRecord(ctx->ev_join, ctx->side));
    rc = ensure_wave(ctx, size_t(W) * H);
    if (rc) return rc;
    WaveBuffers& wb = ctx->wb;
    float *q = nullptr, *pred = nullptr;
    float4* pb = nullptr;
    rc = cache_frame_buffers(ctx, cache, wb.cap, &q, &pb, &pred);
    if (rc) return rc;
    tp.samples = 1;
    tp.max_bounces = 1;  // the path ends in the cache at the first bounce's hit
    const int tblocks = trace_blocks(ctx);
    const bool nee = tp.estimator == MRT_EST_NEE;
    const int dyn = fetch_mode(ctx, 0u), dyn_sh = fetch_mode(ctx, 1u);
#define MRT_LAUNCH(kind, bounce, expr)                                                                   \
    do {                                                                                                 \
        Scope sc_(ctx, s, kind, bounce);                                                                 \
        cudaError_t e_ = (expr);                                                                         \
        if (e_ != cudaSuccess) return fail(ctx, MRT_ECUDA, "%s: %s", #expr, cudaGetErrorString(e_));    \
        ctx->launches++;                                                                                 \
    } while (0)
    MRT_CK(cudaMemsetAsync(wb.counters, 0, kCntSlots * sizeof(uint32_t), s));
    if (cache_query_vertex(cache) == 0u) {
        // the cache supplies the indirect light at the primary hit
        tp.max_bounces = 0;
        MRT_LAUNCH(3, 0, launch_shade_primary(scene->dev, fp, *gbuffer, tp, bn, wb, 0, ctx->d_status, s));
        if (nee)
            MRT_LAUNCH(2, 0, launch_trace_shadow(scene->dev, wb, tp, 0, tblocks, ctx->d_status, ctx->counters, dyn_sh,
                                                 refill_min(ctx), s));
        const uint32_t npix = W * H;
        MRT_LAUNCH(3, 0, launch_cache_query_primary(scene->dev, fp, *gbuffer, q, pb, ctx->d_status, s));
        if (overlap_train) MRT_CK(cudaStreamWaitEvent(s, ctx->ev_join, 0));
        MRT_LAUNCH(7, 0, cache_infer(cache, q, npix, nullptr, pred, ctx->d_status, s));
        MRT_LAUNCH(3, 0, launch_cache_apply(wb, nullptr, npix, pred, pb, s));
    } else {
        // one diffuse bounce, then the cache supplies the indirect light at
        // that hit; both hits' direct light comes from shadow rays
        MRT_LAUNCH(3, 0, launch_shade_primary(scene->dev, fp, *gbuffer, tp, bn, wb, 0, ctx->d_status, s));
        if (nee)
            MRT_LAUNCH(2, 0, launch_trace_shadow(scene->dev, wb, tp, 0, tblocks, ctx->d_status, ctx->counters, dyn_sh,
                                                 refill_min(ctx), s));
        MRT_LAUNCH(1, 1, launch_trace_ext(scene->dev, wb, 1, tblocks, ctx->d_status, ctx->counters, dyn,
                                          refill_min(ctx), s));
        MRT_LAUNCH(3, 1, launch_shade(scene->dev, tp, bn, wb, W, 1, ctx->d_status, s));
        if (nee)
            MRT_LAUNCH(2, 1, launch_trace_shadow(scene->dev, wb, tp, 1, tblocks, ctx->d_status, ctx->counters, dyn_sh,
                                                 refill_min(ctx), s));
        MRT_LAUNCH(3, 1, launch_cache_query(scene->dev, tp, wb, q, pb, ctx->d_status, s));
        if (overlap_train) MRT_CK(cudaStreamWaitEvent(s, ctx->ev_join, 0));
        MRT_LAUNCH(7, 1, cache_infer(cache, q, uint32_t(wb.cap), wb.counters + kCntExt + 1, pred, ctx->d_status, s));
        MRT_LAUNCH(3, 1, launch_cache_apply(wb, wb.counters + kCntExt + 1, uint32_t(wb.cap), pred, pb, s));
    }
    MRT_LAUNCH(3, 0, launch_tally(wb, s));
    MRT_LAUNCH(3, 0, launch_finalize(wb, color, 1, params->accumulate, params->frame_index, s));
#undef MRT_LAUNCH
    return MRT_OK;
}

int mrt_cuda_trace_rays(mrt_ctx* ctx, const mrt_scene* scene, const mrt_ray* rays, uint32_t count, mrt_hit* hits,
                        uint32_t flags, void* stream) {
    if (!ctx || !scene || (count && (!rays || !hits))) return fail(ctx, MRT_EINVAL, "trace_rays: bad arguments");
    cudaSetDevice(ctx->device);
    cudaError_t e = launch_trace_rays(scene->dev, rays, count, hits, (flags & MRT_TRACE_ANY_HIT) != 0, nullptr,
                                      nullptr, ctx->d_status, as_stream(stream));
    if (e != cudaSuccess) return fail(ctx, MRT_ECUDA, "trace_rays launch: %s", cudaGetErrorString(e));
    ctx->launches++;
    return MRT_OK;
}

int mrt_cuda_trace_rays_counted(mrt_ctx* ctx, const mrt_scene* scene, const mrt_ray* rays, uint32_t count,
                                mrt_hit* hits, uint32_t* nodes_visited, uint32_t* tris_visited, void* stream) {
    if (!ctx || !scene || (count && (!rays || !hits || !nodes_visited || !tris_visited)) || scene->kind != 0)
        return fail(ctx, MRT_EINVAL, "trace_rays_counted: bad arguments");
    cudaSetDevice(ctx->device);
    cudaError_t e = launch_trace_rays(scene->dev, rays, count, hits, false, nodes_visited, tris_visited,
                                      ctx->d_status, as_stream(stream));
    if (e != cudaSuccess) return fail(ctx, MRT_ECUDA, "trace_rays_counted launch: %s", cudaGetErrorString(e));
    ctx->launches++;
    return MRT_OK;
}

} // extern "C"

namespace {

// The library-owned g-buffer of the host-buffer frame entry points, sized
// for width x height (reallocated when the size changes).
int frame_gbuffer(mrt_ctx* ctx, const mrt_scene* scene, uint32_t width, uint32_t height, mrt_gbuffer& g) {
    const size_t npix = size_t(width) * height;
    if (ctx->frame_pixels != npix) {
        cudaFree(ctx->d_vis); cudaFree(ctx->d_aux); cudaFree(ctx->d_t); cudaFree(ctx->d_color);
        ctx->d_vis = nullptr; ctx->d_aux = nullptr; ctx->d_t = nullptr; ctx->d_color = nullptr;
        ctx->frame_pixels = 0;
        MRT_CK(cudaMalloc(&ctx->d_vis, npix * sizeof(uint32_t)));
        MRT_CK(cudaMalloc(&ctx->d_aux, npix * (8 + 2)));
        MRT_CK(cudaMalloc(&ctx->d_t, npix * sizeof(float)));
        MRT_CK(cudaMalloc(&ctx->d_color, npix * 3 * sizeof(float)));
        MRT_CK(cudaMemset(ctx->d_color, 0, npix * 3 * sizeof(float)));
        ctx->frame_pixels = npix;
    }
    std::memset(&g, 0, sizeof(g));
    g.visibility = ctx->d_vis;
    g.hit_t = ctx->d_t;
    if (scene->kind == 1) {
        g.normal = static_cast<uint16_t*>(ctx->d_aux);
        g.depth = reinterpret_cast<uint16_t*>(static_cast<char*>(ctx->d_aux) + npix * 8);
    }
    g.width = width;
    g.height = height;
    return MRT_OK;
}

} // namespace

extern "C" {

int mrt_cuda_render_frame_host(mrt_ctx* ctx, const mrt_scene* scene, const mrt_camera_consts* consts,
                               const mrt_trace_params* params, uint32_t width, uint32_t height, uint32_t* visibility,
                               float* hit_t, float* color, void* stream) {
    if (!ctx || !scene || !consts || !params || !color || width == 0 || height == 0)
        return fail(ctx, MRT_EINVAL, "render_frame_host: bad arguments");
    cudaSetDevice(ctx->device);
    const size_t npix = size_t(width) * height;
    mrt_gbuffer g;
    int rc = frame_gbuffer(ctx, scene, width, height, g);
    if (rc) return rc;
    rc = mrt_cuda_primary_rays(ctx, scene, consts, &g, stream);
    if (rc) return rc;
    rc = mrt_cuda_secondary_rays(ctx, scene, &g, consts, params, ctx->d_color, stream);
    if (rc) return rc;
    cudaStream_t s = as_stream(stream);
    if (visibility) MRT_CK(cudaMemcpyAsync(visibility, ctx->d_vis, npix * 4, cudaMemcpyDeviceToHost, s));
    if (hit_t) MRT_CK(cudaMemcpyAsync(hit_t, ctx->d_t, npix * 4, cudaMemcpyDeviceToHost, s));
    MRT_CK(cudaMemcpyAsync(color, ctx->d_color, npix * 12, cudaMemcpyDeviceToHost, s));
    MRT_CK(cudaStreamSynchronize(s));
    return MRT_OK;
}

int mrt_cuda_render_frame_host_async(mrt_ctx* ctx, const mrt_scene* scene, const mrt_camera_consts* consts,
                                     const mrt_trace_params* params, uint32_t width, uint32_t height, float* color,
                                     void* stream) {
    if (!ctx || !scene || !consts || !params || !color || width == 0 || height == 0)
        return fail(ctx, MRT_EINVAL, "render_frame_host_async: bad arguments");
    if (params->accumulate)
        return fail(ctx, MRT_EINVAL, "render_frame_host_async: frames in flight do not accumulate");
    cudaSetDevice(ctx->device);
    const size_t npix = size_t(width) * height;
    mrt_gbuffer g;
    int rc = frame_gbuffer(ctx, scene, width, height, g);
    if (rc) return rc;
    if (!ctx->copy_stream) {
        MRT_CK(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
        for (int b = 0; b < 2; ++b) {
            MRT_CK(cudaEventCreateWithFlags(&ctx->ev_rendered[b], cudaEventDisableTiming));
            MRT_CK(cudaEventCreateWithFlags(&ctx->ev_copied[b], cudaEventDisableTiming));
        }
    }
    if (ctx->async_pixels != npix) {
        MRT_CK(cudaStreamSynchronize(ctx->copy_stream));
        for (int b = 0; b < 2; ++b) {
            cudaFree(ctx->d_color_async[b]);
            ctx->d_color_async[b] = nullptr;
        }
        ctx->async_pixels = 0;
        for (int b = 0; b < 2; ++b) MRT_CK(cudaMalloc(&ctx->d_color_async[b], npix * 3 * sizeof(float)));
        ctx->async_pixels = npix;
    }
    cudaStream_t s = as_stream(stream);
    const uint32_t b = ctx->async_next;
    ctx->async_next ^= 1u;
    // buffer b is free once the read-back of the frame before last is done
    MRT_CK(cudaStreamWaitEvent(s, ctx->ev_copied[b], 0));
    rc = mrt_cuda_primary_rays(ctx, scene, consts, &g, stream);
    if (rc) return rc;
    rc = mrt_cuda_secondary_rays(ctx, scene, &g, consts, params, ctx->d_color_async[b], stream);
    if (rc) return rc;
    MRT_CK(cudaEventRecord(ctx->ev_rendered[b], s));
    MRT_CK(cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_rendered[b], 0));
    MRT_CK(cudaMemcpyAsync(color, ctx->d_color_async[b], npix * 12, cudaMemcpyDeviceToHost, ctx->copy_stream));
    MRT_CK(cudaEventRecord(ctx->ev_copied[b], ctx->copy_stream));
    return MRT_OK;
}

int mrt_cuda_frames_wait(mrt_ctx* ctx) {
    if (!ctx) return MRT_EINVAL;
    cudaSetDevice(ctx->device);
    if (ctx->copy_stream) MRT_CK(cudaStreamSynchronize(ctx->copy_stream));
    return MRT_OK;
}

} // extern "C"
