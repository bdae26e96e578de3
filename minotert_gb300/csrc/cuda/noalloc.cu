// mrt_cuda_primary_rays_noalloc: primary rays without any device allocation,
// for callers that cannot call cudaMalloc (an engine that owns all device
// memory, code inside a stream capture, a plug-in host that forbids
// allocation).  The persistent primary-ray kernel needs scratch memory
// beyond its inputs and outputs -- a work counter -- and here that scratch
// is the file-scope device array below instead of a context allocation.
#include "internal.hpp"

#include <cuda.h>  // CUcontext (the driver calls are fetched through the runtime)

#include <mutex>

namespace mrt {
FrameParams make_frame_params(const mrt_camera_consts* c, uint32_t w, uint32_t h);
}

namespace {

// [0]: work counter of the persistent kernel; the rest is reserved.
// 256 bytes per GPU, kept until exit.
constexpr int kScratchWords = 64;
static __device__ __align__(256) uint32_t g_noalloc_scratch[kScratchWords];

// Set-up of one CUDA context: the device address of that context's copy
// of the array (host code may not use the symbol itself -- on the host it
// is a stand-in, not a device address) and the persistent grid size.
// Entries are keyed by the context's process-unique id (cuCtxGetId), so a
// context created after a device reset, or a caller's own driver-API
// context on the same device, gets its own look-up instead of an address
// that belongs to another context.
struct ContextSetup {
    unsigned long long ctx_id = 0;  // 0: free slot
    uint32_t* scratch = nullptr;
    int blocks = 0;
};
constexpr int kMaxContexts = 64;
std::mutex g_setup_mutex;
ContextSetup g_setup[kMaxContexts];
int g_next_slot = 0;

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

// Driver entry points through the runtime (the library does not link
// libcuda directly).  Called with g_setup_mutex held.
bool driver_entry_points() {
    if (g_ctx_get_current && g_ctx_get_id) return true;
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 4000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !f) {
        cudaGetLastError();
        return false;
    }
    g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !f) {
        cudaGetLastError();
        g_ctx_get_current = nullptr;
        return false;
    }
    g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f);
    return true;
}

// Id of the calling thread's current context; 0 when there is none yet
// (or it was destroyed).
unsigned long long current_context_id() {
    CUcontext c = nullptr;
    if (g_ctx_get_current(&c) != CUDA_SUCCESS || !c) return 0;
    unsigned long long id = 0;
    if (g_ctx_get_id(c, &id) != CUDA_SUCCESS) return 0;
    return id;
}

int setup_context(int dev, ContextSetup& out) {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!driver_entry_points()) return MRT_ECUDA;
    unsigned long long id = current_context_id();
    if (id) {
        for (const ContextSetup& s : g_setup)
            if (s.ctx_id == id) {
                out = s;
                return MRT_OK;
            }
    }
    // First call in this context: look up its copy of the array.  This
    // also makes the runtime's primary context current when the thread has
    // no context yet.
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
        cudaGetLastError();
        return MRT_ECUDA;
    }
    id = current_context_id();
    if (!id) return MRT_ECUDA;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) {
        cudaGetLastError();
        return MRT_ECUDA;
    }
    ContextSetup s;
    s.ctx_id = id;
    s.scratch = static_cast<uint32_t*>(p);
    s.blocks = mrt::trace_blocks_per_sm() * sms;
    g_setup[g_next_slot] = s;  // oldest entry replaced once all slots are used
    g_next_slot = (g_next_slot + 1) % kMaxContexts;
    out = s;
    return MRT_OK;
}

} // namespace

extern "C" int mrt_cuda_primary_rays_noalloc(const mrt_bvh8_node* nodes, uint32_t node_count, const mrt_tri* tris,
                                             uint32_t tri_count, const mrt_material* materials,
                                             uint32_t material_count, const mrt_camera_consts* consts,
                                             const mrt_gbuffer* gbuffer, uint32_t* status, void* stream) {
    if (!nodes || !tris || !materials || !consts || !gbuffer || !gbuffer->visibility || !status || node_count == 0 ||
        tri_count == 0 || material_count == 0 || gbuffer->width == 0 || gbuffer->height == 0)
        return MRT_EINVAL;
    if (uint64_t(gbuffer->width) * gbuffer->height > uint64_t(MRT_NOALLOC_MAX_PIXELS)) return MRT_ERANGE;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return MRT_ECUDA;
    }
    ContextSetup s;
    int rc = setup_context(dev, s);
    if (rc != MRT_OK) return rc;

    mrt::DevScene sc{};
    sc.nodes = reinterpret_cast<const uint4*>(nodes);
    sc.tris = reinterpret_cast<const float4*>(tris);
    sc.mats = materials;
    sc.spheres = nullptr;
    sc.node_count = node_count;
    sc.tri_count = tri_count;
    sc.mat_count = material_count;
    sc.sphere_count = 0;
    const mrt::FrameParams fp = mrt::make_frame_params(consts, gbuffer->width, gbuffer->height);
    // the launcher clears the work counter (scratch[0]) on the stream first
    cudaError_t e = mrt::launch_primary_tri(sc, fp, *gbuffer, status, nullptr, s.scratch, s.blocks, false, 1u,
                                           static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return MRT_ECUDA;
    return MRT_OK;
}
