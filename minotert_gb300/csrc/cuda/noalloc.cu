// mrt_cuda_primary_rays_noalloc: primary rays without any device allocation,
// for callers that cannot call cudaMalloc (an engine that owns all device
// memory, code inside a stream capture, a plug-in host that forbids
// allocation).  The persistent primary-ray kernel needs scratch memory
// beyond its inputs and outputs -- a work counter and a status word -- and
// here that scratch is the file-scope device array below instead of a
// context allocation.
#include "internal.hpp"

#include <mutex>

namespace mrt {
FrameParams make_frame_params(const mrt_camera_consts* c, uint32_t w, uint32_t h);
}

namespace {

// [0]: work counter of the persistent kernel, [1]: status word used when
// the caller passes no status buffer.  256 bytes per GPU, kept until exit.
constexpr int kScratchWords = 64;
static __device__ __align__(256) uint32_t g_noalloc_scratch[kScratchWords];

// Per-device set-up: the device address of this device's copy of the
// array (host code may not use the symbol itself -- on the host it is a
// stand-in, not a device address) and the persistent grid size.
struct DeviceSetup {
    uint32_t* scratch = nullptr;
    int blocks = 0;
};
constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
DeviceSetup g_setup[kMaxDevices];

int setup_device(int dev, DeviceSetup& out) {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    DeviceSetup& s = g_setup[dev];
    if (!s.scratch) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return MRT_ECUDA;
        }
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) {
            cudaGetLastError();
            return MRT_ECUDA;
        }
        s.blocks = mrt::trace_blocks_per_sm() * sms;
        s.scratch = static_cast<uint32_t*>(p);
    }
    out = s;
    return MRT_OK;
}

} // namespace

extern "C" int mrt_cuda_primary_rays_noalloc(const mrt_bvh8_node* nodes, uint32_t node_count, const mrt_tri* tris,
                                             uint32_t tri_count, const mrt_material* materials,
                                             uint32_t material_count, const mrt_camera_consts* consts,
                                             const mrt_gbuffer* gbuffer, uint32_t* status, void* stream) {
    if (!nodes || !tris || !materials || !consts || !gbuffer || !gbuffer->visibility || node_count == 0 ||
        tri_count == 0 || material_count == 0 || gbuffer->width == 0 || gbuffer->height == 0)
        return MRT_EINVAL;
    if (uint64_t(gbuffer->width) * gbuffer->height > uint64_t(MRT_NOALLOC_MAX_PIXELS)) return MRT_ERANGE;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return MRT_ECUDA;
    }
    if (dev < 0 || dev >= kMaxDevices) return MRT_ERANGE;
    DeviceSetup s;
    int rc = setup_device(dev, s);
    if (rc != MRT_OK) return rc;

    cudaStream_t st = static_cast<cudaStream_t>(stream);
    uint32_t* stat = status;
    if (!stat) {
        stat = s.scratch + 1;
        if (cudaMemsetAsync(stat, 0, sizeof(uint32_t), st) != cudaSuccess) {
            cudaGetLastError();
            return MRT_ECUDA;
        }
    }
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
    // the launcher clears the work counter (scratch[0]) on `st` first
    cudaError_t e = mrt::launch_primary_tri(sc, fp, *gbuffer, stat, nullptr, s.scratch, s.blocks, false, 1u,
                                           st);
    if (e != cudaSuccess) return MRT_ECUDA;
    return MRT_OK;
}
