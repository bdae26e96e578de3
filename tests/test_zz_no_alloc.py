"""The no-allocation primary-ray entry point.

mrt_cuda_primary_rays_noalloc serves callers that cannot call cudaMalloc
(an engine that owns every device byte, code inside a stream capture, a
plug-in host that forbids allocation): they hand in their own device
buffers -- scene, g-buffer and a status word -- and the entry point keeps
its scratch, the persistent kernel's work counter, in a fixed 256-byte
device array.  These tests call it through the C ABI twice in a row and
compare every g-buffer output bit for bit with the regular entry point,
mrt_cuda_primary_rays, and with the CPU oracle, the same bar the other
primary-ray tests use.  They pass alone in a fresh process and after the
rest of the suite (this file is collected last).
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from conftest import oracle_consts
from minotert_gb300._lib import MRT_EINVAL, MRT_ERANGE, MRT_OK, GBuffer as GB, lib, ptr
from minotert_gb300.pathtracer import Camera, Pathtracer, camera_consts
from minotert_gb300.scene import DeviceScene

pytestmark = pytest.mark.gpu

FIELDS = ("visibility", "hit_t", "depth", "normal", "motion")


def _gbuffer(ctx, w, h):
    n = w * h
    bufs = {"visibility": ctx.alloc(4 * n), "hit_t": ctx.alloc(4 * n), "depth": ctx.alloc(2 * n),
            "normal": ctx.alloc(8 * n), "motion": ctx.alloc(4 * n)}
    g = GB()
    for k, b in bufs.items():
        setattr(g, k, b.ptr)
    g.width, g.height = w, h
    return g, bufs


def _download(bufs, w, h):
    return {"visibility": bufs["visibility"].download(np.uint32, (h, w)),
            "hit_t": bufs["hit_t"].download(np.uint32, (h, w)),
            "depth": bufs["depth"].download(np.uint16, (h, w)),
            "normal": bufs["normal"].download(np.uint16, (h, w, 4)),
            "motion": bufs["motion"].download(np.uint16, (h, w, 2))}


def _device_free_bytes():
    """Free device memory as the CUDA driver reports it (cuMemGetInfo)."""
    cuda = C.CDLL("libcuda.so.1")
    free, total = C.c_size_t(0), C.c_size_t(0)
    assert cuda.cuMemGetInfo_v2(C.byref(free), C.byref(total)) == 0
    return free.value


def test_noalloc_primary_matches_regular_entry_point_and_oracle(ctx, hf_workload):
    wl, mesh, bvh = hf_workload
    W, H = wl.width, wl.height
    prev = Camera(wl.camera.viewport, wl.camera.verticalFov, wl.camera.nearPlane, (0.4, -26.5, 13.1),
                  wl.camera.yaw + 0.01, wl.camera.pitch)
    # the existing entry point, and the oracle on the same camera pair
    pt = Pathtracer(ctx, DeviceScene.triangles(ctx, mesh, bvh))
    ref = pt.primaryRays((W, H), wl.camera, prev).download()
    assert ctx.status() == 0
    ref["hit_t"] = ref["hit_t"].view(np.uint32)
    orc = oracle.primary(oracle_consts(wl.camera, 0, prev), W, H, bvh.nodes, bvh.tris, mesh.mats)
    orc["hit_t"] = orc["hit_t"].view(np.uint32)
    # the caller's own device buffers: scene, g-buffer, status word
    d_nodes, d_tris, d_mats = ctx.to_device(bvh.nodes), ctx.to_device(bvh.tris), ctx.to_device(mesh.mats)
    d_status = ctx.alloc(4)
    g, bufs = _gbuffer(ctx, W, H)
    consts = camera_consts(wl.camera, prev, 0)
    free_before = None
    for call in range(2):
        for b in bufs.values():
            lib().mrt_cuda_memset(ctx.handle, C.c_void_p(b.ptr), 0xA5, b.nbytes, None)  # stale contents
        d_status.zero()
        ctx.sync()
        if call == 1:
            free_before = _device_free_bytes()
        rc = lib().mrt_cuda_primary_rays_noalloc(ptr(d_nodes), len(bvh.nodes), ptr(d_tris), len(bvh.tris),
                                                  ptr(d_mats), len(mesh.mats), C.byref(consts), C.byref(g),
                                                  ptr(d_status), None)
        assert rc == MRT_OK
        ctx.sync()
        if call == 1:
            # the second call (the array and the kernel are loaded by now)
            # leaves the device's free memory as it was
            assert _device_free_bytes() == free_before
        out = _download(bufs, W, H)
        assert d_status.download(np.uint32, (1,))[0] == 0
        for k in FIELDS:
            assert np.array_equal(out[k], ref[k]), f"call {call}: {k} differs from mrt_cuda_primary_rays"
            assert np.array_equal(out[k], orc[k]), f"call {call}: {k} differs from the oracle"


def test_noalloc_rejects_a_missing_status_word_and_oversized_images(ctx, hf_workload):
    wl, mesh, bvh = hf_workload
    d_nodes, d_tris, d_mats = ctx.to_device(bvh.nodes), ctx.to_device(bvh.tris), ctx.to_device(mesh.mats)
    d_status = ctx.alloc(4)
    g, _bufs = _gbuffer(ctx, wl.width, wl.height)
    consts = camera_consts(wl.camera)
    # without a status word, traversal errors could not be reported
    rc = lib().mrt_cuda_primary_rays_noalloc(ptr(d_nodes), len(bvh.nodes), ptr(d_tris), len(bvh.tris), ptr(d_mats),
                                              len(mesh.mats), C.byref(consts), C.byref(g), None, None)
    assert rc == MRT_EINVAL
    big = GB()
    vis = ctx.alloc(4)
    big.visibility, big.width, big.height = vis.ptr, 1 << 14, 1 << 13  # 2^27 pixels > 2^26
    consts = camera_consts(Camera.reference(big.width, big.height))
    rc = lib().mrt_cuda_primary_rays_noalloc(ptr(d_nodes), len(bvh.nodes), ptr(d_tris), len(bvh.tris), ptr(d_mats),
                                              len(mesh.mats), C.byref(consts), C.byref(big), ptr(d_status), None)
    assert rc == MRT_ERANGE
