"""GPU parity: the CUDA path (through the mrt_cuda C ABI) against the CPU
oracle on the same seeded scenes, cameras and rays.

Bars: triangle ids and FP32 hit t bit-identical (integer/index work and the
same IEEE operation sequence on both sides); g-buffer formats bit-identical;
path-traced colour within the tolerances stated per test (the only
non-reproducible operation is sincosf in the sphere-point sampler).
"""
import math

import numpy as np
import pytest

import oracle
from conftest import oracle_consts, random_rays
from minotert_gb300._lib import (HIT_DTYPE, MRT_EINVAL, MRT_MISS, MRT_STATUS_BAD_NODE, MRT_STATUS_BAD_TRI, RAY_DTYPE,
                                 lib, ptr)
from minotert_gb300.pathtracer import Camera, Pathtracer, Sky, TraceSettings, camera_consts
from minotert_gb300.scene import DeviceScene, reference_spheres

pytestmark = pytest.mark.gpu


def _trace(ctx, dscene, rays, any_hit=False, counted=False):
    n = len(rays)
    d_rays = ctx.to_device(rays)
    d_hits = ctx.alloc(8 * max(n, 1))
    if counted:
        d_nv, d_tv = ctx.alloc(4 * max(n, 1)), ctx.alloc(4 * max(n, 1))
        ctx.check(lib().mrt_cuda_trace_rays_counted(ctx.handle, dscene.handle, ptr(d_rays), n, ptr(d_hits),
                                                    ptr(d_nv), ptr(d_tv), None), "counted")
        return (d_hits.download(HIT_DTYPE, (n,)), d_nv.download(np.uint32, (n,)), d_tv.download(np.uint32, (n,)))
    ctx.check(lib().mrt_cuda_trace_rays(ctx.handle, dscene.handle, ptr(d_rays), n, ptr(d_hits), int(any_hit), None),
              "trace")
    return d_hits.download(HIT_DTYPE, (n,))


@pytest.fixture(scope="module")
def hf_scene(ctx, hf_workload):
    wl, mesh, bvh = hf_workload
    return DeviceScene.triangles(ctx, mesh, bvh)


@pytest.fixture(scope="module")
def ico_scene(ctx, ico_workload):
    wl, mesh, bvh = ico_workload
    return DeviceScene.triangles(ctx, mesh, bvh)


def test_primary_triangles_bit_exact(ctx, hf_workload, hf_scene):
    wl, mesh, bvh = hf_workload
    prev = Camera(wl.camera.viewport, wl.camera.verticalFov, wl.camera.nearPlane, (0.5, -27.0, 13.2),
                  wl.camera.yaw - 0.02, wl.camera.pitch)
    pt = Pathtracer(ctx, hf_scene)
    g = pt.primaryRays((wl.width, wl.height), wl.camera, prev).download()
    assert ctx.status() == 0
    ref = oracle.primary(oracle_consts(wl.camera, 0, prev), wl.width, wl.height, bvh.nodes, bvh.tris, mesh.mats)
    assert np.array_equal(g["visibility"], ref["visibility"])
    assert np.array_equal(g["hit_t"].view(np.uint32), ref["hit_t"].view(np.uint32))
    assert np.array_equal(g["depth"], ref["depth"])
    assert np.array_equal(g["normal"], ref["normal"])
    assert np.array_equal(g["motion"], ref["motion"])
    assert 0.3 < (g["visibility"] != MRT_MISS).mean() <= 1.0


@pytest.mark.parametrize("size", [(1, 1), (17, 13), (64, 200)])
def test_primary_odd_sizes(ctx, hf_workload, hf_scene, size):
    wl, mesh, bvh = hf_workload
    cam = Camera(size, wl.camera.verticalFov, wl.camera.nearPlane, wl.camera.position, wl.camera.yaw,
                 wl.camera.pitch)
    g = Pathtracer(ctx, hf_scene, full_gbuffer=False).primaryRays(size, cam, cam).download()
    ref = oracle.primary(oracle_consts(cam), size[0], size[1], bvh.nodes, bvh.tris, mesh.mats)
    assert np.array_equal(g["visibility"], ref["visibility"])
    assert np.array_equal(g["hit_t"].view(np.uint32), ref["hit_t"].view(np.uint32))


def test_primary_reference_spheres(ctx):
    # scene 0 (scene.glsl:4-11) through primaryRay.comp semantics
    spheres = reference_spheres()
    ds = DeviceScene.from_spheres(ctx, spheres)
    cam = Camera.reference(192, 108)
    g = Pathtracer(ctx, ds).primaryRays((192, 108), cam, cam).download()
    ref = oracle.primary(oracle_consts(cam), 192, 108, spheres=spheres)
    assert np.array_equal(g["visibility"], ref["visibility"])
    hit = g["visibility"] != MRT_MISS
    assert hit.mean() > 0.2
    assert np.array_equal(g["depth"][hit], ref["depth"][hit])
    assert np.array_equal(g["normal"], ref["normal"])


def test_secondary_reference_spheres(ctx, blue_noise):
    # secondaryRays.comp: 8 samples x 8 bounces, same PCG seed everywhere,
    # blue-noise rotation, throughput x albedo, constant sky on escape
    spheres = reference_spheres()
    ds = DeviceScene.from_spheres(ctx, spheres)
    W, H = 160, 90
    cam = Camera.reference(W, H)
    pt = Pathtracer(ctx, ds)
    pt.frame_counter = 5
    gb = pt.primaryRays((W, H), cam, cam)
    sky = Sky(radiance=(0.6, 0.7, 1.0), sun_dir=None)
    col = pt.secondaryRays(gb, cam, sky, blue_noise, TraceSettings(samples=8, bounces=8))
    img = col.download(np.float32, (H, W, 3))
    g = gb.download()
    p = oracle.params_array(8, 8, sky=sky.radiance)
    ref = oracle.secondary_spheres(spheres, oracle_consts(cam, 5), W, H, g["visibility"], g["depth"], g["normal"],
                                   blue_noise, p)
    assert np.isfinite(img).all()
    close = np.isclose(img, ref, rtol=1e-4, atol=1e-6).all(axis=2)
    assert close.mean() > 0.99
    assert np.sqrt(np.mean((img - ref) ** 2)) < 1e-2 * ref.mean()


def test_trace_rays_random_vs_brute_force(ctx, hf_workload, hf_scene):
    wl, mesh, bvh = hf_workload
    rays = random_rays(50000, mesh.lo, mesh.hi, seed=11)
    hits = _trace(ctx, hf_scene, rays)
    ref = oracle.trace_brute(mesh.verts, rays)
    assert np.array_equal(hits["prim"], ref["prim"])
    assert np.array_equal(hits["t"].view(np.uint32), ref["t"].view(np.uint32))
    any_hits = _trace(ctx, hf_scene, rays, any_hit=True)
    assert np.array_equal(any_hits["prim"] == MRT_MISS, ref["prim"] == MRT_MISS)
    assert ctx.status() == 0


def test_trace_rays_tmin_tmax_and_empty(ctx, hf_workload, hf_scene):
    wl, mesh, bvh = hf_workload
    rays = random_rays(5000, mesh.lo, mesh.hi, seed=12)
    full = oracle.trace_brute(mesh.verts, rays)
    rays["tmax"] = np.where(full["prim"] != MRT_MISS, full["t"], np.float32(np.inf))  # t < tmax excludes the hit
    hits = _trace(ctx, hf_scene, rays, any_hit=True)
    ref = oracle.trace_brute(mesh.verts, rays, any_hit=True)
    assert np.array_equal(hits["prim"] == MRT_MISS, ref["prim"] == MRT_MISS)
    empty = _trace(ctx, hf_scene, rays[:0])
    assert len(empty) == 0


def test_traversal_counters_match_oracle(ctx, hf_workload, hf_scene):
    wl, mesh, bvh = hf_workload
    rays = random_rays(20000, mesh.lo, mesh.hi, seed=13)
    hits, nv, tv = _trace(ctx, hf_scene, rays, counted=True)
    ref, st, rnv, rtv = oracle.trace_bvh8(bvh.nodes, bvh.tris, rays, counts=True)
    assert np.array_equal(hits["prim"], ref["prim"])
    assert np.array_equal(nv, rnv) and np.array_equal(tv, rtv)


def test_primary_icospheres_full_size_bit_exact(ctx, ico_workload, ico_scene):
    # 1,034,240 triangles, 1920x1080 primary rays
    wl, mesh, bvh = ico_workload
    g = Pathtracer(ctx, ico_scene, full_gbuffer=False).primaryRays((wl.width, wl.height), wl.camera,
                                                                   wl.camera).download()
    assert ctx.status() == 0
    ref = oracle.primary(oracle_consts(wl.camera), wl.width, wl.height, bvh.nodes, bvh.tris, mesh.mats)
    assert np.array_equal(g["visibility"], ref["visibility"])
    assert np.array_equal(g["hit_t"].view(np.uint32), ref["hit_t"].view(np.uint32))


def test_incoherent_rays_icospheres_vs_oracle(ctx, ico_workload, ico_scene):
    wl, mesh, bvh = ico_workload
    rays = random_rays(200000, mesh.lo * 0.5, mesh.hi * 0.5, seed=14, margin=0.0)
    hits = _trace(ctx, ico_scene, rays)
    ref, st = oracle.trace_bvh8(bvh.nodes, bvh.tris, rays)
    assert np.array_equal(hits["prim"], ref["prim"])
    assert np.array_equal(hits["t"].view(np.uint32), ref["t"].view(np.uint32))
    # and the BVH result equals brute force on a subset
    sub = rays[:300]
    assert np.array_equal(oracle.trace_brute(mesh.verts, sub)["prim"], hits["prim"][:300])


def _pathtrace_gpu(ctx, wl, dscene, bn, frame=0, frames=1, settings=None):
    pt = Pathtracer(ctx, dscene, full_gbuffer=False)
    color = ctx.alloc(12 * wl.width * wl.height)
    for f in range(frames):
        pt.frame_counter = frame + f
        gb = pt.primaryRays((wl.width, wl.height), wl.camera, wl.camera)
        s = settings or wl.settings
        s = TraceSettings(s.samples, s.bounces, s.rr_start, s.rng_mode, frames > 1, f, s.sort_rays, s.exact_trig)
        pt.secondaryRays(gb, wl.camera, wl.sky, bn, s, color=color)
    return color.download(np.float32, (wl.height, wl.width, 3)), gb.download()


def _oracle_params(wl, frame_index=0, accumulate=0, samples=None, bounces=None):
    sd = np.asarray(wl.sky.sun_dir, np.float64)
    sd = (sd / np.linalg.norm(sd)).astype(np.float32)
    s = wl.settings
    return oracle.params_array(samples or s.samples, s.bounces if bounces is None else bounces, s.rr_start,
                               s.rng_mode, 1, accumulate, frame_index, sun=sd, sun_e=wl.sky.sun_irradiance,
                               sky=wl.sky.radiance)


def test_pathtrace_heightfield_vs_oracle_fp32(ctx, hf_workload, hf_scene, blue_noise):
    wl, mesh, bvh = hf_workload
    img, g = _pathtrace_gpu(ctx, wl, hf_scene, blue_noise)
    assert ctx.status() == 0
    ref, counts, st = oracle.pathtrace(bvh.nodes, bvh.tris, mesh.mats, oracle_consts(wl.camera), wl.width, wl.height,
                                       g["visibility"], g["hit_t"], blue_noise, _oracle_params(wl))
    assert np.isfinite(img).all() and (img >= 0).all()
    same = np.isclose(img, ref, rtol=1e-5, atol=1e-6).all(axis=2)
    assert same.mean() > 0.995
    assert np.sqrt(np.mean((img - ref) ** 2)) < 1e-3 * max(ref.mean(), 1e-3) * 30


def test_pathtrace_converged_vs_fp64(ctx, hf_workload, hf_scene, blue_noise):
    # 16 accumulated frames (running mean) against the FP64 oracle on the
    # same frames, rows 64..128; RMSE bar 1% of the mean radiance
    wl, mesh, bvh = hf_workload
    frames = 16
    img, g = _pathtrace_gpu(ctx, wl, hf_scene, blue_noise, frames=frames)
    y0, y1 = 64, 128
    ref = np.zeros_like(img)
    for f in range(frames):
        oracle.pathtrace(bvh.nodes, bvh.tris, mesh.mats, oracle_consts(wl.camera, f), wl.width, wl.height,
                         g["visibility"], g["hit_t"], blue_noise, _oracle_params(wl, f, 1), precision=64, y0=y0,
                         y1=y1, color=ref)
    a, b = img[y0:y1], ref[y0:y1]
    rmse = float(np.sqrt(np.mean((a - b) ** 2)))
    assert rmse < 0.01 * float(b.mean())


def test_pathtrace_icospheres_rows_vs_oracle(ctx, ico_workload, ico_scene, blue_noise):
    wl, mesh, bvh = ico_workload
    img, g = _pathtrace_gpu(ctx, wl, ico_scene, blue_noise)
    assert ctx.status() == 0
    assert np.isfinite(img).all() and (img >= 0).all()
    y0, y1 = 500, 532
    ref, counts, st = oracle.pathtrace(bvh.nodes, bvh.tris, mesh.mats, oracle_consts(wl.camera), wl.width, wl.height,
                                       g["visibility"], g["hit_t"], blue_noise, _oracle_params(wl), y0=y0, y1=y1)
    a, b = img[y0:y1], ref[y0:y1]
    same = np.isclose(a, b, rtol=1e-5, atol=1e-6).all(axis=2)
    assert same.mean() > 0.98
    assert np.sqrt(np.mean((a - b) ** 2)) < 0.05 * b.mean()


def _exact(wl):
    s = wl.settings
    return TraceSettings(s.samples, s.bounces, s.rr_start, s.rng_mode, exact_trig=True)


def _bit_mismatch(a, b):
    """Pixels whose RGB differs from the oracle's in any bit."""
    return int((a.view(np.uint32) != b.view(np.uint32)).any(axis=-1).sum())


def test_pathtrace_heightfield_bit_exact_with_exact_trig(ctx, hf_workload, hf_scene, blue_noise):
    # with the sphere-point sampler's sin/cos in binary64 (the oracle's
    # evaluation) the whole estimator is bit-identical to the FP32 oracle
    wl, mesh, bvh = hf_workload
    img, g = _pathtrace_gpu(ctx, wl, hf_scene, blue_noise, settings=_exact(wl))
    assert ctx.status() == 0
    ref, counts, st = oracle.pathtrace(bvh.nodes, bvh.tris, mesh.mats, oracle_consts(wl.camera), wl.width, wl.height,
                                       g["visibility"], g["hit_t"], blue_noise, _oracle_params(wl))
    assert st == 0
    assert _bit_mismatch(img, ref) == 0


def test_pathtrace_icospheres_rows_bit_exact_with_exact_trig(ctx, ico_workload, ico_scene, blue_noise):
    # the headline estimator (4 bounces, Russian roulette after bounce 2,
    # a shadow ray per vertex) on 1,034,240 triangles, 64 rows x 1920:
    # bit-identical colour.  The one difference the evaluation admits -- a
    # binary64 sine or cosine within a few binary64 ulps of a binary32
    # rounding boundary, about 1e-8 of calls -- does not occur on these
    # inputs, and the inputs are fixed
    wl, mesh, bvh = ico_workload
    img, g = _pathtrace_gpu(ctx, wl, ico_scene, blue_noise, frame=5, settings=_exact(wl))
    assert ctx.status() == 0
    y0, y1 = 480, 544
    ref, counts, st = oracle.pathtrace(bvh.nodes, bvh.tris, mesh.mats, oracle_consts(wl.camera, 5), wl.width,
                                       wl.height, g["visibility"], g["hit_t"], blue_noise, _oracle_params(wl),
                                       y0=y0, y1=y1)
    assert st == 0
    bad = _bit_mismatch(img[y0:y1], ref[y0:y1])
    print(f"pixels differing from the FP32 oracle: {bad} of {(y1 - y0) * wl.width}")
    assert bad == 0


def test_pathtrace_icospheres_converged_vs_fp64(ctx, ico_workload, ico_scene, blue_noise):
    # the headline estimator accumulated over 32 frames (running mean, the
    # default sincosf sampler) against the FP64 oracle over the same frames
    # and random numbers on 128 rows x 1920 pixels.  Bar: RMSE below 1 % of
    # the mean radiance of the band (measured: 0.60 %; the FP32 and FP64
    # paths part where a hit, a miss or a roulette decision flips, and such
    # differences average down as frames accumulate)
    wl, mesh, bvh = ico_workload
    frames = 32
    img, g = _pathtrace_gpu(ctx, wl, ico_scene, blue_noise, frames=frames)
    assert ctx.status() == 0
    y0, y1 = 448, 576
    ref = np.zeros_like(img)
    for f in range(frames):
        _, _, st = oracle.pathtrace(bvh.nodes, bvh.tris, mesh.mats, oracle_consts(wl.camera, f), wl.width, wl.height,
                                    g["visibility"], g["hit_t"], blue_noise, _oracle_params(wl, f, 1), precision=64,
                                    y0=y0, y1=y1, color=ref)
        assert st == 0
    a, b = img[y0:y1].astype(np.float64), ref[y0:y1].astype(np.float64)
    rmse = float(np.sqrt(np.mean((a - b) ** 2)))
    print(f"32-frame RMSE vs FP64: {rmse:.3e} ({rmse / b.mean():.2e} of the mean {b.mean():.4f})")
    assert rmse < 0.01 * float(b.mean())


def test_frame_stats_count_rays(ctx, ico_workload, ico_scene, blue_noise):
    wl, mesh, bvh = ico_workload
    ctx.set_timing(True)
    ctx.frame_stats()
    _pathtrace_gpu(ctx, wl, ico_scene, blue_noise)
    st = ctx.frame_stats()
    ctx.set_timing(False)
    npix = wl.width * wl.height
    assert st.primary_rays == npix
    ext = list(st.extension_rays[:4])
    assert 0 < ext[0] <= npix and all(ext[i + 1] <= ext[i] for i in range(3))
    assert st.extension_rays[4] == 0
    assert 0 < st.shadow_rays <= 5 * npix
    assert st.ms_extend > 0 and st.ms_primary > 0 and st.ms_total > 0
    assert st.launches > 8


def test_render_frame_host_matches_passes(ctx, hf_workload, hf_scene, blue_noise):
    wl, mesh, bvh = hf_workload
    img, g = _pathtrace_gpu(ctx, wl, hf_scene, blue_noise, frame=3)
    consts = camera_consts(wl.camera, wl.camera, 3)
    params = wl.settings.params(wl.sky)
    vis = np.zeros((wl.height, wl.width), np.uint32)
    ht = np.zeros((wl.height, wl.width), np.float32)
    col = np.zeros((wl.height, wl.width, 3), np.float32)
    import ctypes as C
    ctx.check(lib().mrt_cuda_render_frame_host(ctx.handle, hf_scene.handle, C.byref(consts), C.byref(params),
                                               wl.width, wl.height, ptr(vis), ptr(ht), ptr(col), None), "frame")
    assert np.array_equal(vis, g["visibility"])
    assert np.array_equal(col, img)


def test_render_frame_host_async_matches_blocking(ctx, hf_workload, hf_scene, blue_noise):
    # frames in flight (two colour buffers, read-backs on the context's copy
    # stream) give each frame the same image as the blocking entry point
    import ctypes as C
    wl, mesh, bvh = hf_workload
    params = wl.settings.params(wl.sky)
    params.accumulate = 0
    frames = (3, 4, 5)
    ref = {}
    for f in frames:
        col = np.zeros((wl.height, wl.width, 3), np.float32)
        consts = camera_consts(wl.camera, wl.camera, f)
        ctx.check(lib().mrt_cuda_render_frame_host(ctx.handle, hf_scene.handle, C.byref(consts), C.byref(params),
                                                   wl.width, wl.height, None, None, ptr(col), None), "frame")
        ref[f] = col
    out = {f: ctx.host_alloc((wl.height, wl.width, 3), np.float32) for f in frames}
    stream = ctx.stream()
    for f in frames:
        consts = camera_consts(wl.camera, wl.camera, f)
        ctx.check(lib().mrt_cuda_render_frame_host_async(ctx.handle, hf_scene.handle, C.byref(consts),
                                                         C.byref(params), wl.width, wl.height, ptr(out[f]),
                                                         C.c_void_p(stream)), "frame_async")
    ctx.check(lib().mrt_cuda_frames_wait(ctx.handle), "frames_wait")
    assert ctx.status() == 0
    for f in frames:
        assert np.array_equal(np.asarray(out[f]), ref[f]), f
    params.accumulate = 1
    consts = camera_consts(wl.camera, wl.camera, 6)
    rc = lib().mrt_cuda_render_frame_host_async(ctx.handle, hf_scene.handle, C.byref(consts), C.byref(params),
                                                wl.width, wl.height, ptr(out[3]), C.c_void_p(stream))
    assert rc == MRT_EINVAL


def test_corrupt_bvh_reports_status_not_hang(ctx, hf_workload, blue_noise):
    # host-side fault injection: corrupted child / triangle indices must end
    # in a status flag (bounds-checked traversal, iteration cap), the
    # context stays usable
    wl, mesh, bvh = hf_workload
    from minotert_gb300.scene import Bvh8
    nodes = bvh.nodes.copy()
    nodes["child_base"][0] = len(nodes) + 1000
    bad = DeviceScene.triangles(ctx, mesh, Bvh8(nodes, bvh.tris, bvh.depth, bvh.leaf_count, 0.0))
    rays = random_rays(4096, mesh.lo, mesh.hi, seed=15)
    _trace(ctx, bad, rays)
    ctx.sync(timeout_s=30.0)
    assert ctx.status() & MRT_STATUS_BAD_NODE
    nodes = bvh.nodes.copy()
    nodes["tri_base"][:] = len(bvh.tris) + 7
    bad2 = DeviceScene.triangles(ctx, mesh, Bvh8(nodes, bvh.tris, bvh.depth, bvh.leaf_count, 0.0))
    _trace(ctx, bad2, rays)
    ctx.sync(timeout_s=30.0)
    assert ctx.status() & MRT_STATUS_BAD_TRI
    # self-referencing child: the iteration cap ends it
    nodes = bvh.nodes.copy()
    nodes["child_base"][:] = 0
    bad3 = DeviceScene.triangles(ctx, mesh, Bvh8(nodes, bvh.tris, bvh.depth, bvh.leaf_count, 0.0))
    _trace(ctx, bad3, rays)
    ctx.sync(timeout_s=30.0)
    assert ctx.status() != 0
    # the context still works
    good = _trace(ctx, DeviceScene.triangles(ctx, mesh, bvh), rays)
    assert ctx.status() == 0
    assert np.array_equal(good["prim"], oracle.trace_brute(mesh.verts, rays)["prim"])


def test_errors_are_codes_not_crashes(ctx, hf_scene):
    import ctypes as C
    from minotert_gb300._lib import MRT_EINVAL, MRT_ESTATE, GBuffer as GB, TraceParams as TP, Context
    g = GB()
    rc = lib().mrt_cuda_primary_rays(ctx.handle, hf_scene.handle, None, C.byref(g), None)
    assert rc == MRT_EINVAL
    assert b"null" in lib().mrt_cuda_last_error(ctx.handle)
    fresh = Context(0)
    vis = fresh.alloc(4)
    t = fresh.alloc(4)
    g.visibility, g.hit_t, g.width, g.height = vis.ptr, t.ptr, 1, 1
    p = TP()
    p.samples, p.max_bounces = 1, 1
    consts = camera_consts(Camera.reference(1, 1))
    sc = DeviceScene.triangles(fresh, hf_scene.mesh, hf_scene.bvh)
    out = fresh.alloc(12)
    rc = lib().mrt_cuda_secondary_rays(fresh.handle, sc.handle, C.byref(g), C.byref(consts), C.byref(p),
                                       C.c_void_p(out.ptr), None)
    assert rc == MRT_ESTATE  # no blue noise uploaded yet
    p.max_bounces = 99
    fresh.blue_noise(np.zeros((4, 4, 4), np.uint8))
    rc = lib().mrt_cuda_secondary_rays(fresh.handle, sc.handle, C.byref(g), C.byref(consts), C.byref(p),
                                       C.c_void_p(out.ptr), None)
    assert rc != 0


@pytest.mark.parametrize("dyn,prim,blocks,spread,rmin", [(0, 0, 0, 0, 1), (1, 1, 0, 0, 1), (1, 0, 2, 0, 8),
                                                          (0, 1, 1, 0, 1), (3, 0, 0, 7, 8), (1, 0, 3, 7, 32),
                                                          (0, 0, 0, 3, 1), (1, 0, 0, 1, 4)])
def test_schedule_variants_are_bit_identical(ctx, hf_workload, hf_scene, blue_noise, dyn, prim, blocks, spread,
                                             rmin):
    # the launch schedule (fetch mode, persistent primary, blocks per SM,
    # triangle tests spread over the warp, idle lanes before a refill)
    # changes which thread traces a ray, never the result
    wl, mesh, bvh = hf_workload
    saved = ctx.tuning()
    try:
        ctx.set_tuning(dynamic_fetch=dyn, primary_persistent=prim, trace_blocks_per_sm=blocks, tri_spread=spread,
                       refill_min=rmin)
        img, g = _pathtrace_gpu(ctx, wl, hf_scene, blue_noise, frame=2)
    finally:
        lib().mrt_cuda_set_tuning(ctx.handle, saved)
    ctx.set_tuning(dynamic_fetch=1, primary_persistent=1, trace_blocks_per_sm=0, tri_spread=0, refill_min=1)
    ref_img, ref_g = _pathtrace_gpu(ctx, wl, hf_scene, blue_noise, frame=2)
    lib().mrt_cuda_set_tuning(ctx.handle, saved)
    assert np.array_equal(g["visibility"], ref_g["visibility"])
    assert np.array_equal(img.view(np.uint32), ref_img.view(np.uint32))


def test_ray_sorting_gives_identical_images(ctx, ico_workload, ico_scene, blue_noise):
    # sorting reorders the extension queues between bounces; every pixel
    # owns its path, so the image is bit-identical
    wl, mesh, bvh = ico_workload
    saved = ctx.tuning()
    try:
        ctx.set_tuning(sort_min_rays=0xFFFFFFFF)
        ref, _ = _pathtrace_gpu(ctx, wl, ico_scene, blue_noise, frame=1)
        ctx.set_tuning(sort_min_rays=0)
        img, _ = _pathtrace_gpu(ctx, wl, ico_scene, blue_noise, frame=1)
        assert ctx.status() == 0
    finally:
        lib().mrt_cuda_set_tuning(ctx.handle, saved)
    assert np.array_equal(img.view(np.uint32), ref.view(np.uint32))
