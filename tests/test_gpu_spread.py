"""Triangle tests spread over the warp (mrt_tuning.tri_spread): the primary,
extension and shadow kernels that test a step's triangles as (ray, triangle)
pairs across all 32 lanes, with either work schedule, give the per-lane
loop's hits, image and ray counts, bit for bit, through the C ABI."""
import numpy as np
import pytest

import oracle
from conftest import oracle_consts, random_rays
from minotert_gb300.pathtracer import Camera, Pathtracer, TraceSettings
from minotert_gb300.scene import DeviceScene

pytestmark = pytest.mark.gpu


def _render(ctx, ds, wl, bn, settings, spread, tail, dyn=3):
    saved = ctx.tuning()
    ctx.set_tuning(tri_spread=spread, tail_bounce=tail, dynamic_fetch=dyn)
    try:
        pt = Pathtracer(ctx, ds, full_gbuffer=False)
        pt.frame_counter = 5
        gb = pt.primaryRays((wl.width, wl.height), wl.camera, wl.camera)
        ctx.frame_stats()  # reset
        col = pt.secondaryRays(gb, wl.camera, wl.sky, bn, settings)
        img = col.download(np.float32, (wl.height, wl.width, 3))
        st = ctx.frame_stats()
    finally:
        ctx.set_tuning(**{f: getattr(saved, f) for f, _ in saved._fields_})
    return img, list(st.extension_rays), int(st.shadow_rays)


@pytest.mark.parametrize("settings", [TraceSettings(samples=1, bounces=4, rr_start=2, rng_mode=1),
                                      TraceSettings(samples=2, bounces=6, rr_start=0, rng_mode=0)])
def test_spread_matches_per_lane(ctx, hf_workload, blue_noise, settings):
    wl, mesh, bvh = hf_workload
    ds = DeviceScene.triangles(ctx, mesh, bvh)
    ref, ext, shadow = _render(ctx, ds, wl, blue_noise, settings, 0, 0)
    assert ext[0] > 0 and shadow > 0 and np.isfinite(ref).all()
    for spread in (1, 2, 3):
        for dyn in (3, 0):
            img, e, sh = _render(ctx, ds, wl, blue_noise, settings, spread, 0, dyn)
            assert np.array_equal(img.view(np.uint32), ref.view(np.uint32)), (spread, dyn)
            assert e == ext and sh == shadow, (spread, dyn)
    # with the path tail finishing bounces >= 2
    img, e, sh = _render(ctx, ds, wl, blue_noise, settings, 3, 2)
    assert np.array_equal(img.view(np.uint32), ref.view(np.uint32))
    assert e == ext and sh == shadow
    assert ctx.status() == 0


def test_spread_range(ctx):
    from minotert_gb300._lib import MrtError
    saved = int(ctx.tuning().tri_spread)
    with pytest.raises(MrtError):
        ctx.set_tuning(tri_spread=16)
    ctx.set_tuning(tri_spread=saved)
    saved = int(ctx.tuning().refill_min)
    with pytest.raises(MrtError):
        ctx.set_tuning(refill_min=33)
    ctx.set_tuning(refill_min=saved)


@pytest.mark.parametrize("size", [(256, 256), (77, 45), (31, 3)])
def test_spread_primary_matches_oracle(ctx, hf_workload, size):
    # one thread per pixel, warps stepping together; odd sizes leave lanes
    # outside the image that still test other lanes' triangles
    wl, mesh, bvh = hf_workload
    ds = DeviceScene.triangles(ctx, mesh, bvh)
    c = wl.camera
    cam = Camera(viewport=size, verticalFov=c.verticalFov, nearPlane=c.nearPlane, position=c.position, yaw=c.yaw,
                 pitch=c.pitch)
    saved = ctx.tuning()
    try:
        ctx.set_tuning(tri_spread=4, primary_persistent=0)
        g = Pathtracer(ctx, ds, full_gbuffer=False).primaryRays(size, cam, cam).download()
    finally:
        ctx.set_tuning(**{f: getattr(saved, f) for f, _ in saved._fields_})
    ref = oracle.primary(oracle_consts(cam), size[0], size[1], bvh.nodes, bvh.tris, mesh.mats)
    assert np.array_equal(g["visibility"], ref["visibility"])
    assert np.array_equal(g["hit_t"].view(np.uint32), ref["hit_t"].view(np.uint32))
    assert ctx.status() == 0


@pytest.mark.parametrize("tail", [0, 3])
def test_overlapped_shadow_rays_same_image(ctx, hf_workload, blue_noise, tail):
    # shadow rays of vertex b - 1 on a second stream beside the extension
    # rays of bounce b, or both in one merged launch: the same image and ray
    # counts
    wl, mesh, bvh = hf_workload
    ds = DeviceScene.triangles(ctx, mesh, bvh)
    settings = TraceSettings(samples=2, bounces=5, rr_start=1, rng_mode=1)
    saved = ctx.tuning()
    try:
        ctx.set_tuning(overlap_shadow=0)
        ref, ext, shadow = _render(ctx, ds, wl, blue_noise, settings, 3, tail)
        ctx.set_tuning(overlap_shadow=1)
        img, e, sh = _render(ctx, ds, wl, blue_noise, settings, 3, tail)
        assert int(ctx.tuning().overlap_shadow) == 1
        # both queues in one persistent launch
        ctx.set_tuning(overlap_shadow=2)
        img2, e2, sh2 = _render(ctx, ds, wl, blue_noise, settings, 3, tail)
    finally:
        ctx.set_tuning(**{f: getattr(saved, f) for f, _ in saved._fields_})
    assert np.array_equal(img.view(np.uint32), ref.view(np.uint32))
    assert np.array_equal(img2.view(np.uint32), ref.view(np.uint32))
    assert e == ext and sh == shadow and e2 == ext and sh2 == shadow
    assert ctx.status() == 0


def test_corrupt_bvh_in_the_path_tracer(ctx, hf_workload, blue_noise):
    # host-side fault injection through the default schedule (spread
    # triangle tests, overlapped shadow rays, path tail) and the batched
    # kernels: a child or triangle index out of range, or a self-referencing
    # child, ends in a status flag; the context keeps working
    from minotert_gb300._lib import MRT_STATUS_BAD_NODE, MRT_STATUS_BAD_TRI
    from minotert_gb300.scene import Bvh8, DeviceBatch
    wl, mesh, bvh = hf_workload
    settings = TraceSettings(samples=1, bounces=4, rr_start=2, rng_mode=1)
    ref, ext, shadow = _render(ctx, DeviceScene.triangles(ctx, mesh, bvh), wl, blue_noise, settings, 3, 3)
    assert ctx.status() == 0
    cases = []
    nodes = bvh.nodes.copy()
    nodes["child_base"][0] = len(nodes) + 1000
    cases.append((nodes, MRT_STATUS_BAD_NODE))
    nodes = bvh.nodes.copy()
    nodes["tri_base"][:] = len(bvh.tris) + 7
    cases.append((nodes, MRT_STATUS_BAD_TRI))
    nodes = bvh.nodes.copy()
    nodes["child_base"][:] = 0
    cases.append((nodes, 0))
    for nodes, flag in cases:
        bad = Bvh8(nodes, bvh.tris, bvh.depth, bvh.leaf_count, 0.0)
        _render(ctx, DeviceScene.triangles(ctx, mesh, bad), wl, blue_noise, settings, 3, 3)
        ctx.sync(timeout_s=30.0)
        st = ctx.status()
        assert st != 0 and (flag == 0 or st & flag), (flag, st)
        batch = DeviceBatch(ctx, [(mesh, bvh), (mesh, bad)])
        rays = np.concatenate([random_rays(2048, mesh.lo, mesh.hi, seed=3)] * 2)
        offsets = np.array([0, 2048, 4096], np.uint32)
        d_rays = ctx.to_device(rays)
        batch.trace(d_rays, offsets, ctx.alloc(8 * len(rays)))
        batch.pathtrace(d_rays, offsets, settings.params(wl.sky), 1, ctx.alloc(12 * len(rays)), use_graph=False)
        ctx.sync(timeout_s=30.0)
        assert ctx.status() != 0
    img, e, sh = _render(ctx, DeviceScene.triangles(ctx, mesh, bvh), wl, blue_noise, settings, 3, 3)
    assert ctx.status() == 0
    assert np.array_equal(img.view(np.uint32), ref.view(np.uint32)) and e == ext and sh == shadow
