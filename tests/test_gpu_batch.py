"""Batched multi-scene tracing on the GPU against the per-scene oracle.

The batch concatenates scenes into one BVH with rebased indices; a ray's
closest hit must equal the oracle's hit in its own scene (triangle id after
removing the batch offset, and t, bit for bit).  The graph-captured bounce
loop must equal the directly launched one and the per-ray oracle.
"""
import numpy as np
import pytest

import oracle
from minotert_gb300 import workloads
from minotert_gb300._lib import HIT_DTYPE, MRT_MISS
from minotert_gb300.scene import DeviceBatch, build_bvh8

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small_batch(ctx):
    wl = workloads.batched64(seed=3, count=8, tri_range=(1_000, 40_000), ray_range=(2_000, 20_000))
    scenes = []
    for s in wl.scenes:
        m = s.mesh()
        scenes.append((s, m, build_bvh8(m), s.rays_for(m)))
    batch = DeviceBatch(ctx, [(m, b) for _, m, b, _ in scenes])
    rays = np.concatenate([r for *_, r in scenes])
    offsets = np.concatenate([[0], np.cumsum([len(r) for *_, r in scenes])]).astype(np.uint32)
    return wl, scenes, batch, rays, offsets


def test_batch_trace_matches_per_scene_oracle(ctx, small_batch):
    wl, scenes, batch, rays, offsets = small_batch
    d_rays = ctx.to_device(rays)
    d_hits = ctx.alloc(8 * len(rays))
    for any_hit in (False, True):
        batch.trace(d_rays, offsets, d_hits, any_hit=any_hit)
        hits = d_hits.download(HIT_DTYPE, (len(rays),))
        assert ctx.status() == 0
        for s, (_, m, b, r) in enumerate(scenes):
            h = hits[offsets[s]:offsets[s + 1]]
            ref, st = oracle.trace_bvh8(b.nodes, b.tris, r, any_hit=any_hit)
            local = np.where(h["prim"] == MRT_MISS, MRT_MISS, h["prim"] - np.uint32(batch.tri_offsets[s]))
            if any_hit:
                assert np.array_equal(local == MRT_MISS, ref["prim"] == MRT_MISS)
            else:
                assert np.array_equal(local, ref["prim"]), f"scene {s}"
                assert np.array_equal(h["t"].view(np.uint32), ref["t"].view(np.uint32)), f"scene {s}"
        assert (hits["prim"] != MRT_MISS).mean() > 0.2


@pytest.mark.parametrize("use_graph", [False, True])
def test_batch_pathtrace_vs_oracle(ctx, small_batch, use_graph):
    wl, scenes, batch, rays, offsets = small_batch
    d_rays = ctx.to_device(rays)
    d_rad = ctx.alloc(12 * len(rays))
    params = wl.settings.params(wl.sky)
    outs = []
    for frame in (4, 4, 5):  # a graph is captured once and replayed
        batch.pathtrace(d_rays, offsets, params, frame, d_rad, use_graph=use_graph)
        outs.append(d_rad.download(np.float32, (len(rays), 3)))
        assert ctx.status() == 0
    assert np.array_equal(outs[0], outs[1])
    assert not np.array_equal(outs[0], outs[2])  # the frame reaches the graph's kernels
    p = oracle.params_array(1, wl.settings.bounces, 0, 0, 0, sky=wl.sky.radiance)
    ref = np.zeros_like(outs[0])
    for s, (_, m, b, r) in enumerate(scenes):
        rad, st = oracle.pathtrace_rays(b.nodes, b.tris, m.mats, r, p, frame=4, index_base=int(offsets[s]))
        assert st == 0
        ref[offsets[s]:offsets[s + 1]] = rad
    same = np.isclose(outs[0], ref, rtol=1e-5, atol=1e-6).all(axis=1)
    assert same.mean() > 0.99
    assert abs(outs[0].mean() - ref.mean()) < 1e-3 * ref.mean()


def test_batch_graph_equals_direct_launch(ctx, small_batch):
    wl, scenes, batch, rays, offsets = small_batch
    d_rays = ctx.to_device(rays)
    a, b = ctx.alloc(12 * len(rays)), ctx.alloc(12 * len(rays))
    params = wl.settings.params(wl.sky)
    batch.pathtrace(d_rays, offsets, params, 9, a, use_graph=False)
    batch.pathtrace(d_rays, offsets, params, 9, b, use_graph=True)
    ra, rb = a.download(np.float32, (len(rays), 3)), b.download(np.float32, (len(rays), 3))
    assert np.array_equal(ra.view(np.uint32), rb.view(np.uint32))


def test_batch_stack_depths_agree(ctx, small_batch):
    # the traversal stack size is a tuning choice (16, 24, 32 entries): the
    # hits and the path-traced radiance do not depend on it; a size below the
    # batch's BVH depth is refused
    import ctypes as C
    from minotert_gb300._lib import MrtError, lib
    wl, scenes, batch, rays, offsets = small_batch
    d_rays = ctx.to_device(rays)
    d_hits = ctx.alloc(8 * len(rays))
    d_rad = ctx.alloc(12 * len(rays))
    params = wl.settings.params(wl.sky)
    saved = ctx.tuning()
    outs = {}
    try:
        for depth in (16, 24, 32):
            ctx.set_tuning(stack_depth=depth)
            batch.trace(d_rays, offsets, d_hits)
            batch.pathtrace(d_rays, offsets, params, 5, d_rad, use_graph=True)
            outs[depth] = (d_hits.download(HIT_DTYPE, (len(rays),)).copy(),
                           d_rad.download(np.float32, (len(rays), 3)).copy())
        assert ctx.status() == 0
        for depth in (16, 32):
            assert np.array_equal(outs[depth][0], outs[24][0]), depth
            assert np.array_equal(outs[depth][1].view(np.uint32), outs[24][1].view(np.uint32)), depth
        with pytest.raises(MrtError):
            ctx.set_tuning(stack_depth=20)
    finally:
        lib().mrt_cuda_set_tuning(ctx.handle, C.byref(saved))


def test_batch_schedules_agree(ctx, small_batch):
    # per-lane or spread triangle tests, refill whenever one lane is idle or
    # once 8 / 32 are: same hits (closest and any) and radiance, bit for bit
    import ctypes as C
    from minotert_gb300._lib import lib
    wl, scenes, batch, rays, offsets = small_batch
    d_rays = ctx.to_device(rays)
    d_hits = ctx.alloc(8 * len(rays))
    d_rad = ctx.alloc(12 * len(rays))
    params = wl.settings.params(wl.sky)
    saved = ctx.tuning()
    outs = {}
    try:
        for spread, rmin in ((0, 1), (3, 1), (3, 8), (0, 32), (1, 8)):
            ctx.set_tuning(tri_spread=spread, refill_min=rmin)
            batch.trace(d_rays, offsets, d_hits)
            closest = d_hits.download(HIT_DTYPE, (len(rays),)).copy()
            batch.trace(d_rays, offsets, d_hits, any_hit=True)
            anyhit = d_hits.download(HIT_DTYPE, (len(rays),)).copy()
            batch.pathtrace(d_rays, offsets, params, 5, d_rad, use_graph=True)
            outs[(spread, rmin)] = (closest, anyhit, d_rad.download(np.float32, (len(rays), 3)).copy())
        assert ctx.status() == 0
        ref = outs[(0, 1)]
        assert (ref[0]["prim"] != 0xFFFFFFFF).any() and (ref[1]["prim"] != 0xFFFFFFFF).any()
        for k, v in outs.items():
            assert np.array_equal(v[0], ref[0]), k
            assert np.array_equal(v[1], ref[1]), k
            assert np.array_equal(v[2].view(np.uint32), ref[2].view(np.uint32)), k
    finally:
        lib().mrt_cuda_set_tuning(ctx.handle, C.byref(saved))
