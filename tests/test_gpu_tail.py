"""The path tail (mrt_tuning.tail_bounce): one persistent launch finishing the
paths alive at a given bounce gives the image and the ray counts of the
wavefront passes, bit for bit, through the C ABI."""
import numpy as np
import pytest

from minotert_gb300.pathtracer import Pathtracer, TraceSettings
from minotert_gb300.scene import DeviceScene

pytestmark = pytest.mark.gpu


def _render(ctx, ds, wl, bn, settings, tail, from_hits=0, spread=0):
    saved = int(ctx.tuning().tail_bounce)
    saved_fh = int(ctx.tuning().tail_from_hits)
    saved_sp = int(ctx.tuning().tri_spread)
    ctx.set_tuning(tail_bounce=tail, tail_from_hits=from_hits, tri_spread=(saved_sp & 7) | (8 if spread else 0))
    try:
        pt = Pathtracer(ctx, ds, full_gbuffer=False)
        pt.frame_counter = 4
        gb = pt.primaryRays((wl.width, wl.height), wl.camera, wl.camera)
        ctx.frame_stats()  # reset
        col = pt.secondaryRays(gb, wl.camera, wl.sky, bn, settings)
        img = col.download(np.float32, (wl.height, wl.width, 3))
        st = ctx.frame_stats()
    finally:
        ctx.set_tuning(tail_bounce=saved, tail_from_hits=saved_fh, tri_spread=saved_sp)
    return img, list(st.extension_rays), int(st.shadow_rays)


@pytest.mark.parametrize("settings", [TraceSettings(samples=1, bounces=4, rr_start=2, rng_mode=1),
                                      TraceSettings(samples=2, bounces=6, rr_start=0, rng_mode=0)])
def test_tail_matches_wavefront(ctx, hf_workload, blue_noise, settings):
    wl, mesh, bvh = hf_workload
    ds = DeviceScene.triangles(ctx, mesh, bvh)
    ref, ext, shadow = _render(ctx, ds, wl, blue_noise, settings, 0, 0)
    assert ext[0] > 0 and shadow > 0 and np.isfinite(ref).all()
    for tail in (1, 2, settings.bounces):
        for fh in (0, 1):  # the tail traces bounce `tail` itself, or starts from its hits
            for sp in (0, 1):  # per-lane paths, or the warp's steps taken together
                img, e, sh = _render(ctx, ds, wl, blue_noise, settings, tail, fh, sp)
                assert np.array_equal(img.view(np.uint32), ref.view(np.uint32)), (tail, fh, sp)
                assert e == ext and sh == shadow, (tail, fh, sp)
    assert ctx.status() == 0


def test_tail_bounce_range(ctx):
    from minotert_gb300._lib import MrtError
    saved = int(ctx.tuning().tail_bounce)
    with pytest.raises(MrtError):
        ctx.set_tuning(tail_bounce=99)
    ctx.set_tuning(tail_bounce=saved)
