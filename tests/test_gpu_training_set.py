"""The denoiser's training set on the GPU: a camera window renders exactly
the full frame's pixels; host primary rays traced by the batched tracer hit
what primaryRays hits; the batched path trace (which renders the 4,096-spp
targets) and the single-scene tracer (which renders the 1-spp inputs)
estimate the same radiance; the accumulation of ray copies."""
import math

import numpy as np
import pytest

from minotert_gb300 import scene
from minotert_gb300._lib import HIT_DTYPE, MRT_MISS
from minotert_gb300.pathtracer import Camera, Pathtracer, Sky, TraceSettings, primary_rays_host

pytestmark = pytest.mark.gpu

WIN = (40, 24, 64, 48)


def _cam(window=None):
    return Camera((192, 128), math.radians(60.0), 0.01, (18.0, 6.0, 11.0), math.atan2(-6.0, -18.0), -0.5,
                  window=window)


@pytest.fixture(scope="module")
def hf_small(built_lib):
    mesh = scene.heightfield_boxes(2024, 64, 32)
    return mesh, scene.build_bvh8(mesh)


def test_camera_window_renders_the_full_frames_pixels(ctx, hf_small):
    mesh, bvh = hf_small
    pt = Pathtracer(ctx, scene.DeviceScene.triangles(ctx, mesh, bvh), full_gbuffer=False)
    full = pt.primaryRays((192, 128), _cam(), _cam()).download()
    x0, y0, w, h = WIN
    sub = pt.primaryRays((w, h), _cam(WIN), _cam(WIN)).download()
    crop_v, crop_t = full["visibility"][y0:y0 + h, x0:x0 + w], full["hit_t"][y0:y0 + h, x0:x0 + w]
    same = crop_v == sub["visibility"]
    # the window's NDC differ from the full frame's by a rounding: only rays
    # grazing a triangle edge may change triangle
    assert same.mean() > 0.995, same.mean()
    hit = same & (sub["visibility"] != MRT_MISS)
    assert hit.mean() > 0.5
    assert np.allclose(sub["hit_t"][hit], crop_t[hit], rtol=1e-4)


def test_host_primary_rays_hit_what_primary_rays_hits(ctx, hf_small):
    mesh, bvh = hf_small
    cam = _cam(WIN)
    w, h = WIN[2], WIN[3]
    pt = Pathtracer(ctx, scene.DeviceScene.triangles(ctx, mesh, bvh), full_gbuffer=False)
    g = pt.primaryRays((w, h), cam, cam).download()
    rays = primary_rays_host(cam, w, h)
    batch = scene.DeviceBatch(ctx, [(mesh, bvh)])
    d_rays, d_hits = ctx.to_device(rays), ctx.alloc(len(rays) * HIT_DTYPE.itemsize)
    batch.trace(d_rays, np.array([0, len(rays)], np.uint32), d_hits)
    hits = d_hits.download(HIT_DTYPE, (len(rays),)).reshape(h, w)
    same = hits["prim"] == g["visibility"]
    assert same.mean() > 0.995, same.mean()
    hit = same & (hits["prim"] != MRT_MISS)
    assert np.allclose(hits["t"][hit], g["hit_t"][hit], rtol=1e-4)
    batch.close()


def test_accumulate_copies(ctx):
    rng = np.random.default_rng(4)
    groups, copies, count = 3, 5, 4 * 37
    x = rng.standard_normal((groups, copies, count)).astype(np.float32)
    acc0 = rng.standard_normal((groups, count)).astype(np.float32)
    d_x, d_acc = ctx.to_device(x), ctx.to_device(acc0)
    scene.accumulate_copies(ctx, d_acc, d_x, groups, copies, count, 0.25)
    got = d_acc.download(np.float32, (groups, count))
    assert np.allclose(got, acc0 + 0.25 * x.sum(axis=1), atol=1e-5)


@pytest.mark.parametrize("sun", [None, (0.45, -0.35, 0.82)], ids=["sky", "sky+sun"])
def test_batched_targets_and_single_scene_inputs_estimate_the_same_radiance(ctx, hf_small, blue_noise, sun):
    # constant sky (escape estimator) or sky + directional light (next-event
    # estimation with shadow rays), 8 bounces, Russian roulette after 2: the
    # single-scene tracer (blue-noise rotated sequences) and the batched
    # tracer (per-ray PCG) are different estimators of the same radiance,
    # 1,024 samples per pixel each over a 64 x 48 window
    mesh, bvh = hf_small
    cam = _cam(WIN)
    w, h = WIN[2], WIN[3]
    sky = Sky((0.25, 0.32, 0.45), sun, (2.5, 2.5, 2.5))
    pt = Pathtracer(ctx, scene.DeviceScene.triangles(ctx, mesh, bvh), full_gbuffer=False)
    col = ctx.alloc(12 * w * h)
    for f in range(16):
        pt.frame_counter = 7000 + f
        gb = pt.primaryRays((w, h), cam, cam)
        pt.secondaryRays(gb, cam, sky, blue_noise, TraceSettings(64, 8, 2, 1, True, f), color=col)
    single = col.download(np.float32, (h, w, 3))

    copies = 64
    rays = np.tile(primary_rays_host(cam, w, h), copies)
    batch = scene.DeviceBatch(ctx, [(mesh, bvh)])
    d_rays, d_rad = ctx.to_device(rays), ctx.alloc(12 * len(rays))
    acc = ctx.alloc(12 * w * h)
    acc.zero()
    params = TraceSettings(1, 8, 2).params(sky)
    for f in range(16):
        batch.pathtrace(d_rays, np.array([0, len(rays)], np.uint32), params, 100 + f, d_rad)
        batch.accumulate(acc, d_rad, 1, copies, 3 * w * h, 1.0 / (16 * copies))
    batched = acc.download(np.float32, (h, w, 3))
    batch.close()
    assert ctx.status() == 0
    assert np.isfinite(single).all() and np.isfinite(batched).all()
    rel = abs(batched.mean() - single.mean()) / single.mean()
    assert rel < 0.01, (batched.mean(), single.mean())
    # 8 x 8 pixel blocks: ~65k samples per estimator and block
    bs = lambda im: im.reshape(h // 8, 8, w // 8, 8, 3).mean(axis=(1, 3))
    d = (bs(batched) - bs(single)) / np.maximum(bs(single), 1e-3)
    assert np.sqrt(np.mean(d ** 2)) < 0.03, np.sqrt(np.mean(d ** 2))
