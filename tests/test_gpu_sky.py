"""GPU parity of the sky / atmosphere path (mrt_cuda_sky_*) against the CPU
oracle (oracle/post.cpp), and of escaping paths that see the sky.

Both sides evaluate every + - * / with IEEE rounding in the same order; the
differences left come from expf / acosf / cosf / sinf / powf (CUDA's vs the
C library's, a few ulp), so the bars are relative tolerances, tightest
where a stage is fed the other side's LUTs.
"""
import numpy as np
import pytest

import oracle
from conftest import oracle_consts
from minotert_gb300._lib import MRT_MISS
from minotert_gb300.pathtracer import Camera, Pathtracer, Sky as ConstSky, TraceSettings
from minotert_gb300.scene import DeviceScene, reference_spheres
from minotert_gb300.sky import Atmosphere, Sky
from oracle import post

pytestmark = pytest.mark.gpu


def _close(got, ref, typical=2e-5, worst=5e-4, quantile=0.999):
    """Relative error per value (floored at 1e-6 of the largest value):
    the `quantile` within `typical`, all within `worst`.  Both sides share
    exp_cw, so what differs are cosf / sinf / acosf / powf in the directions
    and phase functions."""
    floor = 1e-6 * float(np.abs(ref).max())
    rel = np.abs(got - ref) / (np.abs(ref) + floor)
    q = float(np.quantile(rel, quantile))
    assert q <= typical and rel.max() <= worst, f"rel err q{quantile}={q:.3g} max={rel.max():.3g}"


@pytest.fixture(scope="module")
def atmo(ctx):
    a = Atmosphere(ctx)
    yield a
    a.close()


def _view(atmo, probe=(0.0, 0.0, 0.5)):
    sky = Sky()
    return sky, sky.createView(atmo, np.array(probe, np.float32))


def test_transmittance_lut_vs_oracle(ctx, atmo):
    gpu = atmo.lut(0)
    ref = post.sky_transmittance(atmo.params)
    assert np.allclose(gpu, ref, rtol=2e-5, atol=1e-9)


def test_multiscatter_lut_vs_oracle(ctx, atmo):
    gpu_t = atmo.lut(0)
    gpu = atmo.lut(1)
    # stage alone: the oracle fed the GPU's transmittance LUT
    _close(gpu, post.sky_multiscatter(atmo.params, gpu_t))
    # whole chain
    ref_t = post.sky_transmittance(atmo.params)
    _close(gpu, post.sky_multiscatter(atmo.params, ref_t))


@pytest.mark.parametrize("probe", [(0.0, 0.0, 0.5), (3.0, -2.0, 8.0), (0.0, 0.0, 150.0)])
def test_sky_view_lut_vs_oracle(ctx, atmo, probe):
    sky, view = _view(atmo, probe)
    gpu = atmo.lut(2)
    t, m = atmo.lut(0), atmo.lut(1)
    ref = post.sky_view(atmo.params, t, m, probe, sky.sunDirection, sky.sunIlluminance)
    assert np.isfinite(gpu).all()
    # near the horizon the ray length tMax -- and with it the view march's
    # step count floor(mix(4, 14, tMax / 100 km)), a step function -- moves
    # fast with the zenith angle, so a last-bit cosf difference in a texel's
    # direction shows up at the 1e-4..1e-3 level there
    _close(gpu, ref, typical=5e-4, worst=2e-3, quantile=0.99)


def test_sky_color_vs_oracle(ctx, atmo):
    sky, view = _view(atmo)
    rng = np.random.default_rng(11)
    d = rng.normal(size=(8192, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    # rays into and around the sun disc
    s = sky.sunDirection / np.linalg.norm(sky.sunDirection)
    jitter = rng.normal(scale=2e-3, size=(256, 3)).astype(np.float32)
    ds = s[None, :] + jitter
    ds /= np.linalg.norm(ds, axis=1, keepdims=True)
    d = np.ascontiguousarray(np.concatenate([d, ds, s[None, :]]).astype(np.float32))
    n = len(d)
    d_dirs, d_out = ctx.to_device(d), ctx.alloc(12 * n)
    view.eval(d_dirs, n, d_out)
    gpu = d_out.download(np.float32, (n, 3))
    ref = post.sky_color(atmo.params, atmo.lut(0), atmo.lut(2), view.probe, view.sun, view.sun_e, d)
    assert np.isfinite(gpu).all()
    close = np.isclose(gpu, ref, rtol=2e-5, atol=1e-7).all(axis=1)
    assert close.mean() > 0.999
    assert np.allclose(gpu, ref, rtol=1e-3, atol=1e-6)
    assert (gpu[-1] > 1e4).all()  # the sun itself


def test_reference_spheres_under_the_sky(ctx, atmo, blue_noise):
    # scene 0 exactly as the reference renders it: 8 samples x 8 bounces,
    # escaping paths see skyColor() (sky view + sun disc)
    spheres = reference_spheres()
    ds = DeviceScene.from_spheres(ctx, spheres)
    W, H = 160, 90
    cam = Camera.reference(W, H)
    pt = Pathtracer(ctx, ds)
    pt.frame_counter = 3
    gb = pt.primaryRays((W, H), cam, cam)
    sky, view = _view(atmo, cam.position)
    col = pt.secondaryRays(gb, cam, ConstSky(radiance=(0.0, 0.0, 0.0), sun_dir=None), blue_noise,
                           TraceSettings(samples=8, bounces=8), skyView=view)
    img = col.download(np.float32, (H, W, 3))
    g = gb.download()
    post.bind_sky(atmo.params, atmo.lut(0), atmo.lut(2), view.probe, view.sun, view.sun_e)
    try:
        ref = oracle.secondary_spheres(spheres, oracle_consts(cam, 3), W, H, g["visibility"], g["depth"],
                                       g["normal"], blue_noise, oracle.params_array(8, 8, sky=(0.0, 0.0, 0.0)))
    finally:
        post.bind_sky()
    assert np.isfinite(img).all() and img.max() > 0
    miss = g["visibility"] == MRT_MISS
    assert miss.any() and img[miss].mean() > 0  # the sky shows through
    close = np.isclose(img, ref, rtol=1e-4, atol=1e-6).all(axis=2)
    assert close.mean() > 0.99
    assert np.sqrt(np.mean((img - ref) ** 2)) < 1e-2 * ref.mean()


def test_triangle_paths_under_the_sky(ctx, atmo, hf_workload, blue_noise):
    wl, mesh, bvh = hf_workload
    ds = DeviceScene.triangles(ctx, mesh, bvh)
    pt = Pathtracer(ctx, ds, full_gbuffer=False)
    cam = wl.camera
    gb = pt.primaryRays((wl.width, wl.height), cam, cam)
    sky, view = _view(atmo, cam.position)
    settings = TraceSettings(samples=1, bounces=2)
    col = pt.secondaryRays(gb, cam, ConstSky(radiance=(0.0, 0.0, 0.0), sun_dir=None), blue_noise, settings,
                           skyView=view)
    img = col.download(np.float32, (wl.height, wl.width, 3))
    g = gb.download()
    assert ctx.status() == 0
    post.bind_sky(atmo.params, atmo.lut(0), atmo.lut(2), view.probe, view.sun, view.sun_e)
    try:
        ref, counts, st = oracle.pathtrace(bvh.nodes, bvh.tris, mesh.mats, oracle_consts(cam), wl.width, wl.height,
                                           g["visibility"], g["hit_t"], blue_noise,
                                           oracle.params_array(1, 2, 0, settings.rng_mode, 0, sky=(0.0, 0.0, 0.0)))
    finally:
        post.bind_sky()
    assert np.isfinite(img).all() and img.max() > 0
    close = np.isclose(img, ref, rtol=1e-4, atol=1e-6).all(axis=2)
    assert close.mean() > 0.99
