"""The CUDA path against the reference's own shaders, through the C ABI.

tests/golden/glsl_reference_vectors.npz holds the outputs of the reference's
compute shaders (primaryRay.comp, secondaryRays.comp, the six tonemappers),
compiled for the host from the reference's sources
(tests/golden/make_glsl_vectors.py).  Here the GPU renders the same inputs.
Bars: the primary pass's g-buffer bit-identical (depth and motion on hit
pixels: the shader leaves a miss's undefined); the tonemappers within one
UNORM8 step (the kernels' powf / expf are CUDA's, the vectors' the C
library's); the secondary pass within the tolerance of the GPU-vs-oracle
test (the GPU's sincosf in the sphere-point sampler).
"""
from pathlib import Path

import numpy as np
import pytest

from conftest import oracle_consts  # noqa: F401  (registers the tests dir on sys.path)
from minotert_gb300._lib import MRT_MISS
from minotert_gb300.pathtracer import Camera, Pathtracer, Sky as ConstSky, TraceSettings
from minotert_gb300.post import AMDParams, Tonemapper, UchimuraParams
from minotert_gb300.scene import DeviceScene, reference_spheres

pytestmark = pytest.mark.gpu

GOLD = np.load(Path(__file__).resolve().parent / "golden" / "glsl_reference_vectors.npz")


def test_primary_pass_matches_reference_shader(ctx):
    W, H = 96, 54
    ds = DeviceScene.from_spheres(ctx, reference_spheres())
    cam = Camera.reference(W, H)
    pt = Pathtracer(ctx, ds)
    pt.frame_counter = 3
    g = pt.primaryRays((W, H), cam, cam).download()
    vis = GOLD["prim_visibility"]
    assert np.array_equal(g["visibility"], vis)
    hit = vis != MRT_MISS
    assert np.array_equal(g["depth"][hit], GOLD["prim_depth"][hit])
    assert np.array_equal(g["normal"], GOLD["prim_normal"])
    assert np.array_equal(g["motion"][hit], GOLD["prim_motion"][hit])


def test_tonemappers_match_reference_shaders(ctx):
    img = np.ascontiguousarray(GOLD["tm_in"], np.float32)
    tp = GOLD["tm_params"]
    H, W = img.shape[:2]
    d_img = ctx.to_device(img)
    tm = Tonemapper(ctx)
    exposure = float(tp[0])
    outs = {"linear": tm.linear(d_img, W, H, exposure), "reinhard": tm.reinhard(d_img, W, H, exposure, float(tp[1])),
            "hable": tm.hable(d_img, W, H, exposure), "aces": tm.aces(d_img, W, H, exposure),
            "uchimura": tm.uchimura(d_img, W, H, exposure, UchimuraParams(*map(float, tp[2:8]))),
            "amd": tm.amd(d_img, W, H, exposure, AMDParams(*map(float, tp[8:13])))}
    for name, out in outs.items():
        got = out.download(np.uint8, (H, W, 4))[..., :3]
        diff = np.abs(got.astype(int) - GOLD[f"tm_{name}"].astype(int))
        assert diff.max() <= 1 and (diff == 0).mean() > 0.99, name


def test_secondary_pass_matches_reference_shader(ctx, reference_blue_noise):
    from minotert_gb300.sky import Atmosphere, Sky
    W, H = 48, 27
    ds = DeviceScene.from_spheres(ctx, reference_spheres())
    cam = Camera.reference(W, H)
    pt = Pathtracer(ctx, ds)
    pt.frame_counter = 3
    gb = pt.primaryRays((W, H), cam, cam)
    atmo = Atmosphere(ctx)
    try:
        sky = Sky()
        view = sky.createView(atmo, np.asarray(cam.position, np.float32))
        col = pt.secondaryRays(gb, cam, ConstSky(radiance=(0.0, 0.0, 0.0), sun_dir=None), reference_blue_noise,
                               TraceSettings(samples=8, bounces=8), skyView=view)
        img = col.download(np.float32, (H, W, 3))
    finally:
        atmo.close()
    ref = GOLD["sec_color"]
    assert np.isfinite(img).all()
    close = np.isclose(img, ref, rtol=1e-3, atol=1e-5).all(axis=2)
    assert close.mean() > 0.97
    assert np.sqrt(np.mean((img - ref) ** 2)) < 1e-2 * ref.mean()
