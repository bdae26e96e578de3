"""The oracle against the reference's own shaders (parity pins).

The reference's compute shaders (src/gpu of MinoteRT) are rewritten into C++
against oracle/glsl/glsl.hpp and compiled for the host by
oracle/glsl/build_ref.py (test infrastructure).  These tests compare the
oracle with them:
  * against tests/golden/glsl_reference_vectors.npz, the outputs of those
    shaders on seeded inputs (tests/golden/make_glsl_vectors.py) — always;
  * against the shaders themselves on other inputs — where the reference
    tree is present.
Bars: bit-identical for the random-number generator, ray/sphere, the primary
pass's g-buffer (FP16 as stored), the secondary pass's colour under the sky,
the three sky LUTs and the six tonemappers (UNORM8).  The bilateral filter
agrees to 1e-5 relative on 99.9 % of the pixels and to 1e-4 on all: the
shader samples at uv + d / size, which lands within float rounding of the
whole-column / fractional-row pixel positions the oracle (and the CUDA
kernel) use, and at a depth edge that rounding moves a little weight across
the edge.  The primary pass's depth and motion
are compared on hit pixels only: for a miss the shader projects an
Intersection.t it never assigned (undefined in GLSL).
"""
import ctypes as C
import hashlib
import sys
from pathlib import Path

import numpy as np
import pytest

import oracle
from conftest import oracle_consts
from oracle import post

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
import make_glsl_vectors as mk  # noqa: E402

GOLD = np.load(Path(__file__).resolve().parent / "golden" / "glsl_reference_vectors.npz")
MISS = 0xFFFFFFFF


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


@pytest.fixture(scope="module")
def ref():
    from oracle.glsl import build_ref
    L = build_ref.lib()
    if L is None:
        pytest.skip("reference tree not present: the golden-vector tests cover the pins")
    return L


def _spheres():
    from minotert_gb300.scene import reference_spheres
    return reference_spheres()


def _camera(w, h):
    from minotert_gb300.pathtracer import Camera
    return Camera.reference(w, h)


def _sky():
    atmo = post.earth()
    trans = post.sky_transmittance(atmo)
    ms = post.sky_multiscatter(atmo, trans)
    return atmo, trans, ms


# ---- against the committed vectors -------------------------------------


def test_random_glsl_vectors():
    for s, o, f in zip(GOLD["pcg_state"], GOLD["pcg_out"], GOLD["pcg_float"]):
        assert oracle.pcg(int(s)) == int(o)
        val, _ = oracle.random_float(int(s))
        assert np.float32(val) == f
    got = np.array([oracle.sphere_point(float(x), float(y)) for x, y in GOLD["sp_in"]], np.float32)
    assert np.array_equal(got.view(np.uint32), GOLD["sp_out"].view(np.uint32))


def test_ray_sphere_vectors():
    r = GOLD["rs_in"]
    got = np.array([oracle.ray_sphere(a[0:3], a[3:6], a[6:9], float(a[9])) for a in r], np.float32)
    assert np.array_equal(got.view(np.uint32), GOLD["rs_out"].view(np.uint32))


def test_primary_pass_vectors():
    cam = _camera(96, 54)
    g = oracle.primary(oracle_consts(cam, 3), 96, 54, spheres=_spheres())
    vis = GOLD["prim_visibility"]
    assert np.array_equal(g["visibility"], vis)
    hit = vis != MISS
    assert 0.2 < hit.mean() < 0.9
    assert np.array_equal(g["depth"][hit], GOLD["prim_depth"][hit])
    assert np.array_equal(g["normal"], GOLD["prim_normal"])
    assert np.array_equal(g["motion"][hit], GOLD["prim_motion"][hit])


def test_sky_lut_vectors():
    atmo, trans, ms = _sky()
    probe = np.asarray(_camera(48, 27).position, np.float32)
    view = post.sky_view(atmo, trans, ms, probe, mk.SUN, mk.SUN_E)
    for name, lut in (("trans", trans), ("ms", ms), ("view", view)):
        rgb = np.ascontiguousarray(lut[..., :3])
        probe_txl = rgb[:: max(1, rgb.shape[0] // 4), :: max(1, rgb.shape[1] // 4)]
        assert np.array_equal(probe_txl, GOLD[f"sky_{name}_probe"]), name
        assert hashlib.sha256(rgb.tobytes()).digest() == GOLD[f"sky_{name}_sha256"].tobytes(), name


def test_secondary_pass_vectors():
    from conftest import asset_blue_noise
    atmo, trans, ms = _sky()
    W, H = 48, 27
    cam = _camera(W, H)
    probe = np.asarray(cam.position, np.float32)
    view = post.sky_view(atmo, trans, ms, probe, mk.SUN, mk.SUN_E)
    g = oracle.primary(oracle_consts(cam, 3), W, H, spheres=_spheres())
    post.bind_sky(atmo, trans, view, probe, mk.SUN, mk.SUN_E)
    try:
        col = oracle.secondary_spheres(_spheres(), oracle_consts(cam, 3), W, H, g["visibility"], g["depth"],
                                       g["normal"], asset_blue_noise(), oracle.params_array(8, 8))
    finally:
        post.bind_sky()
    assert np.array_equal(col.view(np.uint32), GOLD["sec_color"].view(np.uint32))


def test_tonemap_vectors():
    for n in mk.TONEMAPS:
        got = post.tonemap(GOLD["tm_in"], n, GOLD["tm_params"])[..., :3]
        assert np.array_equal(got, GOLD[f"tm_{n}"]), n


def test_bilateral_vectors():
    got = post.bilateral(GOLD["bil_color"], GOLD["bil_depth"], GOLD["bil_normal"], 5.0, 2.0, 0.12, 0.001, 7, True)
    ref = GOLD["bil_out"]
    assert np.isfinite(ref).all()
    rel = (np.abs(got - ref) / np.abs(ref)).max(axis=2)
    assert np.mean(rel < 1e-5) > 0.999 and rel.max() < 1e-4


# ---- against the reference's shaders on other inputs -------------------


def test_random_and_sphere_live(ref):
    rng = np.random.default_rng(77)
    for s in rng.integers(0, 2**32, 20000, dtype=np.uint64):
        a = C.c_uint32(int(s))
        assert ref.ref_pcg(C.byref(a)) == oracle.pcg(int(s))
    o3 = (C.c_float * 3)()
    for x, y in rng.uniform(-1, 1, (5000, 2)).astype(np.float32):
        ref.ref_random_sphere_point(float(x), float(y), o3)
        assert np.array_equal(np.array(list(o3), np.float32), np.asarray(oracle.sphere_point(float(x), float(y)),
                                                                          np.float32))


def test_primary_pass_live(ref):
    W, H = 131, 77  # odd sizes
    cam = _camera(W, H)
    consts = oracle_consts(cam, 11, prev=_camera(W, H))
    c = np.ascontiguousarray(consts).view(np.float32)
    vis4 = np.zeros((H, W, 4), np.uint32)
    d4, n4, m4 = (np.zeros((H, W, 4), np.float32) for _ in range(3))
    ref.ref_primary_rays(_p(c), W, H, _p(vis4), _p(d4), _p(n4), _p(m4))
    g = oracle.primary(consts, W, H, spheres=_spheres())
    assert np.array_equal(g["visibility"], vis4[..., 0])
    hit = vis4[..., 0] != MISS
    assert np.array_equal(g["depth"][hit], d4[..., 0].astype(np.float16).view(np.uint16)[hit])
    assert np.array_equal(g["normal"], n4.astype(np.float16).view(np.uint16))


def test_secondary_pass_live(ref):
    from minotert_gb300.scene import blue_noise
    atmo, trans, ms = _sky()
    W, H = 40, 24
    cam = _camera(W, H)
    probe = np.asarray(cam.position, np.float32)
    view = post.sky_view(atmo, trans, ms, probe, mk.SUN, mk.SUN_E)
    consts = oracle_consts(cam, 9)
    g = oracle.primary(consts, W, H, spheres=_spheres())
    bn = blue_noise(3, 64)
    post.bind_sky(atmo, trans, view, probe, mk.SUN, mk.SUN_E)
    try:
        col = oracle.secondary_spheres(_spheres(), consts, W, H, g["visibility"], g["depth"], g["normal"], bn,
                                       oracle.params_array(8, 8))
    finally:
        post.bind_sky()
    vis4 = np.zeros((H, W, 4), np.uint32)
    vis4[..., 0] = g["visibility"]
    dep4 = np.zeros((H, W, 4), np.float32)
    dep4[..., 0] = g["depth"].view(np.float16).astype(np.float32)
    nrm4 = np.ascontiguousarray(g["normal"].view(np.float16).astype(np.float32))
    bn4 = np.ascontiguousarray(bn.astype(np.float32) / np.float32(255.0))
    out = np.zeros((H, W, 4), np.float32)
    c = np.ascontiguousarray(consts).view(np.float32)
    ref.ref_secondary_rays(_p(c), W, H, _p(vis4), _p(dep4), _p(nrm4), _p(bn4), 64, 64, _p(trans), 256, 64,
                           _p(view), 192, 108, _p(atmo), _p(out))
    assert np.array_equal(col.view(np.uint32), out[..., :3].view(np.uint32))


def test_tonemaps_live(ref):
    rng = np.random.default_rng(8)
    img = (rng.gamma(0.5, 2.0, (24, 40, 3)) * 3).astype(np.float32)
    tp = post.tonemap_params(exposure=0.7, reinhard_max=4.0, uchimura=(1.2, 0.9, 0.25, 0.35, 1.2, 0.01),
                             amd=(12.0, 1.6, 0.95, 0.2, 0.16))
    src4 = np.zeros((24, 40, 4), np.float32)
    src4[..., :3] = img
    for n in mk.TONEMAPS:
        d = np.zeros_like(src4)
        pr = mk.tonemap_push(tp, n)
        assert getattr(ref, f"ref_tonemap_{n}")(_p(src4), 40, 24, _p(pr), len(pr), _p(d)) == 0
        assert np.array_equal(post.tonemap(img, n, tp)[..., :3], mk.unorm8(d[..., :3])), n
