"""Golden vectors from the reference's own compute shaders.

Builds the reference's GLSL (src/gpu/*.comp, *.glsl of MinoteRT) for the
host with oracle/glsl/build_ref.py, runs it on seeded inputs and writes the
outputs to tests/golden/glsl_reference_vectors.npz, so that the oracle stays
pinned to the reference where the reference tree is absent.  Run from the
repository root:  python tests/golden/make_glsl_vectors.py

Contents (inputs are regenerated by the tests from the same seeds and stored
where they are random arrays):
  pcg_state, pcg_out, pcg_float      random.glsl pcg / randomFloat
  sp_in, sp_out                      randomSpherePoint
  rs_in, rs_out                      intersect.glsl raySphereIntersect
  prim_*                             primaryRay.comp, reference spheres and
                                     camera, 96 x 54, frame 3 (FP16 bits)
  sec_color                          secondaryRays.comp, 48 x 27, frame 3,
                                     8 samples x 8 bounces, under the sky
  sky_*_sha256, sky_*_probe          the three sky LUTs (SHA-256 of the
                                     float32 bytes and a few texels)
  tm_in, tm_params, tm_<mode>        the six tonemappers, 32 x 32 (UNORM8)
  bil_color, bil_depth, bil_normal,  bilateral.comp, 48 x 32, on the primary
  bil_out                            pass's g-buffer (FP16 bits)
"""
from __future__ import annotations

import ctypes as C
import hashlib
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

OUT = Path(__file__).resolve().parent / "glsl_reference_vectors.npz"
SUN = np.array([-0.435286462, 0.818654716, 0.374606609], np.float32)  # secondaryRays.comp:43
SUN_E = np.full(3, 8.0, np.float32)                                    # secondaryRays.comp:44
TONEMAPS = ("linear", "reinhard", "hable", "aces", "uchimura", "amd")


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def tonemap_push(tp, name):
    """A tonemapper's push constants from the oracle's 13-float parameter block."""
    return np.array({"linear": [tp[0]], "reinhard": [tp[0], tp[1]], "hable": [tp[0]], "aces": [tp[0]],
                     "uchimura": [tp[0], *tp[2:8]], "amd": [tp[0], *tp[8:13]]}[name], np.float32)


def tonemap_input():
    rng = np.random.default_rng(5)
    img = (rng.gamma(0.7, 1.5, (32, 32, 3)) * rng.choice([0.01, 0.3, 1.0, 6.0], (32, 32, 1))).astype(np.float32)
    img[0, :3] = [[0, 0, 0], [1e-7, 2e-6, 0], [50, 0.1, 3]]
    return img


def unorm8(x):
    """FP32 -> UNORM8, round to nearest even (the oracle's and the kernels' rule)."""
    return np.rint(np.clip(x, 0.0, 1.0) * np.float32(255.0)).astype(np.uint8)


def main():
    from conftest import oracle_consts
    from oracle import post
    from oracle.glsl import build_ref
    from minotert_gb300.pathtracer import Camera
    from minotert_gb300.scene import reference_spheres

    L = build_ref.lib()
    if L is None:
        raise SystemExit("the reference tree is not available")
    v = {}
    rng = np.random.default_rng(2024)
    # random.glsl
    st = rng.integers(0, 2**32, 1024, dtype=np.uint64).astype(np.uint32)
    out, fl = np.zeros_like(st), np.zeros(len(st), np.float32)
    for i, s in enumerate(st):
        a = C.c_uint32(int(s))
        out[i] = L.ref_pcg(C.byref(a))
        b = C.c_uint32(int(s))
        fl[i] = L.ref_random_float(C.byref(b))
    v["pcg_state"], v["pcg_out"], v["pcg_float"] = st, out, fl
    sp = rng.uniform(-1, 1, (1024, 2)).astype(np.float32)
    spo = np.zeros((1024, 3), np.float32)
    o3 = (C.c_float * 3)()
    for i, (x, y) in enumerate(sp):
        L.ref_random_sphere_point(float(x), float(y), o3)
        spo[i] = list(o3)
    v["sp_in"], v["sp_out"] = sp, spo
    # intersect.glsl: origin, direction, centre, radius
    rs = np.concatenate([rng.uniform(-1, 1, (1024, 9)), rng.uniform(0.05, 1.0, (1024, 1))], 1).astype(np.float32)
    rso = np.zeros(1024, np.float32)
    for i, r in enumerate(rs):
        a = (C.c_float * 3)(*r[0:3]); d = (C.c_float * 3)(*r[3:6]); c = (C.c_float * 3)(*r[6:9])
        rso[i] = L.ref_ray_sphere(a, d, c, float(r[9]))
    v["rs_in"], v["rs_out"] = rs, rso
    # primaryRay.comp
    W, H = 96, 54
    cam = Camera.reference(W, H)
    consts = np.ascontiguousarray(oracle_consts(cam, 3)).view(np.float32)
    vis4 = np.zeros((H, W, 4), np.uint32)
    d4, n4, m4 = (np.zeros((H, W, 4), np.float32) for _ in range(3))
    L.ref_primary_rays(_p(consts), W, H, _p(vis4), _p(d4), _p(n4), _p(m4))
    v["prim_visibility"] = vis4[..., 0].copy()
    v["prim_depth"] = d4[..., 0].astype(np.float16).view(np.uint16)
    v["prim_normal"] = n4.astype(np.float16).view(np.uint16)
    v["prim_motion"] = m4[..., :2].astype(np.float16).view(np.uint16)
    # sky LUTs
    atmo = post.earth()
    trans = np.zeros((64, 256, 4), np.float32)
    L.ref_sky_transmittance(_p(atmo), _p(trans))
    ms = np.zeros((32, 32, 4), np.float32)
    L.ref_sky_multiscatter(_p(atmo), _p(trans), _p(ms))
    probe = np.asarray(Camera.reference(48, 27).position, np.float32)
    view = np.zeros((108, 192, 4), np.float32)
    L.ref_sky_view(_p(atmo), _p(trans), _p(ms), _p(probe), _p(SUN), _p(SUN_E), _p(view))
    for name, lut in (("trans", trans), ("ms", ms), ("view", view)):
        rgb = np.ascontiguousarray(lut[..., :3])
        v[f"sky_{name}_sha256"] = np.frombuffer(hashlib.sha256(rgb.tobytes()).digest(), np.uint8)
        v[f"sky_{name}_probe"] = rgb[:: max(1, rgb.shape[0] // 4), :: max(1, rgb.shape[1] // 4)].copy()
    # secondaryRays.comp on the primary pass's g-buffer (as stored, FP16)
    W2, H2 = 48, 27
    cam2 = Camera.reference(W2, H2)
    c2 = np.ascontiguousarray(oracle_consts(cam2, 3)).view(np.float32)
    vis4 = np.zeros((H2, W2, 4), np.uint32)
    d4, n4, m4 = (np.zeros((H2, W2, 4), np.float32) for _ in range(3))
    L.ref_primary_rays(_p(c2), W2, H2, _p(vis4), _p(d4), _p(n4), _p(m4))
    dep4 = np.zeros_like(d4)
    dep4[..., 0] = d4[..., 0].astype(np.float16).astype(np.float32)
    nrm4 = np.ascontiguousarray(n4.astype(np.float16).astype(np.float32))
    # the reference's own blue-noise texture, fetched at Gid % 256 (secondaryRays.comp:125)
    bnt = np.load(Path(__file__).resolve().parent / "blue_noise_asset.npz")["rgba"]
    bn4 = np.ascontiguousarray(bnt.astype(np.float32) / np.float32(255.0))
    col = np.zeros((H2, W2, 4), np.float32)
    L.ref_secondary_rays(_p(c2), W2, H2, _p(vis4), _p(dep4), _p(nrm4), _p(bn4), bnt.shape[1], bnt.shape[0], _p(trans),
                         256, 64,
                         _p(view), 192, 108, _p(atmo), _p(col))
    v["sec_color"] = col[..., :3].copy()
    # tonemappers
    img = tonemap_input()
    tp = post.tonemap_params(exposure=1.3)
    src4 = np.zeros((32, 32, 4), np.float32)
    src4[..., :3] = img
    v["tm_in"], v["tm_params"] = img, tp
    for n in TONEMAPS:
        d = np.zeros((32, 32, 4), np.float32)
        pr = tonemap_push(tp, n)
        getattr(L, f"ref_tonemap_{n}")(_p(src4), 32, 32, _p(pr), len(pr), _p(d))
        v[f"tm_{n}"] = unorm8(d[..., :3])
    # bilateral.comp on the reference spheres' g-buffer
    W3, H3 = 48, 32
    cam3 = Camera.reference(W3, H3)
    c3 = np.ascontiguousarray(oracle_consts(cam3)).view(np.float32)
    vis4 = np.zeros((H3, W3, 4), np.uint32)
    d4, n4, m4 = (np.zeros((H3, W3, 4), np.float32) for _ in range(3))
    L.ref_primary_rays(_p(c3), W3, H3, _p(vis4), _p(d4), _p(n4), _p(m4))
    color = np.random.default_rng(3).gamma(2.0, 0.3, (H3, W3, 3)).astype(np.float32)
    c4 = np.zeros((H3, W3, 4), np.float32)
    c4[..., :3] = color
    z4 = np.zeros_like(c4)
    # a miss's depth is undefined in the shader (it projects an unassigned
    # Intersection.t); the filter gets 0 there, the value the oracle and the
    # CUDA primary pass store
    z4[..., 0] = np.where(vis4[..., 0] == 0xFFFFFFFF, 0.0, d4[..., 0]).astype(np.float16).astype(np.float32)
    nn4 = np.ascontiguousarray(n4.astype(np.float16).astype(np.float32))
    prm = np.array([5.0, 2.0, 0.12, 0.001, 0.0], np.float32)
    prm.view(np.uint32)[4] = 7
    out = np.zeros((H3, W3, 4), np.float32)
    L.ref_bilateral(_p(c4), _p(z4), _p(nn4), W3, H3, _p(prm), _p(out))
    v["bil_color"], v["bil_out"] = color, out[..., :3].copy()
    v["bil_depth"] = z4[..., 0].astype(np.float16).view(np.uint16)
    v["bil_normal"] = n4.astype(np.float16).view(np.uint16)
    np.savez_compressed(OUT, **v)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes)")


if __name__ == "__main__":
    main()
