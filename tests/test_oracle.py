"""Pins the CPU oracle against known answers (CPU only).

The reference has no tests or golden files, so the oracle is pinned by
formula-derived vectors (tests/golden/make_golden.py computes them in pure
Python / float64 numpy, independently of oracle.cpp), by numpy's IEEE
half conversion, by analytic intersection cases and by brute-force
cross-checks of its BVH traversal.
"""
import json
import math
from pathlib import Path

import numpy as np
import pytest

import oracle
from conftest import random_rays

GOLD = json.loads((Path(__file__).parent / "golden" / "known_answers.json").read_text())
MISS = 0xFFFFFFFF


def test_pcg_known_answers():
    # random.glsl:22-27
    v, seq = 1, []
    for _ in range(32):
        v = oracle.pcg(v)
        seq.append(v)
    assert seq == GOLD["pcg_from_1"]
    assert [oracle.pcg(x) for x in GOLD["pcg_inputs"]] == GOLD["pcg_outputs"]


def test_random_float_is_24bit_exact():
    # random.glsl:29-31: (pcg & 0xFFFFFF) / 2^24 is exact in float32
    s, vals = 3, []
    for _ in range(8):
        f, s = oracle.random_float(s)
        vals.append(f)
    assert vals == GOLD["random_float_from_3"]
    assert all(0.0 <= x < 1.0 for x in vals)


def test_sphere_point_unit_and_formula():
    # random.glsl:10-19: phi = (x+1) pi, z = y, r = sqrt(1-z^2)
    rng = np.random.default_rng(0)
    for rx, ry in rng.uniform(-1, 1, size=(200, 2)):
        p = oracle.sphere_point(float(rx), float(ry))
        phi = (np.float32(rx) + 1) * 3.14159265359
        ref = np.array([math.sqrt(1 - ry * ry) * math.cos(phi), math.sqrt(1 - ry * ry) * math.sin(phi), ry])
        assert np.allclose(p, ref, atol=2e-6)
        assert abs(np.linalg.norm(p.astype(np.float64)) - 1) < 2e-6


def test_half_conversion_matches_ieee_rne():
    rng = np.random.default_rng(1)
    xs = np.concatenate([rng.normal(scale=s, size=4000) for s in (1e-6, 1e-3, 1, 100, 3e4)]).astype(np.float32)
    xs = np.concatenate([xs, np.float32([0.0, -0.0, 65504, 65519.99, 65520, 1e9, -1e9, 2 ** -24, 2 ** -25,
                                         3 * 2 ** -26, 6.1e-5, np.inf, -np.inf])])
    ours = np.array([oracle.f2h(float(x)) for x in xs], np.uint16)
    ref = xs.astype(np.float16).view(np.uint16)
    assert np.array_equal(ours, ref)
    back = np.array([oracle.h2f(int(h)) for h in ref], np.float32)
    assert np.array_equal(back, ref.view(np.float16).astype(np.float32))


def test_reference_camera_matrices():
    # camera.ixx:26-44 / math.ixx:822-861 against a float64 evaluation
    g = GOLD["reference_camera"]
    a = g["args"]
    c = oracle.camera_consts(a["pos"], a["yaw"], a["pitch"], a["fov"], a["znear"], a["w"], a["h"])
    view, proj = c[0:16], c[16:32]
    assert np.allclose(view, g["view_f64"], atol=1e-6)
    assert np.allclose(proj, g["projection_f64"], rtol=1e-6)
    # inverse(m) * m == I
    for m, inv in ((c[0:16], c[32:48]), (c[16:32], c[48:64])):
        M = m.reshape(4, 4).T.astype(np.float64)
        I = inv.reshape(4, 4).T.astype(np.float64)
        assert np.allclose(I @ M, np.eye(4), atol=1e-4)


def test_ray_sphere_reference_semantics():
    # intersect.glsl:26-37: nearer root only; inside-sphere origin -> negative
    t = oracle.ray_sphere([0, 0, -5], [0, 0, 1], [0, 0, 0], 1.0)
    assert t == pytest.approx(4.0)
    assert oracle.ray_sphere([0, 0, 0], [0, 0, 1], [0, 0, 0], 1.0) == pytest.approx(-1.0)  # inside
    assert oracle.ray_sphere([0, 2, -5], [0, 0, 1], [0, 0, 0], 1.0) == -1.0  # miss
    assert oracle.ray_sphere([0, 0, 5], [0, 0, 1], [0, 0, 0], 1.0) < 0  # behind
    t = oracle.ray_sphere([0, 1, -5], [0, 0, 1], [0, 0, 0], 1.0)  # tangent
    assert t == pytest.approx(5.0)


TRI = [[0, 0, 0], [1, 0, 0], [0, 1, 0]]


@pytest.mark.parametrize("fn", ["f32", "f64"])
def test_watertight_basic(fn):
    f = oracle.intersect_tri if fn == "f32" else oracle.intersect_tri64
    assert f([0.25, 0.25, 1], [0, 0, -1], *TRI) == pytest.approx(1.0)
    assert f([0.25, 0.25, -1], [0, 0, 1], *TRI) == pytest.approx(1.0)  # back face
    assert f([0.75, 0.75, 1], [0, 0, -1], *TRI) is None
    assert f([0.25, 0.25, 1], [0, 0, 1], *TRI) is None  # behind
    assert f([0.2, 0.2, 0.0], [1, 0, 0], *TRI) is None  # in-plane ray
    assert f([0.25, 0.25, 1], [0, 0, -1], [0, 0, 0], [1, 1, 1], [2, 2, 2]) is None  # degenerate


def test_watertight_shared_edges_and_vertices():
    # a fan of triangles around a shared vertex: every ray through the fan
    # region hits at least one triangle -- including rays exactly through
    # the shared vertex and exactly along the shared edges
    c = np.array([0.3, 0.2, 0.0])
    ring = [np.array([math.cos(a), math.sin(a), 0.0]) * 2 + c for a in np.linspace(0, 2 * math.pi, 7)[:-1]]
    tris = [(c, ring[i], ring[(i + 1) % 6]) for i in range(6)]
    rng = np.random.default_rng(3)
    targets = [c] + [c + (r - c) * s for r in ring for s in (0.25, 0.5, 0.999)]
    targets += [c + rng.uniform(-1.2, 1.2, 3) * [1, 1, 0] for _ in range(200)]
    for tgt in targets:
        for o in ([0.1, 0.05, 3.0], [-1.3, 0.7, 2.0], [2.0, -1.0, -4.0]):
            o = np.array(o)
            d = tgt - o
            d /= np.linalg.norm(d)
            hits = [oracle.intersect_tri(o, d, *t) for t in tris]
            inside = np.linalg.norm((tgt - c)[:2]) < 1.6
            if inside:
                assert any(h is not None for h in hits), (tgt, o)


def test_watertight_mesh_closed_icosphere():
    # rays from inside a closed icosphere must hit it (no leaks)
    from minotert_gb300 import scene
    mesh = scene.icospheres(5, 1, 3, 1.0, 1.0, 0)
    center = mesh.verts.reshape(-1, 3).mean(0)
    n = 4000
    rng = np.random.default_rng(4)
    from minotert_gb300._lib import RAY_DTYPE
    rays = np.zeros(n, RAY_DTYPE)
    rays["org"] = center
    d = rng.normal(size=(n, 3))
    rays["dir"] = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    rays["tmax"] = np.inf
    hits = oracle.trace_brute(mesh.verts, rays)
    assert (hits["prim"] != MISS).all()


def test_bvh8_invariants(hf_workload):
    _, mesh, bvh = hf_workload
    info = oracle.bvh8_validate(bvh.nodes, bvh.tris, mesh.verts)
    assert info["error"] == 0
    assert info["depth"] == bvh.depth <= 32
    assert info["max_tris_per_node"] <= 24


def test_bvh8_traversal_equals_brute_force(hf_workload):
    _, mesh, bvh = hf_workload
    rays = random_rays(30000, mesh.lo, mesh.hi, seed=7)
    hb = oracle.trace_brute(mesh.verts, rays)
    hv, st = oracle.trace_bvh8(bvh.nodes, bvh.tris, rays)
    assert st == 0
    assert np.array_equal(hb["prim"], hv["prim"])
    assert np.array_equal(hb["t"], hv["t"])
    ab = oracle.trace_brute(mesh.verts, rays, any_hit=True)
    av, st = oracle.trace_bvh8(bvh.nodes, bvh.tris, rays, any_hit=True)
    assert np.array_equal(ab["prim"] == MISS, av["prim"] == MISS)


def test_bvh8_detects_corruption(hf_workload):
    # host-side fault injection: out-of-range child / triangle indices are
    # reported through the status bits, never by hanging or faulting
    _, mesh, bvh = hf_workload
    nodes = bvh.nodes.copy()
    nodes["child_base"][0] = len(nodes) + 100
    rays = random_rays(2000, mesh.lo, mesh.hi, seed=8)
    _, st = oracle.trace_bvh8(nodes, bvh.tris, rays)
    assert st & 4  # bad node
    nodes = bvh.nodes.copy()
    nodes["tri_base"][:] = len(bvh.tris) + 5
    _, st = oracle.trace_bvh8(nodes, bvh.tris, rays)
    assert st & 8  # bad triangle
    info = oracle.bvh8_validate(nodes, bvh.tris, mesh.verts)
    assert info["error"] != 0


def test_primary_regression_fixture(hf_workload):
    import hashlib
    wl, mesh, bvh = hf_workload
    c = wl.camera
    consts = oracle.camera_consts(c.position, c.yaw, c.pitch, c.verticalFov, c.nearPlane, wl.width, wl.height)
    p = oracle.primary(consts, wl.width, wl.height, bvh.nodes, bvh.tris, mesh.mats)
    g = GOLD["heightfield_boxes_256_primary"]
    for y, x, prim, t in g["samples"]:
        assert p["visibility"][y, x] == prim
        assert p["hit_t"][y, x] == np.float32(t)
    # the primary result does not depend on the BVH: brute force agrees
    assert hashlib.sha256(p["visibility"].tobytes()).hexdigest() == g["visibility_sha256"]
    assert hashlib.sha256(p["hit_t"].tobytes()).hexdigest() == g["hit_t_sha256"]


def test_fp32_and_fp64_pathtracers_agree(hf_workload, blue_noise):
    wl, mesh, bvh = hf_workload
    c = wl.camera
    consts = oracle.camera_consts(c.position, c.yaw, c.pitch, c.verticalFov, c.nearPlane, wl.width, wl.height)
    p = oracle.primary(consts, wl.width, wl.height, bvh.nodes, bvh.tris, mesh.mats)
    prm = oracle.params_array(1, 1, estimator=1, sun=np.float32(wl.sky.sun_dir) / np.linalg.norm(wl.sky.sun_dir),
                              sun_e=wl.sky.sun_irradiance, sky=wl.sky.radiance)
    y0, y1 = 96, 160
    c32, n32, st = oracle.pathtrace(bvh.nodes, bvh.tris, mesh.mats, consts, wl.width, wl.height, p["visibility"],
                                    p["hit_t"], blue_noise, prm, precision=32, y0=y0, y1=y1)
    c64, n64, _ = oracle.pathtrace(bvh.nodes, bvh.tris, mesh.mats, consts, wl.width, wl.height, p["visibility"],
                                   p["hit_t"], blue_noise, prm, precision=64, y0=y0, y1=y1)
    assert st == 0
    a, b = c32[y0:y1], c64[y0:y1]
    rmse = float(np.sqrt(np.mean((a - b) ** 2)))
    # same random numbers: only precision (and rare silhouette flips) differ
    assert rmse < 2e-3 * float(np.mean(b) + 1e-6) * 50
    assert np.mean(np.abs(a - b) < 1e-4) > 0.99
