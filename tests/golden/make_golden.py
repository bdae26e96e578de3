"""Generates tests/golden/known_answers.json.

Two kinds of vectors:
  * formula-derived known answers, computed here in pure Python / numpy
    float64 from the published formulas the reference's shaders use (PCG
    hash random.glsl:22-27, randomFloat :29-31, the camera matrices of
    math.ixx:822-861), independent of the C++ oracle;
  * regression fixtures produced by the oracle and the host modules for the
    seeded workloads (mesh hashes, BVH-independent primary-hit checksums),
    so drift on another host or after a change is caught.
The reference itself ships no tests or golden files; it cannot run here
(Vulkan + MSVC only), so these are the pins.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import math
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))


def pcg_py(v: int) -> int:
    m = 0xFFFFFFFF
    state = (v * 747796405 + 2891336453) & m
    word = (((state >> ((state >> 28) + 4)) ^ state) * 277803737) & m
    return ((word >> 22) ^ word) & m


def camera_f64(pos, yaw, pitch, fov, znear, w, h):
    d = np.array([math.cos(pitch) * math.cos(yaw), math.cos(pitch) * math.sin(yaw), math.sin(pitch)])
    up = np.array([0.0, 0.0, 1.0])
    s = np.cross(up, d)
    s /= np.linalg.norm(s)
    u = np.cross(d, s)
    p = np.asarray(pos, np.float64)
    view = np.eye(4)  # [col][row]
    view[0][0], view[1][0], view[2][0] = -s
    view[0][1], view[1][1], view[2][1] = u
    view[0][2], view[1][2], view[2][2] = d
    view[3][0], view[3][1], view[3][2] = s @ p, -(u @ p), -(d @ p)
    hh = 1.0 / math.tan(0.5 * fov)
    proj = np.zeros((4, 4))
    proj[0][0], proj[1][1], proj[2][3], proj[3][2] = hh * (h / w), hh, 1.0, znear
    # column-major flat: element [col][row] at col*4+row
    return view.reshape(-1), proj.reshape(-1)


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main():
    out = {}
    seq, v = [], 1
    for _ in range(32):
        v = pcg_py(v)
        seq.append(v)
    out["pcg_from_1"] = seq
    out["pcg_inputs"] = [0, 1, 2, 3, 0xFFFFFFFF, 0x12345678, 0xDEADBEEF]
    out["pcg_outputs"] = [pcg_py(x) for x in out["pcg_inputs"]]
    # randomFloat = (pcg & 0xFFFFFF) / 2^24, exact in float32
    out["random_float_from_3"] = []
    v = 3
    for _ in range(8):
        v = pcg_py(v)
        out["random_float_from_3"].append((v & 0xFFFFFF) / 16777216.0)

    # reference default camera (app.ixx:20-32) at the reference window size
    cam = dict(pos=(0.0, -0.001, 0.1), yaw=math.radians(90.0), pitch=0.0, fov=math.radians(60.0), znear=0.001,
               w=960, h=540)
    view, proj = camera_f64(**cam)
    out["reference_camera"] = {"args": cam, "view_f64": view.tolist(), "projection_f64": proj.tolist()}

    # regression fixtures from the host modules + oracle
    from minotert_gb300 import build, scene, workloads
    build.build()
    import oracle
    wl = workloads.heightfield_boxes_256()
    mesh = wl.mesh()
    out["heightfield_boxes_seed1"] = {"tris": mesh.tri_count, "verts_sha256": sha(mesh.verts),
                                      "mats_sha256": sha(mesh.mats)}
    ico = workloads.icospheres_1080p().mesh()
    out["icospheres_seed1"] = {"tris": ico.tri_count, "verts_sha256": sha(ico.verts), "mats_sha256": sha(ico.mats)}
    bn = scene.blue_noise(1, 64)
    out["blue_noise_seed1_64"] = {"sha256": sha(bn)}
    bvh = scene.build_bvh8(mesh)
    c = wl.camera
    consts = oracle.camera_consts(c.position, c.yaw, c.pitch, c.verticalFov, c.nearPlane, wl.width, wl.height)
    prim = oracle.primary(consts, wl.width, wl.height, bvh.nodes, bvh.tris, mesh.mats)
    out["heightfield_boxes_256_primary"] = {
        "visibility_sha256": sha(prim["visibility"]), "hit_t_sha256": sha(prim["hit_t"]),
        "hit_fraction": float((prim["visibility"] != 0xFFFFFFFF).mean()),
        "samples": [[int(y), int(x), int(prim["visibility"][y, x]), float(prim["hit_t"][y, x])]
                    for y, x in [(0, 0), (40, 200), (128, 128), (200, 30), (255, 255), (180, 90)]]}
    (Path(__file__).parent / "known_answers.json").write_text(json.dumps(out, indent=1))
    print("wrote known_answers.json")


if __name__ == "__main__":
    main()
