"""CPU oracle (test infrastructure only): ctypes wrapper of oracle.cpp.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this package, and only as the checker; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .build import OUT, build as build_oracle

_lib = None

HIT_DTYPE = np.dtype([("prim", "<u4"), ("t", "<f4")])


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = build_oracle()
        L = C.CDLL(str(path))
        vp, u32, i32, f32 = C.c_void_p, C.c_uint32, C.c_int, C.c_float
        sig = {
            "orc_pcg": ([u32], u32),
            "orc_random_float": ([C.POINTER(u32)], f32),
            "orc_rotated_random": ([C.POINTER(u32), f32], f32),
            "orc_random_sphere_point": ([f32, f32, vp], None),
            "orc_f2h": ([f32], C.c_uint16),
            "orc_h2f": ([C.c_uint16], f32),
            "orc_ray_sphere": ([vp, vp, vp, f32], f32),
            "orc_camera_consts": ([vp, f32, f32, f32, f32, u32, u32, vp, f32, f32, u32, vp], None),
            "orc_inverse4": ([vp, vp], None),
            "orc_intersect_tri": ([vp, vp, vp, vp, vp, f32, vp], i32),
            "orc_intersect_tri64": ([vp, vp, vp, vp, vp, C.c_double, vp], i32),
            "orc_trace_brute": ([vp, u32, vp, u32, vp, i32, i32], None),
            "orc_trace_bvh8": ([vp, u32, vp, u32, vp, u32, vp, i32, vp, vp, i32], u32),
            "orc_bvh8_validate": ([vp, u32, vp, u32, vp, u32, vp], None),
            "orc_primary": ([vp, u32, vp, u32, vp, vp, u32, vp, u32, u32, u32, u32, vp, vp, vp, vp, vp, i32], u32),
            "orc_secondary_spheres": ([vp, u32, vp, u32, u32, vp, vp, vp, vp, u32, u32, vp, vp, i32], None),
            "orc_pathtrace": ([vp, u32, vp, u32, vp, u32, vp, u32, u32, vp, vp, vp, u32, u32, vp, i32, u32, u32, vp,
                               vp, i32], u32),
            "orc_pathtrace_rays": ([vp, u32, vp, u32, vp, vp, u32, u32, vp, u32, vp, i32], u32),
        }
        for name, (args, res) in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def _p(a):
    return C.c_void_p(0) if a is None else C.c_void_p(a.ctypes.data)


def pcg(v: int) -> int:
    return lib().orc_pcg(v)


def random_float(state: int):
    s = C.c_uint32(state)
    f = lib().orc_random_float(C.byref(s))
    return f, s.value


def sphere_point(rx: float, ry: float) -> np.ndarray:
    out = np.zeros(3, np.float32)
    lib().orc_random_sphere_point(rx, ry, _p(out))
    return out


def f2h(x: float) -> int:
    return lib().orc_f2h(x)


def h2f(h: int) -> float:
    return lib().orc_h2f(h)


def ray_sphere(o, d, c, r) -> float:
    o, d, c = (np.asarray(v, np.float32) for v in (o, d, c))
    return lib().orc_ray_sphere(_p(o), _p(d), _p(c), r)


def camera_consts(pos, yaw, pitch, fov, znear, w, h, prev=None, frame=0) -> np.ndarray:
    """84 floats laid out as mrt_camera_consts (frame counter as uint32 bits)."""
    pos = np.asarray(pos, np.float32)
    ppos, pyaw, ppitch = (pos, yaw, pitch) if prev is None else (np.asarray(prev[0], np.float32), prev[1], prev[2])
    out = np.zeros(84, np.float32)
    lib().orc_camera_consts(_p(pos), yaw, pitch, fov, znear, w, h, _p(ppos), pyaw, ppitch, frame, _p(out))
    return out


def inverse4(m) -> np.ndarray:
    m = np.ascontiguousarray(m, np.float32)
    out = np.zeros(16, np.float32)
    lib().orc_inverse4(_p(m), _p(out))
    return out


def intersect_tri(o, d, v0, v1, v2, tmin=0.0):
    arr = [np.ascontiguousarray(v, np.float32) for v in (o, d, v0, v1, v2)]
    t = np.zeros(1, np.float32)
    hit = lib().orc_intersect_tri(*map(_p, arr), tmin, _p(t))
    return (float(t[0]) if hit else None)


def intersect_tri64(o, d, v0, v1, v2, tmin=0.0):
    o, d = np.ascontiguousarray(o, np.float64), np.ascontiguousarray(d, np.float64)
    vs = [np.ascontiguousarray(v, np.float32) for v in (v0, v1, v2)]
    t = np.zeros(1, np.float64)
    hit = lib().orc_intersect_tri64(_p(o), _p(d), *map(_p, vs), tmin, _p(t))
    return (float(t[0]) if hit else None)


def trace_brute(verts: np.ndarray, rays: np.ndarray, any_hit=False, threads=0) -> np.ndarray:
    verts = np.ascontiguousarray(verts, np.float32)
    rays = np.ascontiguousarray(rays)
    hits = np.zeros(len(rays), HIT_DTYPE)
    lib().orc_trace_brute(_p(verts), verts.shape[0], _p(rays), len(rays), _p(hits), int(any_hit), threads)
    return hits


def trace_bvh8(nodes, tris, rays, any_hit=False, counts=False, threads=0):
    rays = np.ascontiguousarray(rays)
    hits = np.zeros(len(rays), HIT_DTYPE)
    nv = np.zeros(len(rays), np.uint32) if counts else None
    tv = np.zeros(len(rays), np.uint32) if counts else None
    st = lib().orc_trace_bvh8(_p(nodes), len(nodes), _p(tris), len(tris), _p(rays), len(rays), _p(hits),
                              int(any_hit), _p(nv), _p(tv), threads)
    return (hits, st, nv, tv) if counts else (hits, st)


def bvh8_validate(nodes, tris, verts) -> dict:
    info = np.zeros(3, np.uint32)
    verts = np.ascontiguousarray(verts, np.float32)
    lib().orc_bvh8_validate(_p(nodes), len(nodes), _p(tris), len(tris), _p(verts), verts.shape[0], _p(info))
    return {"depth": int(info[0]), "max_tris_per_node": int(info[1]), "error": int(info[2])}


def primary(consts: np.ndarray, w: int, h: int, nodes=None, tris=None, mats=None, spheres=None, threads=0,
            y0=0, y1=None):
    """Returns dict of visibility, hit_t, depth(u16), normal(u16x4), motion(u16x2), status; rows [y0, y1)
    are computed (the rest stay zero)."""
    vis = np.zeros((h, w), np.uint32)
    ht = np.zeros((h, w), np.float32)
    dep = np.zeros((h, w), np.uint16)
    nrm = np.zeros((h, w, 4), np.uint16)
    mot = np.zeros((h, w, 2), np.uint16)
    ns = 0 if spheres is None else len(spheres)
    st = lib().orc_primary(_p(nodes), 0 if nodes is None else len(nodes), _p(tris), 0 if tris is None else len(tris),
                           _p(mats), _p(spheres), ns, _p(consts), w, h, y0, h if y1 is None else y1, _p(vis), _p(ht),
                           _p(dep), _p(nrm), _p(mot), threads)
    return {"visibility": vis, "hit_t": ht, "depth": dep, "normal": nrm, "motion": mot, "status": st}


def params_array(samples, bounces, rr_start=0, rng_mode=0, estimator=0, accumulate=0, frame_index=0,
                 sun=(0, 0, 1), sun_e=(0, 0, 0), sky=(0, 0, 0)) -> np.ndarray:
    """80 bytes laid out as mrt_trace_params."""
    a = np.zeros(20, np.uint32)
    a[:8] = [samples, bounces, rr_start, rng_mode, estimator, accumulate, frame_index, 0]
    f = a.view(np.float32)
    f[8:11] = sun
    f[12:15] = sun_e
    f[16:19] = sky
    return a


def secondary_spheres(spheres, consts, w, h, vis, depth, normal, bn_rgba, params, color=None, threads=0):
    color = np.zeros((h, w, 3), np.float32) if color is None else color
    bn = np.ascontiguousarray(bn_rgba, np.uint8)
    lib().orc_secondary_spheres(_p(spheres), len(spheres), _p(consts), w, h, _p(np.ascontiguousarray(vis)),
                                _p(np.ascontiguousarray(depth)), _p(np.ascontiguousarray(normal)), _p(bn),
                                bn.shape[1], bn.shape[0], _p(params), _p(color), threads)
    return color


def pathtrace(nodes, tris, mats, consts, w, h, vis, hit_t, bn_rgba, params, precision=32, y0=0, y1=None,
              color=None, threads=0):
    color = np.zeros((h, w, 3), np.float32) if color is None else color
    counts = np.zeros(3, np.uint64)
    bn = np.ascontiguousarray(bn_rgba, np.uint8)
    st = lib().orc_pathtrace(_p(nodes), len(nodes), _p(tris), len(tris), _p(mats), len(mats), _p(consts), w, h,
                             _p(np.ascontiguousarray(vis)), _p(np.ascontiguousarray(hit_t)), _p(bn), bn.shape[1],
                             bn.shape[0], _p(params), precision, y0, h if y1 is None else y1, _p(color), _p(counts),
                             threads)
    return color, counts, st


def pathtrace_rays(nodes, tris, mats, rays, params, frame=0, index_base=0, threads=0):
    """Batched bounce loop for the rays of one scene; returns (radiance (n,3), status)."""
    rays = np.ascontiguousarray(rays)
    rad = np.zeros((len(rays), 3), np.float32)
    st = lib().orc_pathtrace_rays(_p(nodes), len(nodes), _p(tris), len(tris), _p(mats), _p(rays), len(rays),
                                  index_base, _p(params), frame, _p(rad), threads)
    return rad, st
