"""CPU oracle (test infrastructure only): wrappers of post.cpp -- the sky /
atmosphere LUTs and miss shader, the joint bilateral filter, the
tonemappers and temporal reprojection.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module, and only as the checker.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import lib as _base_lib

_done = False

TRANS_SHAPE = (64, 256, 4)
MS_SHAPE = (32, 32, 4)
VIEW_SHAPE = (108, 192, 4)

# mrt_atmosphere_params field order (28 floats)
ATMO_FIELDS = [
    ("bottom_radius", 1), ("top_radius", 1), ("rayleigh_density_exp_scale", 1), ("rayleigh_scattering", 3),
    ("mie_density_exp_scale", 1), ("mie_scattering", 3), ("mie_extinction", 3), ("mie_absorption", 3),
    ("mie_phase_g", 1), ("absorption_density0_layer_width", 1), ("absorption_density0_constant_term", 1),
    ("absorption_density0_linear_term", 1), ("absorption_density1_constant_term", 1),
    ("absorption_density1_linear_term", 1), ("absorption_extinction", 3), ("ground_albedo", 3),
]


def lib() -> C.CDLL:
    global _done
    L = _base_lib()
    if not _done:
        vp, u32, f32, i32 = C.c_void_p, C.c_uint32, C.c_float, C.c_int
        sig = {
            "orc_sky_transmittance": ([vp, vp], None),
            "orc_sky_multiscatter": ([vp, vp, vp], None),
            "orc_sky_view": ([vp, vp, vp, vp, vp, vp, vp], None),
            "orc_sky_color": ([vp, vp, vp, vp, vp, vp, vp, u32, vp], None),
            "orc_sky_bind": ([vp, vp, vp, vp, vp, vp], None),
            "orc_bilateral": ([vp, vp, vp, u32, u32, f32, f32, f32, f32, u32, i32, vp], i32),
            "orc_tonemap": ([vp, u32, u32, vp, vp], None),
            "orc_reproject": ([vp, u32, u32, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, f32, f32, f32, vp, vp], None),
        }
        for name, (args, res) in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _done = True
    return L


def _p(a):
    return C.c_void_p(0) if a is None else C.c_void_p(a.ctypes.data)


def _f32(a, n=None):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    if n is not None:
        assert a.size == n
    return a


def earth() -> np.ndarray:
    """Atmosphere::Params::earth() (sky.ixx:59-83) as 28 float32s."""
    f = np.float32  # the reference evaluates these in float
    mie_s = [f(0.003996)] * 3
    mie_e = [f(0.004440)] * 3
    vals = {
        "bottom_radius": 6360.0, "top_radius": 6460.0, "rayleigh_density_exp_scale": f(-1.0) / f(8.0),
        "rayleigh_scattering": [0.005802, 0.013558, 0.033100], "mie_density_exp_scale": f(-1.0) / f(1.2),
        "mie_scattering": mie_s, "mie_extinction": mie_e,
        "mie_absorption": [max(e - s, f(0.0)) for e, s in zip(mie_e, mie_s)],
        "mie_phase_g": 0.8, "absorption_density0_layer_width": 25.0,
        "absorption_density0_constant_term": f(-2.0) / f(3.0), "absorption_density0_linear_term": f(1.0) / f(15.0),
        "absorption_density1_constant_term": f(8.0) / f(3.0), "absorption_density1_linear_term": f(-1.0) / f(15.0),
        "absorption_extinction": [0.000650, 0.001881, 0.000085], "ground_albedo": [0.0, 0.0, 0.0],
    }
    out = []
    for name, n in ATMO_FIELDS:
        v = vals[name]
        out += list(v) if n > 1 else [v]
    return np.array(out, np.float32)


def sky_transmittance(atmo) -> np.ndarray:
    a = _f32(atmo, 28)
    out = np.zeros(TRANS_SHAPE, np.float32)
    lib().orc_sky_transmittance(_p(a), _p(out))
    return out


def sky_multiscatter(atmo, trans) -> np.ndarray:
    a = _f32(atmo, 28)
    t = _f32(trans)
    out = np.zeros(MS_SHAPE, np.float32)
    lib().orc_sky_multiscatter(_p(a), _p(t), _p(out))
    return out


def sky_view(atmo, trans, ms, probe, sun_dir, sun_illuminance) -> np.ndarray:
    a = _f32(atmo, 28)
    t, m, pr, sd, se = _f32(trans), _f32(ms), _f32(probe, 3), _f32(sun_dir, 3), _f32(sun_illuminance, 3)
    out = np.zeros(VIEW_SHAPE, np.float32)
    lib().orc_sky_view(_p(a), _p(t), _p(m), _p(pr), _p(sd), _p(se), _p(out))
    return out


def sky_color(atmo, trans, view, cam, sun_dir, sun_illuminance, dirs) -> np.ndarray:
    a = _f32(atmo, 28)
    d = _f32(dirs).reshape(-1, 3)
    t, v, c, sd, se = _f32(trans), _f32(view), _f32(cam, 3), _f32(sun_dir, 3), _f32(sun_illuminance, 3)
    out = np.zeros_like(d)
    lib().orc_sky_color(_p(a), _p(t), _p(v), _p(c), _p(sd), _p(se), _p(d), d.shape[0], _p(out))
    return out


_bound = None


def bind_sky(atmo=None, trans=None, view=None, cam=None, sun_dir=None, sun_illuminance=None):
    """Escaping paths of the FP32 path-tracing oracle see this sky (like
    mrt_cuda_set_sky); bind_sky() restores the constant sky."""
    global _bound
    if atmo is None:
        lib().orc_sky_bind(None, None, None, None, None, None)
        _bound = None
        return
    arrs = [_f32(atmo, 28), _f32(trans, 256 * 64 * 4), _f32(view, 192 * 108 * 4), _f32(cam, 3), _f32(sun_dir, 3),
            _f32(sun_illuminance, 3)]
    lib().orc_sky_bind(*[_p(a) for a in arrs])
    _bound = arrs


def _half_to_f32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, np.uint16).view(np.float16).astype(np.float32))


def bilateral(color, depth_h, normal_h, sigma=5.0, k_sigma=2.0, threshold=0.12, near_plane=1.0, frame=0,
              dither=True) -> np.ndarray:
    """bilateral.comp over float RGB (H, W, 3) with the g-buffer's R16F depth
    (H, W) and RGBA16F normal (H, W, 4) as uint16 bit patterns."""
    c = _f32(color)
    h, w = c.shape[:2]
    z = _half_to_f32(depth_h).reshape(h, w)
    n = np.ascontiguousarray(_half_to_f32(normal_h).reshape(h, w, 4)[..., :3])
    out = np.zeros((h, w, 3), np.float32)
    rc = lib().orc_bilateral(_p(c), _p(z), _p(n), w, h, sigma, k_sigma, threshold, near_plane, frame, int(dither),
                             _p(out))
    if rc != 0:
        raise ValueError("bilateral radius out of range")
    return out


TONEMAP_MODES = {"linear": 0, "reinhard": 1, "hable": 2, "aces": 3, "uchimura": 4, "amd": 5}


def tonemap_params(exposure=1.0, reinhard_max=8.0, uchimura=(1.0, 1.0, 0.22, 0.4, 1.33, 0.0),
                   amd=(16.0, 2.0, 1.0, 0.18, 0.18)) -> np.ndarray:
    return np.array([exposure, reinhard_max, *uchimura, *amd], np.float32)


def tonemap(color, mode, params=None) -> np.ndarray:
    c = _f32(color)
    n = c.size // 3
    prm = tonemap_params() if params is None else _f32(params, 13)
    m = TONEMAP_MODES[mode] if isinstance(mode, str) else int(mode)
    out = np.zeros(c.shape[:-1] + (4,), np.uint8)
    lib().orc_tonemap(_p(c), n, m, _p(prm), _p(out))
    return out


def reproject(consts, w, h, vis, hit_t, normal, motion, pvis, pdepth, pnormal, sample, hist, hist_len,
              max_history=32.0, normal_cos=0.9, depth_rel=0.05):
    arrs = [np.ascontiguousarray(consts), np.ascontiguousarray(vis, np.uint32), _f32(hit_t),
            np.ascontiguousarray(normal, np.uint16), np.ascontiguousarray(motion, np.uint16),
            np.ascontiguousarray(pvis, np.uint32), np.ascontiguousarray(pdepth, np.uint16),
            np.ascontiguousarray(pnormal, np.uint16), _f32(sample), _f32(hist), _f32(hist_len)]
    out = np.zeros((h, w, 3), np.float32)
    out_len = np.zeros((h, w), np.float32)
    lib().orc_reproject(_p(arrs[0]), w, h, *[_p(a) for a in arrs[1:]], max_history, normal_cos, depth_rel,
                        _p(out), _p(out_len))
    return out, out_len


def exp_cw(x) -> np.ndarray:
    """The deterministic e^x shared with the CUDA kernels, elementwise."""
    L = lib()
    if not hasattr(L.orc_exp_cw, "_set"):
        L.orc_exp_cw.argtypes = [C.c_float]
        L.orc_exp_cw.restype = C.c_float
        L.orc_exp_cw._set = True
    xs = np.asarray(x, np.float32).ravel()
    return np.array([L.orc_exp_cw(float(v)) for v in xs], np.float32).reshape(np.shape(x))
