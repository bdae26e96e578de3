"""ctypes binding of libmrt.so (include/mrt_cuda.h, include/mrt_host.h).

The library is built in-tree by minotert_gb300.build; loading fails loudly
when it is missing -- there is no CPU fallback for any device entry point.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libmrt.so"

MRT_OK, MRT_EINVAL, MRT_ECUDA, MRT_ENOMEM, MRT_ETIMEOUT, MRT_EDEVICE, MRT_ESTATE, MRT_ERANGE = 0, -1, -2, -3, -4, -5, -6, -7
MRT_STATUS_ITER_CAP, MRT_STATUS_STACK_OVF, MRT_STATUS_BAD_NODE, MRT_STATUS_BAD_TRI = 1, 2, 4, 8
MRT_STATUS_QUEUE_OVF, MRT_STATUS_BAD_SCENE, MRT_STATUS_PIPE_TIMEOUT = 0x10, 0x20, 0x40
MRT_MISS = 0xFFFFFFFF
MRT_RNG_REFERENCE, MRT_RNG_PER_PIXEL = 0, 1
MRT_EST_ESCAPE, MRT_EST_NEE = 0, 1
MRT_TRACE_ANY_HIT = 1
MRT_MAX_BOUNCES = 16

_ERR_NAMES = {0: "MRT_OK", -1: "MRT_EINVAL", -2: "MRT_ECUDA", -3: "MRT_ENOMEM", -4: "MRT_ETIMEOUT",
              -5: "MRT_EDEVICE", -6: "MRT_ESTATE", -7: "MRT_ERANGE"}

# numpy dtypes with the exact C layouts
NODE_DTYPE = np.dtype([("origin", "<f4", 3), ("exp", "i1", 3), ("imask", "u1"), ("child_base", "<u4"),
                       ("tri_base", "<u4"), ("meta", "u1", 8), ("q_lo", "u1", (3, 8)), ("q_hi", "u1", (3, 8)),
                       ("reserved", "<u4", 12)])
TRI_DTYPE = np.dtype([("v0", "<f4", 3), ("id", "<u4"), ("v1", "<f4", 3), ("pad1", "<u4"), ("v2", "<f4", 3),
                      ("pad2", "<u4")])
MAT_DTYPE = np.dtype([("normal", "<f4", 3), ("albedo", "<u4")])
SPHERE_DTYPE = np.dtype([("center", "<f4", 3), ("radius", "<f4"), ("albedo", "<f4", 3), ("pad", "<f4")])
RAY_DTYPE = np.dtype([("org", "<f4", 3), ("tmin", "<f4"), ("dir", "<f4", 3), ("tmax", "<f4")])
HIT_DTYPE = np.dtype([("prim", "<u4"), ("t", "<f4")])
assert NODE_DTYPE.itemsize == 128 and TRI_DTYPE.itemsize == 48 and MAT_DTYPE.itemsize == 16
assert SPHERE_DTYPE.itemsize == 32 and RAY_DTYPE.itemsize == 32 and HIT_DTYPE.itemsize == 8


class CameraConsts(C.Structure):
    _fields_ = [("view", C.c_float * 16), ("projection", C.c_float * 16), ("inv_view", C.c_float * 16),
                ("inv_projection", C.c_float * 16), ("prev_view", C.c_float * 16), ("camera_pos", C.c_float * 3),
                ("frame_counter", C.c_uint32)]


class GBuffer(C.Structure):
    _fields_ = [("visibility", C.c_void_p), ("hit_t", C.c_void_p), ("depth", C.c_void_p), ("normal", C.c_void_p),
                ("motion", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32)]


class TraceParams(C.Structure):
    _fields_ = [("samples", C.c_uint32), ("max_bounces", C.c_uint32), ("rr_start", C.c_uint32),
                ("rng_mode", C.c_uint32), ("estimator", C.c_uint32), ("accumulate", C.c_uint32),
                ("frame_index", C.c_uint32), ("sort_rays", C.c_uint32), ("sun_dir", C.c_float * 3),
                ("exact_trig", C.c_uint32), ("sun_irradiance", C.c_float * 3), ("pad1", C.c_float),
                ("sky_radiance", C.c_float * 3), ("pad2", C.c_float)]


class FrameStats(C.Structure):
    _fields_ = [("primary_rays", C.c_uint64), ("extension_rays", C.c_uint64 * MRT_MAX_BOUNCES),
                ("shadow_rays", C.c_uint64), ("nodes_primary", C.c_uint64), ("tris_primary", C.c_uint64),
                ("nodes_extension", C.c_uint64 * MRT_MAX_BOUNCES), ("tris_extension", C.c_uint64 * MRT_MAX_BOUNCES),
                ("nodes_shadow", C.c_uint64), ("tris_shadow", C.c_uint64), ("ms_primary", C.c_float), ("ms_extend", C.c_float),
                ("ms_extend_b", C.c_float * MRT_MAX_BOUNCES), ("ms_shadow", C.c_float), ("ms_shade", C.c_float),
                ("ms_sort", C.c_float), ("ms_total", C.c_float), ("ms_cache_train", C.c_float),
                ("ms_cache_infer", C.c_float), ("launches", C.c_uint32), ("pad", C.c_uint32)]


class Tuning(C.Structure):
    _fields_ = [("trace_blocks_per_sm", C.c_uint32), ("dynamic_fetch", C.c_uint32),
                ("primary_persistent", C.c_uint32), ("sort_min_rays", C.c_uint32), ("tail_bounce", C.c_uint32),
                ("stack_depth", C.c_uint32), ("tri_spread", C.c_uint32), ("refill_min", C.c_uint32),
                ("overlap_shadow", C.c_uint32), ("tail_from_hits", C.c_uint32)]


class CacheConfig(C.Structure):
    _fields_ = [("log2_table", C.c_uint32), ("base_res", C.c_float), ("max_res", C.c_float), ("lr_grid", C.c_float),
                ("lr_mlp", C.c_float), ("seed", C.c_uint32), ("train_paths", C.c_uint32), ("train_steps", C.c_uint32),
                ("train_bounces", C.c_uint32), ("query_vertex", C.c_uint32)]


class DeviceInfo(C.Structure):
    _fields_ = [("name", C.c_char * 96), ("sm_count", C.c_int32), ("cc_major", C.c_int32), ("cc_minor", C.c_int32),
                ("trace_blocks_per_sm_max", C.c_uint32), ("total_mem", C.c_uint64), ("l2_bytes", C.c_uint64)]


class Camera_C(C.Structure):
    _fields_ = [("viewport", C.c_uint32 * 2), ("vertical_fov", C.c_float), ("near_plane", C.c_float),
                ("position", C.c_float * 3), ("yaw", C.c_float), ("pitch", C.c_float)]


class Mesh_C(C.Structure):
    _fields_ = [("verts", C.POINTER(C.c_float)), ("materials", C.c_void_p), ("tri_count", C.c_uint32),
                ("pad", C.c_uint32), ("bounds_lo", C.c_float * 3), ("bounds_hi", C.c_float * 3)]


class BvhBuildParams(C.Structure):
    _fields_ = [("sah_bins", C.c_uint32), ("max_leaf_tris", C.c_uint32), ("threads", C.c_uint32),
                ("trav_cost_pct", C.c_uint32), ("collapse", C.c_uint32), ("prim_cost_pct", C.c_uint32)]


class Bvh8_C(C.Structure):
    _fields_ = [("nodes", C.c_void_p), ("tris", C.c_void_p), ("node_count", C.c_uint32), ("tri_count", C.c_uint32),
                ("depth", C.c_uint32), ("leaf_count", C.c_uint32), ("build_ms", C.c_double), ("sah_cost", C.c_double)]


class BilateralParams(C.Structure):
    _fields_ = [("sigma", C.c_float), ("k_sigma", C.c_float), ("threshold", C.c_float), ("near_plane", C.c_float),
                ("frame_counter", C.c_uint32), ("dither", C.c_uint32)]


class TonemapParams(C.Structure):
    _fields_ = [("mode", C.c_uint32), ("exposure", C.c_float), ("reinhard_max", C.c_float),
                ("uchimura", C.c_float * 6), ("amd", C.c_float * 5)]


class ReprojectParams(C.Structure):
    _fields_ = [("max_history", C.c_float), ("normal_cos", C.c_float), ("depth_rel", C.c_float),
                ("pad", C.c_float)]


assert C.sizeof(CameraConsts) == 84 * 4 and C.sizeof(TraceParams) == 80
assert C.sizeof(BilateralParams) == 24 and C.sizeof(TonemapParams) == 56 and C.sizeof(ReprojectParams) == 16


class MrtError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{_ERR_NAMES.get(code, code)}: {msg}")
        self.code = code


_lib = None


def lib() -> C.CDLL:
    """The loaded libmrt.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m minotert_gb300.build` "
                               "(there is no CPU fallback)")
        L = C.CDLL(str(LIB_PATH))
        vp, u32, i32, sz = C.c_void_p, C.c_uint32, C.c_int, C.c_size_t
        pp = C.POINTER(C.c_void_p)
        sig = {
            "mrt_cuda_abi_version": ([], i32),
            "mrt_cuda_create": ([pp, i32], i32),
            "mrt_cuda_destroy": ([vp], i32),
            "mrt_cuda_last_error": ([vp], C.c_char_p),
            "mrt_cuda_status": ([vp, C.POINTER(u32), i32], i32),
            "mrt_cuda_sync": ([vp, vp, C.c_double], i32),
            "mrt_cuda_set_timing": ([vp, i32], i32),
            "mrt_cuda_set_counters": ([vp, i32], i32),
            "mrt_cuda_set_tuning": ([vp, C.POINTER(Tuning)], i32),
            "mrt_cuda_get_tuning": ([vp, C.POINTER(Tuning)], i32),
            "mrt_cuda_device_info": ([vp, C.POINTER(DeviceInfo)], i32),
            "mrt_cuda_frame_stats": ([vp, C.POINTER(FrameStats)], i32),
            "mrt_cuda_read_sweep": ([vp, vp, sz, u32, vp, u32, vp], i32),
            "mrt_cuda_alloc": ([vp, sz, pp], i32),
            "mrt_cuda_free": ([vp, vp], i32),
            "mrt_cuda_host_alloc": ([vp, sz, pp], i32),
            "mrt_cuda_host_free": ([vp, vp], i32),
            "mrt_cuda_copy_h2d": ([vp, vp, vp, sz, vp], i32),
            "mrt_cuda_copy_d2h": ([vp, vp, vp, sz, vp], i32),
            "mrt_cuda_copy_d2d": ([vp, vp, vp, sz, vp], i32),
            "mrt_cuda_memset": ([vp, vp, i32, sz, vp], i32),
            "mrt_cuda_stream_create": ([vp, pp], i32),
            "mrt_cuda_stream_destroy": ([vp, vp], i32),
            "mrt_cuda_event_create": ([vp, pp], i32),
            "mrt_cuda_event_destroy": ([vp, vp], i32),
            "mrt_cuda_event_record": ([vp, vp, vp], i32),
            "mrt_cuda_event_elapsed": ([vp, vp, vp, C.POINTER(C.c_float)], i32),
            "mrt_cuda_scene_upload_triangles": ([vp, vp, u32, vp, u32, vp, u32, pp], i32),
            "mrt_cuda_scene_upload_spheres": ([vp, vp, u32, pp], i32),
            "mrt_cuda_scene_destroy": ([vp, vp], i32),
            "mrt_cuda_blue_noise_upload": ([vp, vp, u32, u32], i32),
            "mrt_cuda_primary_rays": ([vp, vp, C.POINTER(CameraConsts), C.POINTER(GBuffer), vp], i32),
            "mrt_cuda_secondary_rays": ([vp, vp, C.POINTER(GBuffer), C.POINTER(CameraConsts),
                                         C.POINTER(TraceParams), vp, vp], i32),
            "mrt_cuda_trace_rays": ([vp, vp, vp, u32, vp, u32, vp], i32),
            "mrt_cuda_trace_rays_counted": ([vp, vp, vp, u32, vp, vp, vp, vp], i32),
            "mrt_cuda_render_frame_host": ([vp, vp, C.POINTER(CameraConsts), C.POINTER(TraceParams), u32, u32,
                                            vp, vp, vp, vp], i32),
            "mrt_cuda_render_frame_host_async": ([vp, vp, C.POINTER(CameraConsts), C.POINTER(TraceParams), u32,
                                                  u32, vp, vp], i32),
            "mrt_cuda_frames_wait": ([vp], i32),
            "mrt_cuda_primary_rays_noalloc": ([vp, u32, vp, u32, vp, u32, C.POINTER(CameraConsts),
                                               C.POINTER(GBuffer), vp, vp], i32),
            "mrt_cuda_cache_create": ([vp, C.POINTER(CacheConfig), pp], i32),
            "mrt_cuda_cache_destroy": ([vp, vp], i32),
            "mrt_cuda_cache_set_bounds": ([vp, vp, C.POINTER(C.c_float), C.POINTER(C.c_float)], i32),
            "mrt_cuda_cache_infer": ([vp, vp, vp, u32, vp, vp], i32),
            "mrt_cuda_cache_train_step": ([vp, vp, vp, vp, u32, i32, C.POINTER(C.c_float), vp], i32),
            "mrt_cuda_cache_params": ([vp, vp, i32, vp, sz, i32], i32),
            "mrt_cuda_cache_frame": ([vp, vp, vp, C.POINTER(GBuffer), C.POINTER(CameraConsts), C.POINTER(TraceParams),
                                      vp, i32, vp], i32),
            "mrt_cuda_denoiser_create": ([vp, u32, pp], i32),
            "mrt_cuda_denoiser_destroy": ([vp, vp], i32),
            "mrt_cuda_denoiser_param_count": ([vp, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)], i32),
            "mrt_cuda_denoiser_set_tcgen05": ([vp, i32], i32),
            "mrt_cuda_cache_set_tcgen05": ([vp, i32], i32),
            "mrt_cuda_cache_set_overlap": ([vp, i32], i32),
            "mrt_cuda_denoiser_features": ([vp, vp, C.POINTER(GBuffer), vp, C.c_float, vp, vp], i32),
            "mrt_cuda_denoiser_infer": ([vp, vp, vp, u32, u32, u32, vp, vp], i32),
            "mrt_cuda_denoiser_train_step": ([vp, vp, vp, vp, u32, u32, u32, C.c_float, i32, C.POINTER(C.c_float),
                                              vp], i32),
            "mrt_cuda_denoiser_params": ([vp, vp, i32, vp, sz, i32], i32),
            "mrt_atmosphere_earth": ([vp], None),
            "mrt_cuda_sky_create": ([vp, pp], i32),
            "mrt_cuda_sky_destroy": ([vp, vp], i32),
            "mrt_cuda_sky_atmosphere": ([vp, vp, vp, vp], i32),
            "mrt_cuda_sky_view": ([vp, vp, vp, vp, vp, vp], i32),
            "mrt_cuda_sky_lut": ([vp, vp, i32, vp, sz], i32),
            "mrt_cuda_sky_eval": ([vp, vp, vp, vp, u32, vp, vp], i32),
            "mrt_cuda_set_sky": ([vp, vp], i32),
            "mrt_bilateral_defaults": ([C.POINTER(BilateralParams)], None),
            "mrt_cuda_bilateral": ([vp, C.POINTER(GBuffer), vp, C.POINTER(BilateralParams), vp, vp], i32),
            "mrt_tonemap_defaults": ([C.POINTER(TonemapParams)], None),
            "mrt_cuda_tonemap": ([vp, vp, u32, u32, C.POINTER(TonemapParams), vp, vp], i32),
            "mrt_cuda_reproject": ([vp, C.POINTER(GBuffer), C.POINTER(GBuffer), C.POINTER(CameraConsts), vp, vp, vp,
                                    C.POINTER(ReprojectParams), vp, vp, vp], i32),
            "mrt_cuda_batch_create": ([vp, u32, vp, vp, vp, vp, vp, pp], i32),
            "mrt_cuda_batch_destroy": ([vp, vp], i32),
            "mrt_cuda_batch_trace": ([vp, vp, vp, vp, vp, u32, vp], i32),
            "mrt_cuda_batch_pathtrace": ([vp, vp, vp, vp, C.POINTER(TraceParams), u32, vp, i32, vp], i32),
            "mrt_cuda_accumulate_copies": ([vp, vp, vp, u32, u32, C.c_size_t, C.c_float, vp], i32),
            # host modules
            "mrt_camera_view": ([C.POINTER(Camera_C), C.POINTER(C.c_float)], None),
            "mrt_camera_projection": ([C.POINTER(Camera_C), C.POINTER(C.c_float)], None),
            "mrt_mat4_inverse": ([C.POINTER(C.c_float), C.POINTER(C.c_float)], None),
            "mrt_camera_consts_make": ([C.POINTER(Camera_C), C.POINTER(Camera_C), u32, C.POINTER(CameraConsts)],
                                       None),
            "mrt_mesh_free": ([C.POINTER(Mesh_C)], None),
            "mrt_scene_heightfield_boxes": ([C.c_uint64, u32, u32, C.POINTER(Mesh_C)], i32),
            "mrt_scene_icospheres": ([C.c_uint64, u32, u32, C.c_float, C.c_float, u32, C.POINTER(Mesh_C)], i32),
            "mrt_heightfield_grid_for": ([u32], u32),
            "mrt_bvh8_build": ([vp, u32, C.POINTER(BvhBuildParams), C.POINTER(Bvh8_C)], i32),
            "mrt_bvh8_free": ([C.POINTER(Bvh8_C)], None),
            "mrt_scene_reference": ([vp], u32),
            "mrt_camera_reference": ([u32, u32, C.POINTER(Camera_C)], None),
            "mrt_blue_noise_generate": ([u32, u32, vp], i32),
            "mrt_png_decode_rgba8": ([vp, sz, vp, sz, C.POINTER(u32), C.POINTER(u32)], i32),
            "mrt_png_load_rgba8": ([C.c_char_p, vp, sz, C.POINTER(u32), C.POINTER(u32)], i32),
        }
        for name, (args, res) in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def ptr(a) -> C.c_void_p:
    """Address of a numpy array's data (or an int device pointer)."""
    if a is None:
        return C.c_void_p(0)
    if isinstance(a, (int, np.integer)):
        return C.c_void_p(int(a))
    if isinstance(a, DeviceBuffer):
        return C.c_void_p(a.ptr)
    return C.c_void_p(a.ctypes.data)


class Context:
    """An mrt_ctx on one CUDA device (mrt_cuda_create / mrt_cuda_destroy)."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        rc = lib().mrt_cuda_create(C.byref(self._h), device)
        if rc != MRT_OK:
            raise MrtError(rc, f"mrt_cuda_create(device={device}) failed")
        self.device = device

    @property
    def handle(self):
        return self._h

    def check(self, rc: int, what: str = ""):
        if rc != MRT_OK:
            msg = lib().mrt_cuda_last_error(self._h)
            raise MrtError(rc, f"{what}: {msg.decode() if msg else ''}")

    def close(self):
        if self._h:
            lib().mrt_cuda_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # memory
    def alloc(self, nbytes: int) -> "DeviceBuffer":
        p = C.c_void_p()
        self.check(lib().mrt_cuda_alloc(self._h, nbytes, C.byref(p)), "alloc")
        return DeviceBuffer(self, p.value or 0, nbytes)

    def to_device(self, arr: np.ndarray, stream=None) -> "DeviceBuffer":
        arr = np.ascontiguousarray(arr)
        buf = self.alloc(max(arr.nbytes, 1))
        buf.upload(arr, stream)
        return buf

    def status(self, clear: bool = True) -> int:
        f = C.c_uint32()
        self.check(lib().mrt_cuda_status(self._h, C.byref(f), 1 if clear else 0), "status")
        return f.value

    def sync(self, stream=None, timeout_s: float = 0.0):
        self.check(lib().mrt_cuda_sync(self._h, ptr(stream), timeout_s), "sync")

    def set_timing(self, on: bool):
        self.check(lib().mrt_cuda_set_timing(self._h, 1 if on else 0), "set_timing")

    def device_info(self) -> DeviceInfo:
        d = DeviceInfo()
        self.check(lib().mrt_cuda_device_info(self._h, C.byref(d)), "device_info")
        return d

    def tuning(self) -> Tuning:
        t = Tuning()
        self.check(lib().mrt_cuda_get_tuning(self._h, C.byref(t)), "get_tuning")
        return t

    def set_tuning(self, **kw):
        t = self.tuning()
        for k, v in kw.items():
            setattr(t, k, int(v))
        self.check(lib().mrt_cuda_set_tuning(self._h, C.byref(t)), "set_tuning")

    def set_counters(self, on: bool):
        self.check(lib().mrt_cuda_set_counters(self._h, 1 if on else 0), "set_counters")

    def set_sky(self, view):
        """Escaping paths see `view` (a sky.SkyView); None: the constant
        sky_radiance of the trace parameters."""
        self.check(lib().mrt_cuda_set_sky(self._h, None if view is None else view.handle), "set_sky")
        self._sky = view  # keeps the LUTs alive while bound

    def frame_stats(self) -> FrameStats:
        st = FrameStats()
        self.check(lib().mrt_cuda_frame_stats(self._h, C.byref(st)), "frame_stats")
        return st

    def blue_noise(self, rgba: np.ndarray):
        rgba = np.ascontiguousarray(rgba, dtype=np.uint8)
        h, w = rgba.shape[:2]
        self.check(lib().mrt_cuda_blue_noise_upload(self._h, ptr(rgba), w, h), "blue_noise_upload")

    def stream(self):
        s = C.c_void_p()
        self.check(lib().mrt_cuda_stream_create(self._h, C.byref(s)), "stream_create")
        return s.value

    def event(self):
        e = C.c_void_p()
        self.check(lib().mrt_cuda_event_create(self._h, C.byref(e)), "event_create")
        return e.value

    def record(self, ev, stream=None):
        self.check(lib().mrt_cuda_event_record(self._h, C.c_void_p(ev), ptr(stream)), "event_record")

    def elapsed_ms(self, a, b) -> float:
        ms = C.c_float()
        self.check(lib().mrt_cuda_event_elapsed(self._h, C.c_void_p(a), C.c_void_p(b), C.byref(ms)), "elapsed")
        return ms.value

    def host_alloc(self, shape, dtype) -> np.ndarray:
        """Pinned host array (freed with the context's lifetime of the array owner)."""
        dt = np.dtype(dtype)
        n = int(np.prod(shape)) * dt.itemsize
        p = C.c_void_p()
        self.check(lib().mrt_cuda_host_alloc(self._h, max(n, 1), C.byref(p)), "host_alloc")
        buf = (C.c_char * max(n, 1)).from_address(p.value)
        arr = np.frombuffer(buf, dtype=dt, count=int(np.prod(shape))).reshape(shape)
        return arr


class DeviceBuffer:
    def __init__(self, ctx: Context, p: int, nbytes: int):
        self.ctx, self.ptr, self.nbytes = ctx, p, nbytes

    def upload(self, arr: np.ndarray, stream=None):
        arr = np.ascontiguousarray(arr)
        assert arr.nbytes <= self.nbytes
        self.ctx.check(lib().mrt_cuda_copy_h2d(self.ctx.handle, C.c_void_p(self.ptr), ptr(arr), arr.nbytes,
                                               ptr(stream)), "copy_h2d")
        if stream is None:
            self.ctx.sync()

    def download(self, dtype, shape, stream=None) -> np.ndarray:
        out = np.empty(shape, dtype=dtype)
        assert out.nbytes <= self.nbytes
        self.ctx.check(lib().mrt_cuda_copy_d2h(self.ctx.handle, ptr(out), C.c_void_p(self.ptr), out.nbytes,
                                               ptr(stream)), "copy_d2h")
        self.ctx.sync(stream)
        return out

    def zero(self, stream=None):
        self.ctx.check(lib().mrt_cuda_memset(self.ctx.handle, C.c_void_p(self.ptr), 0, self.nbytes, ptr(stream)),
                       "memset")

    def free(self):
        if self.ptr and self.ctx.handle:
            lib().mrt_cuda_free(self.ctx.handle, C.c_void_p(self.ptr))
        self.ptr = 0

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
