"""Headless renderer (mrt_renderer_*): the reference's Renderer_impl::draw
(src/gfx/renderer.ixx:39-68) without a window -- sky, primary and secondary
rays, optional reprojected history, denoiser, tonemapper -- into RGBA8 on
the device, with PPM / PFM writers."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import (BilateralParams, Context, ReprojectParams, TonemapParams, TraceParams, lib, ptr)
from .pathtracer import Camera

ACCUM_NONE, ACCUM_REPROJECT = 0, 1
DENOISE_NONE, DENOISE_BILATERAL = 0, 1
SKY_CONSTANT, SKY_ATMOSPHERE = 0, 1


class RenderSettings(C.Structure):
    _fields_ = [("trace", TraceParams), ("sky_mode", C.c_uint32), ("accumulation", C.c_uint32),
                ("denoise", C.c_uint32), ("pad", C.c_uint32), ("atmosphere", C.c_float * 28),
                ("sun_dir", C.c_float * 3), ("sun_illuminance", C.c_float * 3), ("bilateral", BilateralParams),
                ("reproject", ReprojectParams), ("tonemap", TonemapParams)]

    @classmethod
    def defaults(cls) -> "RenderSettings":
        s = cls()
        lib().mrt_render_settings_defaults(C.byref(s))
        return s


assert C.sizeof(RenderSettings) == 328


def _bind():
    L = lib()
    if getattr(L, "_renderer_bound", False):
        return L
    vp, u32, i32 = C.c_void_p, C.c_uint32, C.c_int
    from ._lib import Camera_C
    for name, args, res in [
        ("mrt_render_settings_defaults", [C.POINTER(RenderSettings)], None),
        ("mrt_renderer_create", [vp, vp, u32, u32, C.POINTER(vp)], i32),
        ("mrt_renderer_destroy", [vp], i32),
        ("mrt_renderer_draw", [vp, C.POINTER(Camera_C), C.POINTER(RenderSettings), vp], i32),
        ("mrt_renderer_plane", [vp, i32], vp),
        ("mrt_renderer_read", [vp, vp, vp, vp], i32),
        ("mrt_write_ppm", [C.c_char_p, vp, u32, u32], i32),
        ("mrt_write_pfm", [C.c_char_p, vp, u32, u32], i32),
    ]:
        fn = getattr(L, name)
        fn.argtypes, fn.restype = args, res
    L._renderer_bound = True
    return L


class Renderer:
    """Renderer_impl (renderer.ixx:39-68) without window, ImGui or swapchain.
    blue_noise: an RGBA8 texture to sample instead of the generated 64 x 64
    tile -- the reference's constructor loads assets/blue_noise.png
    (renderer.ixx:101-110; scene.load_png decodes it the same way)."""

    def __init__(self, ctx: Context, scene, width: int, height: int, blue_noise: np.ndarray | None = None):
        L = _bind()
        self.ctx, self.scene, self.width, self.height = ctx, scene, int(width), int(height)
        h = C.c_void_p()
        ctx.check(L.mrt_renderer_create(ctx.handle, scene.handle, self.width, self.height, C.byref(h)),
                  "renderer_create")
        self._h = h
        if blue_noise is not None:
            ctx.blue_noise(blue_noise)

    def draw(self, camera: Camera, settings: RenderSettings | None = None, stream=None):
        s = settings or RenderSettings.defaults()
        self.ctx.check(_bind().mrt_renderer_draw(self._h, C.byref(camera._c()), C.byref(s), ptr(stream)),
                       "renderer_draw")

    def plane(self, which: int) -> int:
        return _bind().mrt_renderer_plane(self._h, which) or 0

    def read(self, stream=None):
        n = self.width * self.height
        rgba = np.zeros((self.height, self.width, 4), np.uint8)
        hdr = np.zeros((self.height, self.width, 3), np.float32)
        self.ctx.check(_bind().mrt_renderer_read(self._h, ptr(rgba), ptr(hdr), ptr(stream)), "renderer_read")
        return rgba, hdr

    def close(self):
        if self._h:
            _bind().mrt_renderer_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def write_ppm(path: str, rgba: np.ndarray):
    rgba = np.ascontiguousarray(rgba, np.uint8)
    h, w = rgba.shape[:2]
    if _bind().mrt_write_ppm(str(path).encode(), ptr(rgba), w, h) != 0:
        raise OSError(f"cannot write {path}")


def write_pfm(path: str, rgb: np.ndarray):
    rgb = np.ascontiguousarray(rgb, np.float32)
    h, w = rgb.shape[:2]
    if _bind().mrt_write_pfm(str(path).encode(), ptr(rgb), w, h) != 0:
        raise OSError(f"cannot write {path}")
