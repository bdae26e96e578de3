"""Post-processing on device buffers: the joint bilateral filter
(Denoiser::bilateral, src/gfx/modules/denoiser.ixx), the tonemappers
(Tonemapper, src/gfx/modules/tonemapper.ixx) and temporal reprojection of
the accumulated colour with the g-buffer's motion vectors (new)."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

from ._lib import (BilateralParams as BilateralParams_C, CameraConsts, Context, DeviceBuffer,
                   ReprojectParams as ReprojectParams_C, TonemapParams as TonemapParams_C, lib, ptr)

TONEMAP_LINEAR, TONEMAP_REINHARD, TONEMAP_HABLE, TONEMAP_ACES, TONEMAP_UCHIMURA, TONEMAP_AMD = range(6)


@dataclass
class BilateralParams:
    """denoiser.ixx:20-31 (make_default: sigma 5, kSigma 2, threshold 0.12)."""
    sigma: float = 5.0
    kSigma: float = 2.0
    threshold: float = 0.12

    def c(self, near_plane: float, frame_counter: int, dither: bool = True) -> BilateralParams_C:
        p = BilateralParams_C()
        p.sigma, p.k_sigma, p.threshold = self.sigma, self.kSigma, self.threshold
        p.near_plane, p.frame_counter, p.dither = near_plane, frame_counter, int(dither)
        return p


class Denoiser:
    """The reference's plain denoiser: bilateral() over the path-traced
    colour, guided by the g-buffer's depth and normal."""

    def __init__(self, ctx: Context):
        self.ctx = ctx

    def bilateral(self, color: DeviceBuffer, gbuffer, camera, params: BilateralParams | None = None,
                  frame_counter: int = 0, out: DeviceBuffer | None = None, dither: bool = True,
                  stream=None) -> DeviceBuffer:
        params = params or BilateralParams()
        out = out or self.ctx.alloc(12 * gbuffer.width * gbuffer.height)
        p = params.c(camera.nearPlane, frame_counter, dither)
        self.ctx.check(lib().mrt_cuda_bilateral(self.ctx.handle, C.byref(gbuffer.c()), ptr(color), C.byref(p),
                                                ptr(out), ptr(stream)), "bilateral")
        return out


@dataclass
class UchimuraParams:
    """tonemapper.ixx:20-40."""
    maxBrightness: float = 1.0
    contrast: float = 1.0
    linearStart: float = 0.22
    linearLength: float = 0.4
    blackTightness: float = 1.33
    pedestal: float = 0.0

    def values(self):
        return [self.maxBrightness, self.contrast, self.linearStart, self.linearLength, self.blackTightness,
                self.pedestal]


@dataclass
class AMDParams:
    """tonemapper.ixx:42-57."""
    hdrMax: float = 16.0
    contrast: float = 2.0
    shoulder: float = 1.0
    midIn: float = 0.18
    midOut: float = 0.18

    def values(self):
        return [self.hdrMax, self.contrast, self.shoulder, self.midIn, self.midOut]


class Tonemapper:
    """Exposure, curve, sRGB encode, RGBA8 (one launch per image)."""

    def __init__(self, ctx: Context):
        self.ctx = ctx

    def _run(self, mode, color, width, height, exposure, out, stream, reinhard_max=8.0, uchimura=None, amd=None):
        p = TonemapParams_C()
        lib().mrt_tonemap_defaults(C.byref(p))
        p.mode, p.exposure, p.reinhard_max = mode, exposure, reinhard_max
        if uchimura is not None:
            for k, v in enumerate(uchimura.values()):
                p.uchimura[k] = v
        if amd is not None:
            for k, v in enumerate(amd.values()):
                p.amd[k] = v
        out = out or self.ctx.alloc(4 * width * height)
        self.ctx.check(lib().mrt_cuda_tonemap(self.ctx.handle, ptr(color), width, height, C.byref(p), ptr(out),
                                              ptr(stream)), "tonemap")
        return out

    def linear(self, color, width, height, exposure=1.0, out=None, stream=None):
        return self._run(TONEMAP_LINEAR, color, width, height, exposure, out, stream)

    def reinhard(self, color, width, height, exposure=1.0, hdrMax=8.0, out=None, stream=None):
        return self._run(TONEMAP_REINHARD, color, width, height, exposure, out, stream, reinhard_max=hdrMax)

    def hable(self, color, width, height, exposure=1.0, out=None, stream=None):
        return self._run(TONEMAP_HABLE, color, width, height, exposure, out, stream)

    def aces(self, color, width, height, exposure=1.0, out=None, stream=None):
        return self._run(TONEMAP_ACES, color, width, height, exposure, out, stream)

    def uchimura(self, color, width, height, exposure=1.0, params: UchimuraParams | None = None, out=None,
                 stream=None):
        return self._run(TONEMAP_UCHIMURA, color, width, height, exposure, out, stream,
                         uchimura=params or UchimuraParams())

    def amd(self, color, width, height, exposure=1.0, params: AMDParams | None = None, out=None, stream=None):
        return self._run(TONEMAP_AMD, color, width, height, exposure, out, stream, amd=params or AMDParams())


@dataclass
class ReprojectParams:
    max_history: float = 32.0
    normal_cos: float = 0.9
    depth_rel: float = 0.05

    def c(self) -> ReprojectParams_C:
        p = ReprojectParams_C()
        p.max_history, p.normal_cos, p.depth_rel = self.max_history, self.normal_cos, self.depth_rel
        return p


def reproject(ctx: Context, cur, prev, consts: CameraConsts, sample, hist, hist_len, out, out_len,
              params: ReprojectParams | None = None, stream=None):
    """Folds this frame's estimate `sample` into the reprojected history
    (mrt_cuda_reproject); `consts` are this frame's camera constants with
    prev_view = the previous frame's view."""
    p = (params or ReprojectParams()).c()
    ctx.check(lib().mrt_cuda_reproject(ctx.handle, C.byref(cur.c()), C.byref(prev.c()), C.byref(consts), ptr(sample),
                                       ptr(hist), ptr(hist_len), C.byref(p), ptr(out), ptr(out_len), ptr(stream)),
              "reproject")
