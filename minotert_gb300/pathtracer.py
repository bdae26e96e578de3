"""Host mirror of MinoteRT's path-tracer module over the mrt_cuda C ABI.

Keeps the reference's interface (src/gfx/modules/pathtracer.ixx:18-200,
src/gfx/camera.ixx:10-44) so a renderer written against it switches over
by changing the device layer only:

    Camera(viewport, verticalFov, nearPlane, position, yaw, pitch)
        .view(), .projection(), .direction()
    Pathtracer.primaryRays(size, camera, prevCamera) -> GBuffer
    Pathtracer.secondaryRays(gbuffer, camera, sky, blueNoise) -> color

Differences, by design: the scene is a Pathtracer member (the reference
compiles its 5 spheres into the shaders, scene.glsl:4-11); `sky` is a Sky
(constant radiance + optional directional light) in place of the
atmosphere LUTs; errors raise MrtError (the reference throws
runtime_error_fmt, src/stx/except.ixx:12-20); g-buffer images are device
buffers owned by the returned GBuffer instead of vuk futures.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from ._lib import (MRT_EST_ESCAPE, MRT_EST_NEE, MRT_RNG_REFERENCE, Camera_C, CameraConsts, Context, DeviceBuffer,
                   GBuffer as GBuffer_C, TraceParams, lib, ptr)
from .scene import DeviceScene


@dataclass
class Camera:
    """src/gfx/camera.ixx:10-26 (movement speeds omitted)."""
    viewport: tuple
    verticalFov: float
    nearPlane: float
    position: tuple
    yaw: float
    pitch: float
    # (x0, y0, width, height): render only this pixel window of the
    # viewport's frustum (an off-centre projection: pixel (x, y) of the
    # window sees what pixel (x0 + x, y0 + y) of the full viewport sees).
    # New; the reference always renders the whole viewport.
    window: tuple | None = None

    def direction(self) -> np.ndarray:
        cp, sp = math.cos(self.pitch), math.sin(self.pitch)
        return np.array([cp * math.cos(self.yaw), cp * math.sin(self.yaw), sp], np.float32)

    def _c(self) -> Camera_C:
        c = Camera_C()
        c.viewport[0], c.viewport[1] = int(self.viewport[0]), int(self.viewport[1])
        c.vertical_fov, c.near_plane = float(self.verticalFov), float(self.nearPlane)
        for k in range(3):
            c.position[k] = float(self.position[k])
        c.yaw, c.pitch = float(self.yaw), float(self.pitch)
        return c

    def view(self) -> np.ndarray:
        """4x4 column-major (m[col*4+row]) look(position, direction, +Z)."""
        out = (C.c_float * 16)()
        lib().mrt_camera_view(C.byref(self._c()), out)
        return np.array(out[:], np.float32)

    def projection(self) -> np.ndarray:
        out = (C.c_float * 16)()
        lib().mrt_camera_projection(C.byref(self._c()), out)
        return np.array(out[:], np.float32)

    @classmethod
    def reference(cls, width: int, height: int) -> "Camera":
        """The reference's start-up camera (src/app.ixx:20-32)."""
        return cls((width, height), math.radians(60.0), 0.001, (0.0, -0.001, 0.1), math.radians(90.0), 0.0)


def camera_consts(camera: Camera, prev: Camera | None = None, frame_counter: int = 0) -> CameraConsts:
    """The per-dispatch constants of pathtracer.ixx:86-105 / 171-184; with a
    camera window, the projection narrowed to that window."""
    out = CameraConsts()
    pc = (prev or camera)._c()
    lib().mrt_camera_consts_make(C.byref(camera._c()), C.byref(pc), frame_counter, C.byref(out))
    if camera.window is not None:
        window_projection(out, camera.viewport, camera.window)
    return out


def window_projection(consts: CameraConsts, viewport, window) -> None:
    """Narrow the projection of `consts` (made for the full `viewport`) to
    the pixel window (x0, y0, w, h), in place.  The kernels map pixel (x, y)
    of a w x h image to NDC (2 (x + 0.5) / w - 1, 1 - 2 (y + 0.5) / h); the
    full viewport's NDC of pixel (x0 + x, y0 + y) is the affine map
    ndc_full = a * ndc_window + b per axis with a = (w / W, h / H),
    b = ((w + 2 x0) / W - 1, 1 - (2 y0 + h) / H).  So the window's inverse
    projection is inv_projection * T (T: that map on x and y, identity on z
    and w) and its projection T^-1 * projection (depth is unchanged)."""
    W, H = float(viewport[0]), float(viewport[1])
    x0, y0, w, h = (float(v) for v in window)
    ax, ay = w / W, h / H
    bx, by = (w + 2.0 * x0) / W - 1.0, 1.0 - (2.0 * y0 + h) / H
    # column-major 4x4 (m[col * 4 + row])
    P = np.array(consts.projection[:], np.float64).reshape(4, 4).T
    Pi = np.array(consts.inv_projection[:], np.float64).reshape(4, 4).T
    T = np.array([[ax, 0, 0, bx], [0, ay, 0, by], [0, 0, 1, 0], [0, 0, 0, 1]], np.float64)
    Pw = np.linalg.inv(T) @ P
    Piw = Pi @ T
    consts.projection[:] = [float(v) for v in Pw.T.reshape(-1).astype(np.float32)]
    consts.inv_projection[:] = [float(v) for v in Piw.T.reshape(-1).astype(np.float32)]


def primary_rays_host(camera: Camera, width: int, height: int) -> np.ndarray:
    """The pinhole rays primaryRays traces (primaryRay.comp:46-51), for a
    width x height image of `camera` (or of its window), computed on the host
    in FP64 and stored as RAY_DTYPE (tmin 0, tmax inf): the primary rays of
    a batched path trace that is to see what primaryRays sees."""
    from ._lib import RAY_DTYPE
    c = camera_consts(camera)
    iv = np.array(c.inv_view[:], np.float64).reshape(4, 4).T
    ip = np.array(c.inv_projection[:], np.float64).reshape(4, 4).T
    xs = (np.arange(width, dtype=np.float64) + 0.5) / width * 2.0 - 1.0
    ys = (1.0 - (np.arange(height, dtype=np.float64) + 0.5) / height) * 2.0 - 1.0
    ndc = np.stack(np.broadcast_arrays(xs[None, :], ys[:, None], 1.0, 1.0), -1).reshape(-1, 4)
    vd = ndc @ ip.T
    vd[:, 3] = 0.0
    wd = (vd @ iv.T)[:, :3]
    wd /= np.linalg.norm(wd, axis=1, keepdims=True)
    rays = np.zeros(width * height, RAY_DTYPE)
    rays["org"] = (iv @ np.array([0.0, 0.0, 0.0, 1.0]))[:3].astype(np.float32)
    rays["dir"] = wd.astype(np.float32)
    rays["tmin"] = 0.0
    rays["tmax"] = np.inf
    return rays


@dataclass
class Sky:
    """Light for the secondary pass: constant sky radiance on escape and an
    optional directional light sampled with shadow rays."""
    radiance: tuple = (0.25, 0.32, 0.45)
    sun_dir: tuple | None = None
    sun_irradiance: tuple = (2.5, 2.5, 2.5)


@dataclass
class TraceSettings:
    samples: int = 8          # secondaryRays.comp:128
    bounces: int = 8          # secondaryRays.comp:129
    rr_start: int = 0
    rng_mode: int = MRT_RNG_REFERENCE
    accumulate: bool = False
    frame_index: int = 0
    sort_rays: bool = False
    exact_trig: bool = False  # sphere-point sin/cos in binary64 (the oracle's), see mrt_trace_params

    def params(self, sky: Sky) -> TraceParams:
        p = TraceParams()
        p.samples, p.max_bounces, p.rr_start = self.samples, self.bounces, self.rr_start
        p.rng_mode = self.rng_mode
        p.estimator = MRT_EST_NEE if sky.sun_dir is not None else MRT_EST_ESCAPE
        p.accumulate, p.frame_index, p.sort_rays = int(self.accumulate), self.frame_index, int(self.sort_rays)
        p.exact_trig = int(self.exact_trig)
        sd = np.asarray(sky.sun_dir if sky.sun_dir is not None else (0.0, 0.0, 1.0), np.float64)
        sd = (sd / np.linalg.norm(sd)).astype(np.float32)
        for k in range(3):
            p.sun_dir[k] = float(sd[k])
            p.sun_irradiance[k] = float(sky.sun_irradiance[k])
            p.sky_radiance[k] = float(sky.radiance[k])
        return p


@dataclass
class GBuffer:
    """pathtracer.ixx:22-27: visibility R32_UINT, depth R16F, normal RGBA16F,
    motion RG16F, plus the FP32 hit distance of the triangle path."""
    width: int
    height: int
    visibility: DeviceBuffer
    hit_t: DeviceBuffer
    depth: DeviceBuffer
    normal: DeviceBuffer
    motion: DeviceBuffer
    _c: GBuffer_C = field(default=None, repr=False)

    def c(self) -> GBuffer_C:
        if self._c is None:
            g = GBuffer_C()
            g.visibility, g.hit_t = self.visibility.ptr, self.hit_t.ptr
            g.depth = self.depth.ptr if self.depth is not None else None
            g.normal = self.normal.ptr if self.normal is not None else None
            g.motion = self.motion.ptr if self.motion is not None else None
            g.width, g.height = self.width, self.height
            self._c = g
        return self._c

    def download(self) -> dict:
        n = self.width * self.height
        out = {"visibility": self.visibility.download(np.uint32, (self.height, self.width)),
               "hit_t": self.hit_t.download(np.float32, (self.height, self.width))}
        if self.depth is not None:
            out["depth"] = self.depth.download(np.uint16, (self.height, self.width))
        if self.normal is not None:
            out["normal"] = self.normal.download(np.uint16, (self.height, self.width, 4))
        if self.motion is not None:
            out["motion"] = self.motion.download(np.uint16, (self.height, self.width, 2))
        return out


class Pathtracer:
    """Pathtracer (pathtracer.ixx:18-200) over one scene on one context."""

    def __init__(self, ctx: Context, scene: DeviceScene, full_gbuffer: bool = True):
        self.ctx, self.scene = ctx, scene
        self.full_gbuffer = full_gbuffer
        self._gb = None
        self._bn_id = None
        self.frame_counter = 0

    def _gbuffer(self, w: int, h: int) -> GBuffer:
        if self._gb is None or (self._gb.width, self._gb.height) != (w, h):
            n = w * h
            full = self.full_gbuffer or self.scene.kind == "spheres"
            a = self.ctx.alloc
            self._gb = GBuffer(w, h, a(4 * n), a(4 * n), a(2 * n) if full else None, a(8 * n) if full else None,
                               a(4 * n) if full else None)
        return self._gb

    def primaryRays(self, size, camera: Camera, prevCamera: Camera, stream=None) -> GBuffer:
        w, h = int(size[0]), int(size[1])
        g = self._gbuffer(w, h)
        consts = camera_consts(camera, prevCamera, self.frame_counter)
        self.ctx.check(lib().mrt_cuda_primary_rays(self.ctx.handle, self.scene.handle, C.byref(consts),
                                                   C.byref(g.c()), ptr(stream)), "primaryRays")
        return g

    def secondaryRays(self, gbuffer: GBuffer, camera: Camera, sky: Sky, blueNoise: np.ndarray,
                      settings: TraceSettings | None = None, color: DeviceBuffer | None = None,
                      stream=None, skyView=None) -> DeviceBuffer:
        """secondaryRays (pathtracer.ixx:118-195).  `sky` holds the constant
        sky radiance and the NEE light; `skyView` (a sky.SkyView, as
        secondaryRays' atmo + skyView arguments) makes escaping paths see
        the atmosphere instead of the constant radiance."""
        settings = settings or TraceSettings()
        if self._bn_id is not id(blueNoise):
            self.ctx.blue_noise(blueNoise)
            self._bn_id = id(blueNoise)
        color = color or self.ctx.alloc(12 * gbuffer.width * gbuffer.height)
        consts = camera_consts(camera, camera, self.frame_counter)
        params = settings.params(sky)
        if skyView is not None:
            self.ctx.set_sky(skyView)
        try:
            self.ctx.check(lib().mrt_cuda_secondary_rays(self.ctx.handle, self.scene.handle, C.byref(gbuffer.c()),
                                                         C.byref(consts), C.byref(params), C.c_void_p(color.ptr),
                                                         ptr(stream)), "secondaryRays")
        finally:
            if skyView is not None:
                self.ctx.set_sky(None)
        return color

    # snake_case aliases
    primary_rays = primaryRays
    secondary_rays = secondaryRays

    def next_frame(self):
        self.frame_counter += 1
