"""Sky and atmosphere (mrt_cuda_sky_*): the host mirror of the reference's
Atmosphere and Sky modules (src/gfx/modules/sky.ixx).

    atmo = Atmosphere(ctx, Atmosphere.earth())   # transmittance + multi-scattering LUTs
    sky = Sky()
    view = sky.createView(atmo, camera.position)  # sky-view LUT at the camera
    ctx.set_sky(view)                             # escaping paths now see this sky
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import Context, lib, ptr

TRANSMITTANCE_SIZE = (256, 64)    # sky.ixx:24
MULTI_SCATTERING_SIZE = (32, 32)  # sky.ixx:27
VIEW_SIZE = (192, 108)            # sky.ixx:184


class Atmosphere:
    """Precomputed atmosphere: transmittance and multiple-scattering LUTs
    (Atmosphere ctor, sky.ixx:84-174).  `params` is a float32 array of the
    28 mrt_atmosphere_params values."""

    def __init__(self, ctx: Context, params: np.ndarray | None = None, stream=None):
        self.ctx = ctx
        self.params = np.ascontiguousarray(Atmosphere.earth() if params is None else params, np.float32)
        if self.params.size != 28:
            raise ValueError("atmosphere params: 28 floats expected")
        h = C.c_void_p()
        ctx.check(lib().mrt_cuda_sky_create(ctx.handle, C.byref(h)), "sky_create")
        self._h = h
        ctx.check(lib().mrt_cuda_sky_atmosphere(ctx.handle, h, ptr(self.params), ptr(stream)), "sky_atmosphere")

    @staticmethod
    def earth() -> np.ndarray:
        """Atmosphere::Params::earth() (sky.ixx:59-83)."""
        out = np.zeros(28, np.float32)
        lib().mrt_atmosphere_earth(ptr(out))
        return out

    @property
    def handle(self):
        return self._h

    def lut(self, which: int) -> np.ndarray:
        """0: transmittance (64, 256, 4); 1: multi-scattering (32, 32, 4);
        2: the last sky view (108, 192, 4)."""
        w, h = (TRANSMITTANCE_SIZE, MULTI_SCATTERING_SIZE, VIEW_SIZE)[which]
        out = np.zeros((h, w, 4), np.float32)
        self.ctx.check(lib().mrt_cuda_sky_lut(self.ctx.handle, self._h, which, ptr(out), out.size), "sky_lut")
        return out

    def close(self):
        if self._h:
            lib().mrt_cuda_sky_destroy(self.ctx.handle, self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Sky:
    """Sun parameters and sky views (Sky, sky.ixx:179-262).  A view is built
    into the atmosphere's LUT set; the returned object is the atmosphere
    itself, ready for Context.set_sky and eval()."""

    def __init__(self):
        self.sunDirection = np.array([-0.435286462, 0.818654716, 0.374606609], np.float32)  # sky.ixx:186
        self.sunIlluminance = np.array([8.0, 8.0, 8.0], np.float32)                           # sky.ixx:187

    def createView(self, atmo: Atmosphere, probePos, stream=None) -> "SkyView":
        pos = np.ascontiguousarray(probePos, np.float32)
        sun = np.ascontiguousarray(self.sunDirection, np.float32)
        e = np.ascontiguousarray(self.sunIlluminance, np.float32)
        atmo.ctx.check(lib().mrt_cuda_sky_view(atmo.ctx.handle, atmo.handle, ptr(pos), ptr(sun), ptr(e),
                                               ptr(stream)), "sky_view")
        return SkyView(atmo, pos, sun, e)


class SkyView:
    def __init__(self, atmo: Atmosphere, probe, sun, sun_e):
        self.atmo = atmo
        self.probe, self.sun, self.sun_e = probe.copy(), sun.copy(), sun_e.copy()

    @property
    def handle(self):
        return self.atmo.handle

    def eval(self, d_dirs, n: int, d_out, camera_pos=None, stream=None):
        """skyColor for n device directions (float3) into d_out (float3)."""
        cam = np.ascontiguousarray(self.probe if camera_pos is None else camera_pos, np.float32)
        self.atmo.ctx.check(lib().mrt_cuda_sky_eval(self.atmo.ctx.handle, self.atmo.handle, ptr(cam), ptr(d_dirs),
                                                    n, ptr(d_out), ptr(stream)), "sky_eval")
