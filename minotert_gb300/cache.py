"""Learned radiance cache (mrt_cuda_cache_*): hash-grid encoding + 64-wide
MLP trained online, queried at the first diffuse bounce."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import CacheConfig, Context, lib, ptr

N_WEIGHTS = 4 * 64 * 64 + 16 * 64


def default_config(**kw) -> CacheConfig:
    c = CacheConfig()
    c.log2_table, c.base_res, c.max_res = 19, 16.0, 2048.0
    c.lr_grid, c.lr_mlp = 1e-2, 1e-3
    c.seed, c.train_paths, c.train_steps, c.train_bounces = 1, 65536, 4, 8
    c.query_vertex = 1
    for k, v in kw.items():
        setattr(c, k, v)
    return c


class RadianceCache:
    def __init__(self, ctx: Context, cfg: CacheConfig | None = None, bounds=None):
        self.ctx = ctx
        self.cfg = cfg or default_config()
        h = C.c_void_p()
        ctx.check(lib().mrt_cuda_cache_create(ctx.handle, C.byref(self.cfg), C.byref(h)), "cache_create")
        self._h = h
        if bounds is not None:
            self.set_bounds(*bounds)

    @property
    def handle(self):
        return self._h

    @property
    def grid_floats(self) -> int:
        return 16 * (1 << self.cfg.log2_table) * 2

    def set_bounds(self, lo, hi):
        lo = (C.c_float * 3)(*map(float, lo))
        hi = (C.c_float * 3)(*map(float, hi))
        self.ctx.check(lib().mrt_cuda_cache_set_bounds(self.ctx.handle, self._h, lo, hi), "cache_set_bounds")

    def set_tcgen05(self, enable: bool):
        """Inference and training on tcgen05 (default) or on the mma.sync kernels."""
        self.ctx.check(lib().mrt_cuda_cache_set_tcgen05(self._h, int(enable)), "cache_set_tcgen05")

    def set_overlap(self, enable: bool):
        """frame(): train on the context's second stream while the frame's rays
        are traced (default), or first, on the caller's stream."""
        self.ctx.check(lib().mrt_cuda_cache_set_overlap(self._h, int(enable)), "cache_set_overlap")

    def infer(self, d_queries, n: int, d_out, stream=None):
        self.ctx.check(lib().mrt_cuda_cache_infer(self.ctx.handle, self._h, ptr(d_queries), n, ptr(d_out),
                                                  ptr(stream)), "cache_infer")

    def train_step(self, d_queries, d_targets, n: int, update: bool = True, want_loss: bool = False, stream=None):
        loss = C.c_float(0.0)
        self.ctx.check(lib().mrt_cuda_cache_train_step(self.ctx.handle, self._h, ptr(d_queries), ptr(d_targets), n,
                                                       int(update), C.byref(loss) if want_loss else None,
                                                       ptr(stream)), "cache_train_step")
        return loss.value if want_loss else None

    def params(self, which: int) -> np.ndarray:
        n = N_WEIGHTS if which < 2 else self.grid_floats
        out = np.zeros(n, np.float32)
        self.ctx.check(lib().mrt_cuda_cache_params(self.ctx.handle, self._h, which, ptr(out), n, 0), "cache_params")
        return out

    def set_params(self, which: int, values: np.ndarray):
        values = np.ascontiguousarray(values, np.float32)
        self.ctx.check(lib().mrt_cuda_cache_params(self.ctx.handle, self._h, which, ptr(values), values.size, 1),
                       "cache_params")

    def frame(self, scene, gbuffer, consts, params, color, train: bool = True, stream=None):
        self.ctx.check(lib().mrt_cuda_cache_frame(self.ctx.handle, self._h, scene.handle, C.byref(gbuffer.c()),
                                                  C.byref(consts), C.byref(params), ptr(color), int(train),
                                                  ptr(stream)), "cache_frame")

    def close(self):
        if self._h and self.ctx.handle:
            lib().mrt_cuda_cache_destroy(self.ctx.handle, self._h)
        self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
