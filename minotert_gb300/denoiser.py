"""Learned CNN denoiser (mrt_cuda_denoiser_*): a 3-level U-Net trained on
pairs the path tracer renders itself; the plain accumulation stays the
fallback."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import Context, lib, ptr

# (ca, cb, cout, ups, relu, scale) per layer, as in csrc/cuda/denoise.cu
TOPOLOGY = [(16, 0, 32, 0, 1, 0), (32, 0, 32, 0, 1, 0), (32, 0, 64, 0, 1, 1), (64, 0, 64, 0, 1, 1),
            (64, 0, 128, 0, 1, 2), (128, 0, 128, 0, 1, 2), (128, 64, 64, 1, 1, 1), (64, 0, 64, 0, 1, 1),
            (64, 32, 32, 1, 1, 0), (32, 0, 32, 0, 1, 0), (32, 0, 16, 0, 0, 0)]


class Denoiser:
    def __init__(self, ctx: Context, seed: int = 1):
        self.ctx = ctx
        h = C.c_void_p()
        ctx.check(lib().mrt_cuda_denoiser_create(ctx.handle, seed, C.byref(h)), "denoiser_create")
        self._h = h
        nw, nb = C.c_size_t(), C.c_size_t()
        lib().mrt_cuda_denoiser_param_count(h, C.byref(nw), C.byref(nb))
        self.n_weights, self.n_biases = nw.value, nb.value

    @property
    def handle(self):
        return self._h

    def set_tcgen05(self, mode):
        """Forward convolutions: 2 (or True) persistent warp-specialised
        tcgen05 kernels (default), 1 tcgen05 with one CTA per tile, 0 (or
        False) mma.sync.  The training backward runs on the tensor cores in
        mode 2 and on FP32 CUDA-core kernels in modes 1 and 0."""
        mode = 2 if mode is True else int(mode)
        self.ctx.check(lib().mrt_cuda_denoiser_set_tcgen05(self._h, mode), "denoiser_set_tcgen05")

    def features(self, scene, gbuffer, d_color, diagonal: float, d_features, stream=None):
        self.ctx.check(lib().mrt_cuda_denoiser_features(self.ctx.handle, scene.handle, C.byref(gbuffer.c()),
                                                        ptr(d_color), float(diagonal), ptr(d_features),
                                                        ptr(stream)), "denoiser_features")

    def infer(self, d_features, batch, width, height, d_out, stream=None):
        self.ctx.check(lib().mrt_cuda_denoiser_infer(self.ctx.handle, self._h, ptr(d_features), batch, width, height,
                                                     ptr(d_out), ptr(stream)), "denoiser_infer")

    def train_step(self, d_features, d_targets, batch, width, height, lr=1e-3, update=True, want_loss=False,
                   stream=None):
        loss = C.c_float(0.0)
        self.ctx.check(lib().mrt_cuda_denoiser_train_step(self.ctx.handle, self._h, ptr(d_features), ptr(d_targets),
                                                          batch, width, height, float(lr), int(update),
                                                          C.byref(loss) if want_loss else None, ptr(stream)),
                       "denoiser_train_step")
        return loss.value if want_loss else None

    def params(self, which: int = 0) -> np.ndarray:
        n = self.n_weights + self.n_biases
        out = np.zeros(n, np.float32)
        self.ctx.check(lib().mrt_cuda_denoiser_params(self.ctx.handle, self._h, which, ptr(out), n, 0), "params")
        return out

    def set_params(self, values: np.ndarray):
        values = np.ascontiguousarray(values, np.float32)
        self.ctx.check(lib().mrt_cuda_denoiser_params(self.ctx.handle, self._h, 0, ptr(values), values.size, 1),
                       "params")

    def close(self):
        if self._h and self.ctx.handle:
            lib().mrt_cuda_denoiser_destroy(self.ctx.handle, self._h)
        self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def to_bf16_bits(x: np.ndarray) -> np.ndarray:
    """float32 -> bfloat16 bit patterns (round to nearest even)."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32)
    r = u + np.uint32(0x7FFF) + ((u >> 16) & np.uint32(1))
    return (r >> 16).astype(np.uint16)


def from_bf16_bits(b: np.ndarray) -> np.ndarray:
    return (b.astype(np.uint32) << 16).view(np.float32)
