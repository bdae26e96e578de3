"""CPU ORACLE (test infrastructure only): FP64 restatement of the U-Net
denoiser -- 3x3 convolutions with bias and ReLU, 2x2 average pooling,
nearest 2x upsampling with skip concatenation, L1 loss in log(1 + x) --
with an analytic backward pass, for the checks of the CUDA kernels.
Layouts follow include/mrt_cuda.h (mrt_cuda_denoiser_params): layer l's
weights are [cout][3x3 tap][cin], then all biases.  Used only by tests/.
"""
from __future__ import annotations

import numpy as np

TOPOLOGY = [(16, 0, 32, 0, 1, 0), (32, 0, 32, 0, 1, 0), (32, 0, 64, 0, 1, 1), (64, 0, 64, 0, 1, 1),
            (64, 0, 128, 0, 1, 2), (128, 0, 128, 0, 1, 2), (128, 64, 64, 1, 1, 1), (64, 0, 64, 0, 1, 1),
            (64, 32, 32, 1, 1, 0), (32, 0, 32, 0, 1, 0), (32, 0, 16, 0, 0, 0)]


def bf16(x):
    u = np.ascontiguousarray(x, np.float32).view(np.uint32)
    r = (u + np.uint32(0x7FFF) + ((u >> 16) & np.uint32(1))) & np.uint32(0xFFFF0000)
    return r.view(np.float32).astype(np.float64)


def split(params):
    ws, bs, off = [], [], 0
    for ca, cb, co, *_ in TOPOLOGY:
        n = co * 9 * (ca + cb)
        ws.append(params[off:off + n].reshape(co, 9, ca + cb).astype(np.float64))
        off += n
    for ca, cb, co, *_ in TOPOLOGY:
        bs.append(params[off:off + co].astype(np.float64))
        off += co
    return ws, bs


def conv(x, w, b):
    """x (N,H,W,C) -> (N,H,W,cout), 3x3, zero padding."""
    n, h, wd, c = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    y = np.zeros((n, h, wd, w.shape[0])) + b
    for tap in range(9):
        dy, dx = tap // 3 - 1, tap % 3 - 1
        y += xp[:, 1 + dy:1 + dy + h, 1 + dx:1 + dx + wd, :] @ w[:, tap, :].T
    return y


def conv_bwd(x, w, dz):
    n, h, wd, c = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    gw = np.zeros_like(w)
    gxp = np.zeros_like(xp)
    for tap in range(9):
        dy, dx = tap // 3 - 1, tap % 3 - 1
        win = xp[:, 1 + dy:1 + dy + h, 1 + dx:1 + dx + wd, :]
        gw[:, tap, :] = np.einsum("nhwo,nhwi->oi", dz, win)
        gxp[:, 1 + dy:1 + dy + h, 1 + dx:1 + dx + wd, :] += dz @ w[:, tap, :]
    return gxp[:, 1:-1, 1:-1, :], gw, dz.sum(axis=(0, 1, 2))


def pool(x):
    return 0.25 * (x[:, 0::2, 0::2] + x[:, 1::2, 0::2] + x[:, 0::2, 1::2] + x[:, 1::2, 1::2])


def up(x):
    return x.repeat(2, axis=1).repeat(2, axis=2)


def forward(params, x, round_bf16=True):
    """Returns (activations list, inputs list per layer, output)."""
    ws, bs = split(params)
    if round_bf16:
        ws = [bf16(w) for w in ws]
    q = bf16 if round_bf16 else (lambda a: a)
    acts, ins = [], []

    def run(l, inp):
        ins.append(inp)
        z = conv(inp, ws[l], bs[l])
        y = np.maximum(z, 0.0) if TOPOLOGY[l][4] else z
        y = q(y)
        acts.append(y)
        return y

    a0 = run(0, x)
    s0 = run(1, a0)
    p0 = q(pool(s0))
    a2 = run(2, p0)
    s1 = run(3, a2)
    p1 = q(pool(s1))
    a4 = run(4, p1)
    a5 = run(5, a4)
    a6 = run(6, np.concatenate([up(a5), s1], axis=3))
    a7 = run(7, a6)
    a8 = run(8, np.concatenate([up(a7), s0], axis=3))
    a9 = run(9, a8)
    out = run(10, a9)
    return acts, ins, out


def loss_and_grads(params, x, target, round_bf16=True):
    ws, bs = split(params)
    wsq = [bf16(w) for w in ws] if round_bf16 else ws
    acts, ins, out = forward(params, x, round_bf16)
    n = out.shape[0] * out.shape[1] * out.shape[2] * 3
    # residual on demodulated radiance: the prediction is the input's
    # log(1 + radiance / albedo) plus the output (albedo 0 counts as 1)
    a = np.where(x[..., 3:6] > 0, x[..., 3:6], 1.0)
    d = out[..., :3] + x[..., :3] - np.log1p(np.maximum(target, 0.0) / a)
    loss = np.abs(d).sum() / n
    g = [None] * 11
    g[10] = np.zeros_like(out)
    g[10][..., :3] = np.sign(d) / n
    gws, gbs = [None] * 11, [None] * 11
    gins = [None] * 11

    def back(l):
        dz = g[l] * (acts[l] > 0) if TOPOLOGY[l][4] else g[l]
        gi, gws[l], gbs[l] = conv_bwd(ins[l], wsq[l], dz)
        gins[l] = gi

    def add(i, v):
        g[i] = v if g[i] is None else g[i] + v

    def unpool(gp):
        return 0.25 * up(gp)

    def down(gu):  # gradient through nearest upsampling: sum of the 2x2 children
        return gu[:, 0::2, 0::2] + gu[:, 1::2, 0::2] + gu[:, 0::2, 1::2] + gu[:, 1::2, 1::2]

    back(10); add(9, gins[10])
    back(9); add(8, gins[9])
    back(8); add(7, down(gins[8][..., :64])); add(1, gins[8][..., 64:])
    back(7); add(6, gins[7])
    back(6); add(5, down(gins[6][..., :128])); add(3, gins[6][..., 128:])
    back(5); add(4, gins[5])
    back(4); add(3, unpool(gins[4]))
    back(3); add(2, gins[3])
    back(2); add(1, unpool(gins[2]))
    back(1); add(0, gins[1])
    back(0)
    flat = np.concatenate([gw.reshape(-1) for gw in gws] + [gb for gb in gbs])
    return loss, flat, out
