"""CPU ORACLE (test infrastructure only): FP64 restatement of the learned
radiance cache -- hash-grid encoding, 64-wide ReLU MLP, relative L2 loss --
with an analytic backward pass, for the gradient checks of the CUDA
kernels.  Used only by tests/.

Layouts follow include/mrt_cuda.h (mrt_cuda_cache_params): MLP weights are
4 hidden layers of 64x64 [out][in] then 16 output rows of 64 (3 used);
grid features are 16 levels x 2^log2_t entries x 2.
"""
from __future__ import annotations

import numpy as np

LEVELS, WIDTH, HIDDEN, OUTROWS, ENC = 16, 64, 4, 16, 32
N_WEIGHTS = HIDDEN * WIDTH * WIDTH + OUTROWS * WIDTH


def level_scales(base_res: float, max_res: float):
    growth = np.float32(np.exp((np.log(np.float32(max_res)) - np.log(np.float32(base_res))) / np.float32(LEVELS - 1)))
    lg = np.log2(growth, dtype=np.float32)
    return [np.float32(base_res) * np.exp2(np.float32(l) * lg, dtype=np.float32) for l in range(LEVELS)]


def corners(q: np.ndarray, log2_t: int, base_res: float, max_res: float):
    """Corner table indices (global: level * T + local) and trilinear
    weights, shapes (n, 16, 8)."""
    T = 1 << log2_t
    p = np.clip(q[:, :3].astype(np.float32), 0.0, 1.0)
    n = len(q)
    idx = np.zeros((n, LEVELS, 8), np.int64)
    w = np.zeros((n, LEVELS, 8), np.float64)
    for l, s in enumerate(level_scales(base_res, max_res)):
        res = int(np.ceil(s)) + 2
        dense = res ** 3 <= T
        f = (p * s).astype(np.float32)
        i0 = np.floor(f)
        t = (f - i0).astype(np.float64)
        i0 = i0.astype(np.uint64)
        for c in range(8):
            cx, cy, cz = c & 1, (c >> 1) & 1, c >> 2
            x, y, z = i0[:, 0] + np.uint64(cx), i0[:, 1] + np.uint64(cy), i0[:, 2] + np.uint64(cz)
            if dense:
                li = x + np.uint64(res) * (y + np.uint64(res) * z)
            else:
                m = np.uint64(0xFFFFFFFF)
                li = ((x * np.uint64(1)) & m) ^ ((y * np.uint64(2654435761)) & m) ^ ((z * np.uint64(805459861)) & m)
                li = li & np.uint64(T - 1)
            idx[:, l, c] = np.int64(l * T) + li.astype(np.int64)
            w[:, l, c] = (t[:, 0] if cx else 1 - t[:, 0]) * (t[:, 1] if cy else 1 - t[:, 1]) * \
                         (t[:, 2] if cz else 1 - t[:, 2])
    return idx, w


def encode(grid: np.ndarray, q: np.ndarray, idx, w) -> np.ndarray:
    """(n, 64) input rows: 32 features, normal, direction, zeros."""
    g = grid.reshape(-1, 2).astype(np.float64)
    feats = np.einsum("nlc,nlcf->nlf", w, g[idx])  # (n, 16, 2)
    x = np.zeros((len(q), WIDTH))
    x[:, :ENC] = feats.reshape(len(q), ENC)
    x[:, ENC:ENC + 6] = q[:, 3:9]
    return x


def layers(W: np.ndarray):
    Wh = [W[l * 4096:(l + 1) * 4096].reshape(WIDTH, WIDTH).astype(np.float64) for l in range(HIDDEN)]
    Wo = W[HIDDEN * 4096:].reshape(OUTROWS, WIDTH)[:3].astype(np.float64)
    return Wh, Wo


def forward(W, x, fp16_acts: bool = False):
    Wh, Wo = layers(W)
    hs = [x]
    h = x
    for Wl in Wh:
        h = np.maximum(h @ Wl.T, 0.0)
        if fp16_acts:
            h = h.astype(np.float16).astype(np.float64)
        hs.append(h)
    return hs, h @ Wo.T


def loss_and_grads(grid, W, q, target, log2_t, base_res, max_res, fp16: bool = True):
    """Relative L2 loss mean_r sum_k (y - t)^2 / (sg(y)^2 + 0.01) and its
    gradients w.r.t. the MLP weights (flat, N_WEIGHTS) and the grid (flat)."""
    if fp16:  # what the kernels see: FP16 weights, grid and input rows
        W = W.astype(np.float16).astype(np.float64)
        grid = grid.astype(np.float16).astype(np.float64)
    idx, w = corners(q, log2_t, base_res, max_res)
    x = encode(grid, q, idx, w)
    if fp16:
        x = x.astype(np.float16).astype(np.float64)
    hs, y = forward(W, x, fp16_acts=fp16)
    n = len(q)
    den = y * y + 0.01
    loss = np.sum((y - target) ** 2 / den) / n
    d = 2.0 * (y - target) / den / n  # (n, 3)
    Wh, Wo = layers(W)
    gW = np.zeros(N_WEIGHTS)
    gWo = d.T @ hs[HIDDEN]  # (3, 64)
    gW[HIDDEN * 4096:HIDDEN * 4096 + 3 * WIDTH] = gWo.reshape(-1)
    dh = d @ Wo
    for l in range(HIDDEN - 1, -1, -1):
        dz = dh * (hs[l + 1] > 0)
        gW[l * 4096:(l + 1) * 4096] = (dz.T @ hs[l]).reshape(-1)
        dh = dz @ Wh[l]
    dx = dh[:, :ENC].reshape(n, LEVELS, 2)
    ggrid = np.zeros((grid.size // 2, 2))
    np.add.at(ggrid, idx.reshape(-1), (w[..., None] * dx[:, :, None, :]).reshape(-1, 2))
    return loss, gW, ggrid.reshape(-1), y


def predict(grid, W, q, log2_t, base_res, max_res):
    idx, w = corners(q, log2_t, base_res, max_res)
    x = encode(grid.astype(np.float16).astype(np.float64), q, idx, w).astype(np.float16).astype(np.float64)
    return forward(W.astype(np.float16).astype(np.float64), x, fp16_acts=True)[1]
