"""CPU checks of the radiance-cache oracle: its analytic backward against
FP64 finite differences (the oracle then judges the CUDA gradients)."""
import numpy as np

from oracle import nrc


def _setup(seed=0, n=24, log2_t=10):
    rng = np.random.default_rng(seed)
    q = np.zeros((n, 9))
    q[:, :3] = rng.uniform(0.05, 0.95, (n, 3))
    nn = rng.normal(size=(n, 3))
    q[:, 3:6] = nn / np.linalg.norm(nn, axis=1, keepdims=True)
    dd = rng.normal(size=(n, 3))
    q[:, 6:9] = dd / np.linalg.norm(dd, axis=1, keepdims=True)
    W = np.zeros(nrc.N_WEIGHTS)
    for l in range(nrc.HIDDEN):
        W[l * 4096:(l + 1) * 4096] = rng.uniform(-0.3, 0.3, 4096)
    W[nrc.HIDDEN * 4096:nrc.HIDDEN * 4096 + 3 * 64] = rng.uniform(-0.3, 0.3, 192)
    grid = rng.uniform(-0.5, 0.5, 16 * (1 << log2_t) * 2)
    t = rng.uniform(0.1, 1.0, (n, 3))
    return q, W, grid, t, log2_t


def test_oracle_gradients_match_finite_differences():
    q, W, grid, t, log2_t = _setup()
    args = (q, t, log2_t, 16.0, 512.0)
    loss, gW, gG, _ = nrc.loss_and_grads(grid, W, *args, fp16=False)
    # the relative L2 loss treats its denominator as a constant: use a
    # target-independent check by freezing it at the current prediction
    rng = np.random.default_rng(1)
    def f(Wv, Gv):
        idx, w = nrc.corners(q, log2_t, 16.0, 512.0)
        x = nrc.encode(Gv, q, idx, w)
        hs, y = nrc.forward(Wv, x)
        _, _, _, y0 = nrc.loss_and_grads(grid, W, *args, fp16=False)
        return np.sum((y - t) ** 2 / (y0 * y0 + 0.01)) / len(q)
    eps = 1e-6
    for k in rng.choice(np.flatnonzero(gW), 25, replace=False):
        Wp, Wm = W.copy(), W.copy()
        Wp[k] += eps
        Wm[k] -= eps
        fd = (f(Wp, grid) - f(Wm, grid)) / (2 * eps)
        assert abs(fd - gW[k]) <= 1e-5 * max(1.0, abs(fd)), (k, fd, gW[k])
    for k in rng.choice(np.flatnonzero(gG), 25, replace=False):
        Gp, Gm = grid.copy(), grid.copy()
        Gp[k] += eps
        Gm[k] -= eps
        fd = (f(W, Gp) - f(W, Gm)) / (2 * eps)
        assert abs(fd - gG[k]) <= 1e-5 * max(1.0, abs(fd)), (k, fd, gG[k])


def test_hash_levels_dense_then_hashed():
    T = 1 << 19
    s = nrc.level_scales(16.0, 2048.0)
    dense = [(int(np.ceil(x)) + 2) ** 3 <= T for x in s]
    assert dense[0] and not dense[-1]
    assert abs(float(s[-1]) - 2048.0) < 1.0
