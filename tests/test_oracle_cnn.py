"""CPU check of the denoiser oracle's analytic backward against FP64
finite differences (the oracle then judges the CUDA kernels)."""
import numpy as np

from oracle import cnn


def test_cnn_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    n_params = sum(co * 9 * (ca + cb) + co for ca, cb, co, *_ in cnn.TOPOLOGY)
    params = rng.normal(scale=0.08, size=n_params)
    x = rng.uniform(0, 1, (1, 8, 8, 16))
    x[..., 10:] = 0.0
    t = rng.uniform(0, 2, (1, 8, 8, 3))
    loss, g, out = cnn.loss_and_grads(params, x, t, round_bf16=False)

    def f(p):
        return cnn.loss_and_grads(p, x, t, round_bf16=False)[0]

    eps = 1e-6
    idx = rng.choice(np.flatnonzero(np.abs(g) > 1e-6), 30, replace=False)
    for k in idx:
        pp, pm = params.copy(), params.copy()
        pp[k] += eps
        pm[k] -= eps
        fd = (f(pp) - f(pm)) / (2 * eps)
        assert abs(fd - g[k]) <= 1e-4 * max(1e-3, abs(fd)) + 1e-7, (k, fd, g[k])
