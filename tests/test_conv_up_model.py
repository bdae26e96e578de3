"""CPU model of the denoiser's phase-decomposed upsampling convolution
(k_conv_up and k_up_weights in minotert_gb300/csrc/cuda/conv_tc.cuh): the
3x3 convolution of [nearest-upsampled A ++ B] computed the kernel's way —
A's halo at its own resolution with 2x2 merged weights per output phase
(four A-variants (s, px), accumulator blocks [phase px][output row j], the
rows a halo row reaches stacked along N), B's halo as even / odd pixel
planes (q) with the tap rows stacked along N — must equal the direct
convolution, with every output of a tile written exactly once.  The index
arithmetic restates the kernel's (tiles of R low-resolution rows x 126
columns, 128 accumulator rows)."""
import numpy as np
import pytest

COLS, ENTRIES = 126, 128
S = {(0, 0): [0], (0, 1): [1, 2], (1, 0): [0, 1], (1, 1): [2]}  # (phase, shift) -> taps
VAR = [(0, 0), (1, 0), (1, 1), (2, 1)]                         # A-variants (s, px)
BLK = [(1, 1), (0, 1), (1, 0), (0, 0)]                         # (py, ry) for j = 2t-3 .. 2t
MEM = [(0, 0), (0, 1), (0, 2), (1, 0), (1, 1), (1, 2)]         # B-members (px, kx)


def _conv_up_model(A, B, W, R):
    hl, wl, ca = A.shape
    h, w, cb = B.shape
    cout = W.shape[0]
    nk, nka = (ca + cb) // 16, ca // 16

    def w_a(k, v):  # merged weights of variant v: 4 blocks x cout rows
        s, px = VAR[v]
        rx = s - px
        out = np.zeros((4 * cout, 16))
        for b, (py, ry) in enumerate(BLK):
            out[b * cout:(b + 1) * cout] = sum(W[:, ky * 3 + kx, 16 * k:16 * k + 16]
                                               for ky in S[(py, ry)] for kx in S[(px, rx)])
        return out

    def w_b(k, m):  # member m's weights: tap rows ky = 2, 1, 0 stacked
        px, kx = MEM[m]
        return np.concatenate([W[:, (2 - b) * 3 + kx, 16 * k:16 * k + 16] for b in range(3)])

    out = np.full((h, w, cout), np.nan)
    for Y0 in range(0, hl, R):
        for X0 in range(0, wl, COLS):
            D = np.zeros((4 * R, ENTRIES, cout))  # block px * 2R + j
            for k in range(nk):
                if k < nka:
                    halo = np.zeros((R + 2, ENTRIES + 4, 16))
                    for t in range(R + 2):
                        Y = Y0 - 1 + t
                        for e in range(ENTRIES + 2):
                            X = X0 - 1 + e
                            if 0 <= Y < hl and 0 <= X < wl:
                                halo[t, e] = A[Y, X, 16 * k:16 * k + 16]
                    for t in range(R + 2):
                        jlo, jhi = max(0, 2 * t - 3), min(2 * R - 1, 2 * t)
                        if jlo > jhi:
                            continue
                        for v, (s, px) in enumerate(VAR):
                            wv = w_a(k, v)[(jlo - (2 * t - 3)) * cout:(jhi - (2 * t - 3) + 1) * cout]
                            res = halo[t, s:s + ENTRIES] @ wv.T
                            for jj in range(jhi - jlo + 1):
                                D[px * 2 * R + jlo + jj] += res[:, jj * cout:(jj + 1) * cout]
                else:
                    c = 16 * k - ca
                    halo = np.zeros((2, 2 * R + 2, ENTRIES + 2, 16))  # [q][full-resolution row][entry]
                    for fr in range(2 * R + 2):
                        for q in range(2):
                            for e in range(ENTRIES):
                                y, x = 2 * Y0 - 1 + fr, 2 * (X0 - 1 + e) + q
                                if 0 <= y < h and 0 <= x < w:
                                    halo[q, fr, e] = B[y, x, c:c + 16]
                    for fr in range(2 * R + 2):
                        jlo, jhi = max(0, fr - 2), min(2 * R - 1, fr)
                        if jlo > jhi:
                            continue
                        for m, (px, kx) in enumerate(MEM):
                            q = (px + kx + 1) & 1
                            o = (px + kx - 1 - q) // 2 + 1
                            wm = w_b(k, m)[(jlo - (fr - 2)) * cout:(jhi - (fr - 2) + 1) * cout]
                            res = halo[q, fr, o:o + ENTRIES] @ wm.T
                            for jj in range(jhi - jlo + 1):
                                D[px * 2 * R + jlo + jj] += res[:, jj * cout:(jj + 1) * cout]
            for blk in range(4 * R):  # the epilogue: block (px, j) -> output (2 Y0 + j, 2 (X0 + i) + px)
                px, j = blk // (2 * R), blk % (2 * R)
                for i in range(COLS):
                    y, x = 2 * Y0 + j, 2 * (X0 + i) + px
                    if x < w and y < h:
                        assert np.isnan(out[y, x, 0]), "an output written twice"
                        out[y, x] = D[blk, i]
    return out


@pytest.mark.parametrize("ca,cb,cout,hl,wl,R", [(32, 16, 16, 5, 7, 2), (32, 16, 16, 4, 9, 1), (16, 32, 16, 3, 130, 2)])
def test_phase_decomposed_upsampling_equals_the_direct_convolution(ca, cb, cout, hl, wl, R):
    rng = np.random.default_rng(0)
    A = rng.standard_normal((hl, wl, ca))
    B = rng.standard_normal((2 * hl, 2 * wl, cb))
    W = rng.standard_normal((cout, 9, ca + cb))
    X = np.concatenate([A.repeat(2, 0).repeat(2, 1), B], -1)
    h, w = 2 * hl, 2 * wl
    Xp = np.pad(X, ((1, 1), (1, 1), (0, 0)))
    ref = np.zeros((h, w, cout))
    for t in range(9):
        ky, kx = t // 3, t % 3
        ref += Xp[ky:ky + h, kx:kx + w] @ W[:, t, :].T
    got = _conv_up_model(A, B, W, R)
    assert not np.isnan(got).any()
    assert np.max(np.abs(got - ref)) < 1e-9
