"""CPU model of the denoiser's weight-gradient GEMM (k_conv_wgrad in
minotert_gb300/csrc/cuda/wgrad_tc.cuh): per channel chunk of NC inputs, the
im2col of 64-pixel row segments staged as blocks of 16 pixels x 8 channels
(block t * NC/8 + c8 for tap t, then a block of ones for the bias), the
dz operand as blocks of 16 pixels x 8 output channels, one M = 128 x K = 16
product per (16-pixel step, 128-row tile), and the epilogue mapping the
accumulator rows back to (tap, input channel) — against the direct sums
dW[co][tap][ci] = sum dz * x_shifted and db = sum dz.  Upsampled and
concatenated sources are resolved in the gather, as in the kernel."""
import numpy as np
import pytest

SEG = 64  # pixels of a row segment per stage


def _wgrad_model(X, dz, NC):
    n, h, w, cin = X.shape
    cout = dz.shape[-1]
    nc8, co8 = NC // 8, cout // 8
    groups = 9 * nc8 + 1
    tiles = (groups + 15) // 16
    ksteps = SEG // 16
    gw, gb = np.zeros((cout, 9, cin)), np.zeros(cout)
    segs_x = (w + SEG - 1) // SEG
    for chunk in range(cin // NC):
        c0 = chunk * NC
        D = np.zeros((tiles * 128, cout))
        for r in range(n * h * segs_x):
            xs, y, nn = r % segs_x, (r // segs_x) % h, r // (segs_x * h)
            x0 = xs * SEG
            a = np.full((ksteps, tiles * 16, 16, 8), np.nan)  # [k-step][block][pixel][channel]; unused blocks: garbage
            a[:, 9 * nc8] = 1.0                             # the bias block
            b = np.zeros((ksteps, co8, 16, 8))
            for i in range(9 * SEG * nc8):                  # the gather's element map
                c8, p, t = i % nc8, (i // nc8) % SEG, i // (nc8 * SEG)
                yy, xx, c = y + t // 3 - 1, x0 + p + t % 3 - 1, c0 + 8 * c8
                ok = 0 <= yy < h and 0 <= xx < w
                a[p >> 4, t * nc8 + c8, p & 15] = X[nn, yy, xx, c:c + 8] if ok else 0.0
            for i in range(SEG * co8):
                c8, p = i % co8, i // co8
                xx = x0 + p
                b[p >> 4, c8, p & 15] = dz[nn, y, xx, 8 * c8:8 * c8 + 8] if xx < w else 0.0
            for j in range(ksteps):
                bm = b[j].transpose(1, 0, 2).reshape(16, cout)          # K = 16 pixels x N = cout
                for m in range(tiles):
                    am = a[j, 16 * m:16 * m + 16].transpose(0, 2, 1).reshape(128, 16)  # M = block * 8 + channel
                    with np.errstate(invalid="ignore"):
                        D[m * 128:(m + 1) * 128] += am @ bm
        for m in range(tiles):  # the epilogue
            for lane in range(128):
                blk, cc = 16 * m + lane // 8, lane % 8
                if blk < 9 * nc8:
                    t, ci = blk // nc8, c0 + (blk % nc8) * 8 + cc
                    gw[:, t, ci] += D[m * 128 + lane]
                elif blk == 9 * nc8 and cc == 0 and chunk == 0:
                    gb += D[m * 128 + lane]
    return gw, gb


@pytest.mark.parametrize("n,h,w,ca,cb,cout,ups,NC", [(1, 4, 70, 32, 0, 32, 0, 32), (1, 4, 40, 16, 0, 32, 0, 16),
                                                     (1, 4, 20, 64, 32, 16, 1, 32)])
def test_im2col_weight_gradient_equals_the_direct_sums(n, h, w, ca, cb, cout, ups, NC):
    rng = np.random.default_rng(1)
    ha, wa = (h // 2, w // 2) if ups else (h, w)
    A = rng.standard_normal((n, ha, wa, ca))
    B = rng.standard_normal((n, h, w, cb)) if cb else None
    dz = rng.standard_normal((n, h, w, cout))
    U = A.repeat(2, 1).repeat(2, 2) if ups else A
    X = np.concatenate([U, B], -1) if cb else U
    Xp = np.pad(X, ((0, 0), (1, 1), (1, 1), (0, 0)))
    gw_ref = np.zeros((cout, 9, X.shape[-1]))
    for t in range(9):
        ky, kx = t // 3, t % 3
        gw_ref[:, t, :] = np.einsum("nhwo,nhwi->oi", dz, Xp[:, ky:ky + h, kx:kx + w])
    gw, gb = _wgrad_model(X, dz, NC)
    assert np.max(np.abs(gw - gw_ref)) < 1e-9
    assert np.max(np.abs(gb - dz.sum((0, 1, 2)))) < 1e-9
