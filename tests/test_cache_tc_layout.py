"""CPU model of the radiance cache's tcgen05 backward (k_cache_bwd_tc in
minotert_gb300/csrc/cuda/nrc.cu): its shared-memory map, the shared-memory
matrix descriptors of its MMAs (no swizzle; K-major and MN-major reads) and
the tensor-memory columns they accumulate into, checked against a plain
backward of the same 4 x 64 + 16 MLP.  Every operand element is read at the
address the descriptor arithmetic gives, inside the CTA's allocation; two
layers share tensor-memory columns by lanes through zero-padded A rows.
The constants restate the kernel's."""
import numpy as np

ROWS, WIDTH, OUT_ROWS, HIDDEN = 128, 64, 16, 4
PLANE = ROWS * 16                      # one 8-element K plane of a 128-row tile
IMG, DY_IMG = ROWS * WIDTH * 2, ROWS * OUT_ROWS * 2
LAYER_B = WIDTH * 16 * (WIDTH // 8)    # one hidden layer's weights
W_BYTES = HIDDEN * LAYER_B + OUT_ROWS * 16 * (WIDTH // 8)
DY, W = 0, DY_IMG                      # shared-memory map of k_cache_bwd_tc
D1 = W + W_BYTES
Z = D1 + IMG
D2 = Z + IMG
H = D2 + IMG                           # image i = input of layer i
SMEM = H + (HIDDEN + 1) * IMG + 64


def _kmajor(mem, start, lbo, sbo, m, k):
    """Element (m, k) of a K-major no-swizzle operand: core matrices of 8 rows
    x 16 bytes, SBO between 8-row groups, LBO between 8-element K groups."""
    mm, kk = np.meshgrid(np.arange(m), np.arange(k), indexing="ij")
    off = start + (mm // 8) * sbo + (kk // 8) * lbo + (mm % 8) * 16 + (kk % 8) * 2
    assert off.min() >= 0 and off.max() + 2 <= SMEM
    return mem[off // 2]


def _mnmajor(mem, start, lbo, sbo, mn, k):
    """Element (mn, k) of an MN-major no-swizzle operand: core matrices of 8
    K rows x 16 bytes of 8 MN elements, LBO between K groups, SBO between MN
    groups."""
    mm, kk = np.meshgrid(np.arange(mn), np.arange(k), indexing="ij")
    off = start + (mm // 8) * sbo + (kk // 8) * lbo + (kk % 8) * 16 + (mm % 8) * 2
    assert off.min() >= 0 and off.max() + 2 <= SMEM
    return mem[off // 2]


def _put_image(mem, base, x):
    r, c = np.meshgrid(np.arange(x.shape[0]), np.arange(x.shape[1]), indexing="ij")
    mem[(base + (c // 8) * PLANE + r * 16 + (c % 8) * 2) // 2] = x


def _h16(x):
    return np.asarray(x, np.float16).astype(np.float64)


def test_backward_descriptors_and_tensor_memory_match_a_plain_backward():
    rng = np.random.default_rng(0)
    w = [_h16(rng.normal(size=(WIDTH, WIDTH)) * 0.2) for _ in range(HIDDEN)]
    w.append(_h16(rng.normal(size=(OUT_ROWS, WIDTH)) * 0.2))
    w[HIDDEN][3:] = 0.0
    mem = np.zeros(SMEM // 2)
    for l in range(HIDDEN + 1):  # the forward's K-plane weight layout
        rows = WIDTH if l < HIDDEN else OUT_ROWS
        o, i = np.meshgrid(np.arange(rows), np.arange(WIDTH), indexing="ij")
        off = W + l * LAYER_B + (i // 8) * (rows * 16) + o * 16 + (i % 8) * 2
        mem[off // 2] = w[l]
    hs = [_h16(rng.normal(size=(ROWS, WIDTH)))]
    for l in range(HIDDEN):
        hs.append(_h16(np.maximum(hs[-1] @ w[l].T, 0.0)))
    dy = np.zeros((ROWS, OUT_ROWS))
    dy[:, :3] = _h16(rng.normal(size=(ROWS, 3)))
    # plain backward (FP16 operands, as the kernel's)
    ref_dw = [None] * (HIDDEN + 1)
    dz = dy
    ref_dw[HIDDEN] = dz.T @ hs[HIDDEN]
    dh = dz @ w[HIDDEN]
    for l in range(HIDDEN - 1, -1, -1):
        dz = _h16(np.where(hs[l + 1] > 0, dh, 0.0))
        ref_dw[l] = dz.T @ hs[l]
        dh = dz @ w[l]
    # the kernel: five phases, tensor memory 128 lanes x 256 columns
    tmem = np.zeros((128, 256))
    _put_image(mem, DY, dy)
    for i in range(HIDDEN + 1):
        _put_image(mem, H + i * IMG, hs[i])
    for p in range(HIDDEN + 1):
        h = H + (HIDDEN - p) * IMG
        upper = p in (2, 4)
        dzb = DY if p == 0 else (D1 if p & 1 else D2)
        a_dw = Z if upper else dzb
        col = 192 if p == 0 else (64 if p <= 2 else 128)
        clears = not upper
        for k in range(ROWS // 16):  # dW += dZ^T H, both MN-major
            a = _mnmajor(mem, a_dw + 256 * k, 128, PLANE, 128, 16)
            b = _mnmajor(mem, h + 256 * k, 128, PLANE, WIDTH, 16).T
            prod = a @ b
            if k == 0 and clears:
                tmem[:, col:col + WIDTH] = prod
            else:
                tmem[:, col:col + WIDTH] += prod
        if p == 0:  # dH = dZ W, W read MN-major
            a = _kmajor(mem, dzb, PLANE, 128, 128, 16)
            b = _mnmajor(mem, W + HIDDEN * LAYER_B, 128, OUT_ROWS * 16, WIDTH, 16).T
            tmem[:, :WIDTH] = a @ b
        else:
            wl = W + (HIDDEN - p) * LAYER_B
            for k in range(WIDTH // 16):
                a = _kmajor(mem, dzb + 2 * k * PLANE, PLANE, 128, 128, 16)
                b = _mnmajor(mem, wl + 256 * k, 128, WIDTH * 16, WIDTH, 16).T
                tmem[:, :WIDTH] = a @ b if k == 0 else tmem[:, :WIDTH] + a @ b
        if p < HIDDEN:  # the next dZ, masked by ReLU'(layer input), as FP16
            _put_image(mem, D2 if p & 1 else D1, _h16(np.where(hs[HIDDEN - p] > 0, tmem[:, :WIDTH], 0.0)))
        else:
            d_in = tmem[:, :WIDTH].copy()
    got = {3: tmem[0:64, 64:128], 2: tmem[64:128, 64:128], 1: tmem[0:64, 128:192], 0: tmem[64:128, 128:192],
           HIDDEN: tmem[0:16, 192:256]}
    for l in range(HIDDEN + 1):
        assert np.allclose(got[l], ref_dw[l], rtol=1e-12, atol=1e-12), l
    assert np.allclose(d_in, dh, rtol=1e-12, atol=1e-12)


def test_shared_memory_map_fits_and_padding_rows_stay_inside():
    # the output layer's dW product reads 128 A rows, 16 real: its 16 row
    # groups of 2 KB from dL/dy onwards end inside the weights
    assert DY + 16 * PLANE <= D1
    assert SMEM <= 227 * 1024
    # every bulk copy and descriptor start is 16-byte aligned
    for off in (DY, W, D1, Z, D2, H, H + IMG):
        assert off % 16 == 0
