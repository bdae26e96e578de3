"""The CNN denoiser on the GPU: forward (BF16 tensor-core convolutions) and
gradients against the FP64 oracle (oracle/cnn.py, checked against finite
differences), training convergence, and features from a rendered frame."""
import numpy as np
import pytest

from oracle import cnn
from minotert_gb300.denoiser import Denoiser, from_bf16_bits, to_bf16_bits

pytestmark = pytest.mark.gpu


def _inputs(n, h, w, seed):
    rng = np.random.default_rng(seed)
    x = np.zeros((n, h, w, 16), np.float32)
    x[..., :10] = rng.uniform(0, 1, (n, h, w, 10))
    t = rng.uniform(0, 2, (n, h, w, 3)).astype(np.float32)
    return x, t


def test_denoiser_forward_matches_oracle(ctx):
    d = Denoiser(ctx, seed=2)
    x, _ = _inputs(2, 16, 24, 1)
    xb = to_bf16_bits(x)
    d_x = ctx.to_device(xb)
    d_o = ctx.alloc(2 * 16 * 24 * 3 * 4)
    d.infer(d_x, 2, 24, 16, d_o)
    y = d_o.download(np.float32, (2, 16, 24, 3))
    params = d.params(0).astype(np.float64)
    _, _, out = cnn.forward(params, from_bf16_bits(xb).astype(np.float64).reshape(2, 16, 24, 16))
    xin = from_bf16_bits(xb).astype(np.float64).reshape(2, 16, 24, 16)
    alb = np.where(xin[..., 3:6] > 0, xin[..., 3:6], 1.0)
    ref = np.expm1(np.maximum(out[..., :3] + xin[..., :3], 0.0)) * alb
    assert np.all(np.isfinite(y))
    err = np.abs(y - ref)
    assert np.max(err) < 3e-2 * max(1.0, np.abs(ref).max()), np.max(err)
    assert np.mean(err) < 3e-3 * max(1.0, np.abs(ref).mean())


def test_denoiser_gradients_match_oracle(ctx):
    d = Denoiser(ctx, seed=3)
    x, t = _inputs(2, 16, 16, 4)
    xb = to_bf16_bits(x)
    d_x, d_t = ctx.to_device(xb), ctx.to_device(t)
    loss = d.train_step(d_x, d_t, 2, 16, 16, update=False, want_loss=True)
    g = d.params(1).astype(np.float64)
    params = d.params(0).astype(np.float64)
    rloss, rg, _ = cnn.loss_and_grads(params, from_bf16_bits(xb).astype(np.float64).reshape(2, 16, 16, 16),
                                      t.astype(np.float64))
    assert abs(loss - rloss) < 2e-2 * rloss
    cos = g @ rg / (np.linalg.norm(g) * np.linalg.norm(rg))
    assert cos > 0.995, cos
    assert abs(np.linalg.norm(g) / np.linalg.norm(rg) - 1) < 0.05


def test_denoiser_training_reduces_loss(ctx):
    # learn to remove additive noise from a smooth colour field guided by
    # clean albedo features
    rng = np.random.default_rng(5)
    n, h, w = 4, 32, 32
    yy, xx = np.mgrid[0:h, 0:w] / 32.0
    clean = np.stack([0.5 + 0.3 * np.sin(4 * xx), 0.4 + 0.3 * yy, 0.3 + 0.2 * np.cos(3 * yy)], -1)
    t = np.repeat(clean[None], n, 0).astype(np.float32)
    x = np.zeros((n, h, w, 16), np.float32)
    noisy = np.clip(t * rng.gamma(2.0, 0.5, t.shape), 0, None)
    x[..., :3] = np.log1p(noisy)
    x[..., 3:6] = clean
    d = Denoiser(ctx, seed=6)
    d_x, d_t = ctx.to_device(to_bf16_bits(x)), ctx.to_device(t)
    first = d.train_step(d_x, d_t, n, w, h, lr=2e-3, want_loss=True)
    for _ in range(300):
        d.train_step(d_x, d_t, n, w, h, lr=2e-3)
    last = d.train_step(d_x, d_t, n, w, h, lr=2e-3, want_loss=True)
    assert last < first / 4, (first, last)


def test_denoiser_features_from_a_frame(ctx, hf_workload, blue_noise):
    from minotert_gb300.pathtracer import Pathtracer, TraceSettings
    from minotert_gb300.scene import DeviceScene
    wl, mesh, bvh = hf_workload
    ds = DeviceScene.triangles(ctx, mesh, bvh)
    pt = Pathtracer(ctx, ds, full_gbuffer=False)
    gb = pt.primaryRays((wl.width, wl.height), wl.camera, wl.camera)
    col = pt.secondaryRays(gb, wl.camera, wl.sky, blue_noise, wl.settings)
    d = Denoiser(ctx)
    feats = ctx.alloc(wl.width * wl.height * 16 * 2)
    d.features(ds, gb, col, float(np.linalg.norm(mesh.hi - mesh.lo)), feats)
    f = from_bf16_bits(feats.download(np.uint16, (wl.height, wl.width, 16)))
    img = col.download(np.float32, (wl.height, wl.width, 3))
    g = gb.download()
    hit = g["visibility"] != 0xFFFFFFFF
    alb = mesh.albedo()[g["visibility"][hit]]
    assert np.allclose(f[hit][:, 3:6], alb, atol=1e-2)
    a = np.ones_like(img)
    a[hit] = f[hit][:, 3:6]
    ir = np.log1p(img / a)
    assert np.allclose(f[..., :3], ir, atol=2e-2 * ir.max())
    assert np.all(f[..., 10:] == 0)
    out = ctx.alloc(wl.width * wl.height * 12)
    d.infer(feats, 1, wl.width, wl.height, out)
    assert np.isfinite(out.download(np.float32, (wl.height, wl.width, 3))).all()


def test_denoiser_inference_is_size_and_batch_consistent(ctx):
    # a pixel's output depends only on the inputs within the network's
    # receptive field (about 20 pixels), so the interior of a 128x128 crop
    # taken at an offset that is a multiple of 4 (the pooling alignment) must
    # equal the same pixels of the full 1920x1080 image, and an image must
    # give the same output alone and inside a batch
    d = Denoiser(ctx, seed=5)
    rng = np.random.default_rng(12)
    W, H = 1920, 1080
    x = np.zeros((H, W, 16), np.float32)
    x[..., :10] = rng.uniform(0, 1, (H, W, 10))
    xb = to_bf16_bits(x)
    d_x = ctx.to_device(xb)
    d_o = ctx.alloc(W * H * 12)
    d.infer(d_x, 1, W, H, d_o)
    full = d_o.download(np.float32, (H, W, 3))
    for (y0, x0) in [(0, 0), (476, 900), (952, 1792)]:
        crop = np.ascontiguousarray(xb[y0:y0 + 128, x0:x0 + 128])
        c_x, c_o = ctx.to_device(crop), ctx.alloc(128 * 128 * 12)
        d.infer(c_x, 1, 128, 128, c_o)
        part = c_o.download(np.float32, (128, 128, 3))
        inner = (slice(32, 96), slice(32, 96))
        assert np.array_equal(part[inner], full[y0 + 32:y0 + 96, x0 + 32:x0 + 96]), (y0, x0)
    two = np.ascontiguousarray(np.stack([xb[:128, :128], xb[128:256, :128]]))
    t_x, t_o = ctx.to_device(two), ctx.alloc(2 * 128 * 128 * 12)
    d.infer(t_x, 2, 128, 128, t_o)
    pair = t_o.download(np.float32, (2, 128, 128, 3))
    one_x, one_o = ctx.to_device(np.ascontiguousarray(xb[128:256, :128])), ctx.alloc(128 * 128 * 12)
    d.infer(one_x, 1, 128, 128, one_o)
    assert np.array_equal(pair[1], one_o.download(np.float32, (128, 128, 3)))


@pytest.mark.parametrize("shape", [(2, 16, 24), (1, 64, 200), (1, 540, 960), (1, 1080, 1920)])
def test_denoiser_tcgen05_matches_mma_sync(ctx, shape):
    # the same network on the three forward paths: persistent warp-
    # specialised tcgen05 kernels (mode 2, default), tcgen05 with one CTA
    # per tile (mode 1) and mma.sync (mode 0).  The layers without
    # upsampling issue the same MMAs in the same order in modes 2 and 1; the
    # two upsampling layers of mode 2 are phase-decomposed (2 x 2 merged
    # weights, rounded to BF16), so mode 2 agrees with the others to BF16
    # rounding, like mma.sync, whose FP32 summation order differs: layer
    # outputs to BF16 rounding, the decoded radiance to ~1 %.  The shapes
    # cover partial and multiple 126-column tiles of the phase-decomposed
    # layers and the persistent CTAs' loops over many tiles
    n, h, w = shape
    d = Denoiser(ctx, seed=7)
    rng = np.random.default_rng(3)
    x = np.zeros((n, h, w, 16), np.float32)
    x[..., :10] = rng.uniform(0, 1, (n, h, w, 10))
    xb = to_bf16_bits(x)
    d_x = ctx.to_device(xb)
    outs = []
    for mode in (2, 1, 0):
        d.set_tcgen05(mode)
        d_o = ctx.alloc(n * h * w * 12)
        d.infer(d_x, n, w, h, d_o)
        outs.append(d_o.download(np.float32, (n, h, w, 3)))
    d.set_tcgen05(2)
    assert ctx.status() == 0
    ws, tile, b = outs
    assert np.isfinite(ws).all()
    for other in (tile, b):
        err = np.abs(ws - other)
        assert err.max() < 3e-2 * max(1.0, np.abs(other).max()), err.max()
        assert err.mean() < 2e-3 * max(1.0, np.abs(other).mean())


@pytest.mark.parametrize("shape", [(2, 16, 16), (1, 36, 200), (8, 128, 128)])
def test_denoiser_tensor_core_backward_matches_fp32(ctx, shape):
    # one training step's gradients from the tcgen05 backward (mode 2: BF16
    # pre-activation gradients, data gradients as mirrored convolutions,
    # weight and bias gradients as GEMMs over the pixels) against the FP32
    # CUDA-core backward (mode 1, whose forward differs from mode 2's only in
    # the upsampling layers' BF16 rounding of merged weights); per layer,
    # weights and biases separately, so a broken tap, channel chunk or bias
    # column shows by name.  Shapes: the gradient test's tiny
    # images, a width of two 128-pixel segments with a ragged end, and the
    # training batch (8 crops of 128 x 128)
    n, h, w = shape
    x, t = _inputs(n, h, w, 7)
    d_x, d_t = ctx.to_device(to_bf16_bits(x)), ctx.to_device(t)
    res = {}
    for mode in (2, 1):
        d = Denoiser(ctx, seed=9)
        d.set_tcgen05(mode)
        loss = d.train_step(d_x, d_t, n, w, h, update=False, want_loss=True)
        res[mode] = (loss, d.params(1).astype(np.float64))
        d.close()
    assert ctx.status() == 0
    (l_tc, g_tc), (l_fp, g_fp) = res[2], res[1]
    assert abs(l_tc - l_fp) <= 1e-3 * abs(l_fp), (l_tc, l_fp)
    assert np.isfinite(g_tc).all()
    ws_tc, bs_tc = cnn.split(g_tc)
    ws_fp, bs_fp = cnn.split(g_fp)
    # the two forwards differ by the upsampling layers' merged-weight
    # rounding, which the 512 pixels of the smallest case average least
    tol = 6e-2 if n * h * w < 4096 else 3e-2
    for l, (a, b) in enumerate(zip(ws_tc + bs_tc, ws_fp + bs_fp)):
        name = f"{'w' if l < len(ws_tc) else 'b'}{l % len(ws_tc)}"
        a, b = a.ravel(), b.ravel()
        nb = np.linalg.norm(b)
        if nb == 0:
            assert np.linalg.norm(a) == 0, name
            continue
        rel = np.linalg.norm(a - b) / nb
        assert rel < tol, (name, rel)
    cos = g_tc @ g_fp / (np.linalg.norm(g_tc) * np.linalg.norm(g_fp))
    assert cos > 0.999, cos
