"""Learned radiance cache on the GPU: forward and gradients of the CUDA
kernels against the FP64 oracle (oracle/nrc.py, itself checked against
finite differences), training convergence, and what the trained cache gains
over the plain path tracer at equal frame count."""
import numpy as np
import pytest

from oracle import nrc
from minotert_gb300.cache import RadianceCache, default_config

pytestmark = pytest.mark.gpu

LOG2_T = 14


def _queries(n, seed):
    rng = np.random.default_rng(seed)
    q = np.zeros((n, 9), np.float32)
    q[:, :3] = rng.uniform(0.02, 0.98, (n, 3))
    nn = rng.normal(size=(n, 3))
    q[:, 3:6] = nn / np.linalg.norm(nn, axis=1, keepdims=True)
    dd = rng.normal(size=(n, 3))
    q[:, 6:9] = dd / np.linalg.norm(dd, axis=1, keepdims=True)
    return q


def _cache(ctx, seed=1):
    c = RadianceCache(ctx, default_config(log2_table=LOG2_T, base_res=16.0, max_res=512.0, seed=seed))
    rng = np.random.default_rng(seed)
    W = c.params(0)
    W[nrc.HIDDEN * 4096:nrc.HIDDEN * 4096 + 3 * 64] = rng.uniform(-0.3, 0.3, 192)  # non-trivial outputs
    c.set_params(0, W)
    G = rng.uniform(-0.5, 0.5, c.grid_floats).astype(np.float32)
    c.set_params(2, G)
    return c, W, G


def test_cache_forward_matches_oracle(ctx):
    c, W, G = _cache(ctx)
    q = _queries(1000, 2)
    d_q, d_o = ctx.to_device(q), ctx.alloc(12 * len(q))
    c.infer(d_q, len(q), d_o)
    y = d_o.download(np.float32, (len(q), 3))
    ref = nrc.predict(G.astype(np.float64), W.astype(np.float64), q.astype(np.float64), LOG2_T, 16.0, 512.0)
    assert np.all(np.isfinite(y))
    err = np.abs(y - ref)
    assert np.max(err) < 2e-2 * max(1.0, np.max(np.abs(ref)))
    assert np.mean(err) < 2e-3 * max(1.0, np.mean(np.abs(ref)))


@pytest.mark.parametrize("n", [1, 127, 1000, 200001])
def test_cache_inference_tcgen05_matches_mma_sync_and_oracle(ctx, n):
    # the tcgen05 kernel (128-query tiles, accumulators in tensor memory) and
    # the mma.sync kernel on the same weights: both FP16 operands with FP32
    # accumulation, so they differ only where an FP32 sum rounds to another
    # FP16 activation.  Ragged sizes cover partial tiles; 200,001 queries
    # (1,563 tiles) take the persistent CTAs (4 per SM) round the tile loop
    c, W, G = _cache(ctx, seed=9)
    q = _queries(n, 10)
    d_q, d_tc, d_mma = ctx.to_device(q), ctx.alloc(12 * n), ctx.alloc(12 * n)
    c.infer(d_q, n, d_tc)
    c.set_tcgen05(False)
    c.infer(d_q, n, d_mma)
    c.set_tcgen05(True)
    assert ctx.status() == 0
    y_tc, y_mma = d_tc.download(np.float32, (n, 3)), d_mma.download(np.float32, (n, 3))
    assert np.all(np.isfinite(y_tc))
    scale = max(1.0, float(np.max(np.abs(y_mma))))
    assert np.max(np.abs(y_tc - y_mma)) < 1e-2 * scale
    assert np.mean(np.abs(y_tc - y_mma)) < 1e-3 * scale
    sub = slice(0, min(n, 1000))
    ref = nrc.predict(G.astype(np.float64), W.astype(np.float64), q[sub].astype(np.float64), LOG2_T, 16.0, 512.0)
    err = np.abs(y_tc[sub] - ref)
    assert np.max(err) < 2e-2 * max(1.0, np.max(np.abs(ref)))
    assert np.mean(err) < 2e-3 * max(1.0, np.mean(np.abs(ref)))


@pytest.mark.parametrize("tcgen05,n", [(True, 512), (True, 1008), (True, 16), (False, 512)])
def test_cache_gradients_match_oracle(ctx, tcgen05, n):
    # tcgen05 training (128-row tiles; 1008 rows = 7 full tiles + 112, 16
    # rows = one ragged tile) and the mma.sync kernels against the FP64
    # oracle's loss and gradients (FP16 operands as in the kernels)
    c, W, G = _cache(ctx, seed=3)
    c.set_tcgen05(tcgen05)
    q = _queries(n, 4)
    t = np.random.default_rng(5).uniform(0.1, 1.0, (len(q), 3)).astype(np.float32)
    d_q, d_t = ctx.to_device(q), ctx.to_device(t)
    loss = c.train_step(d_q, d_t, len(q), update=False, want_loss=True)
    assert ctx.status() == 0
    gW, gG = c.params(1).astype(np.float64), c.params(3).astype(np.float64)
    rloss, rgW, rgG, _ = nrc.loss_and_grads(G.astype(np.float64), W.astype(np.float64), q.astype(np.float64),
                                            t.astype(np.float64), LOG2_T, 16.0, 512.0, fp16=True)
    assert abs(loss - rloss) < 2e-2 * rloss
    for a, b in ((gW, rgW), (gG, rgG)):
        cos = a @ b / (np.linalg.norm(a) * np.linalg.norm(b))
        assert cos > 0.999, cos
        assert abs(np.linalg.norm(a) / np.linalg.norm(b) - 1.0) < 0.03


@pytest.mark.parametrize("tcgen05", [True, False])
def test_grid_adam_updates_only_touched_entries(ctx, tcgen05):
    # The grid's Adam is lazy per entry: the scatter flags the entries it
    # adds a gradient to, and the step updates those (and clears their
    # gradients) while every other entry keeps its features bit for bit.
    c, W, G = _cache(ctx, seed=17)
    c.set_tcgen05(tcgen05)
    q = _queries(300, 18)
    t = np.random.default_rng(19).uniform(0.1, 1.0, (len(q), 3)).astype(np.float32)
    d_q, d_t = ctx.to_device(q), ctx.to_device(t)
    g0 = c.params(2)
    c.train_step(d_q, d_t, len(q), update=False)
    grad = c.params(3).reshape(-1, 2)
    touched = np.any(grad != 0.0, axis=1)
    assert 0 < touched.sum() < len(touched) // 4
    c.train_step(d_q, d_t, len(q), update=True)
    assert ctx.status() == 0
    g1 = c.params(2).reshape(-1, 2)
    g0 = g0.reshape(-1, 2)
    assert np.array_equal(g1[~touched], g0[~touched])
    moved = np.any(g1[touched] != g0[touched], axis=1)
    assert moved.mean() > 0.99
    assert not np.any(c.params(3))
    # the first Adam step (b1 0.9, b2 0.99, bias-corrected, eps 1e-10): the
    # corrected moments are G and G^2, so a feature moves by lr * G / (|G| +
    # eps) = lr * sign(G); G is the two passes' sum, with grad's sign
    lr = default_config().lr_grid
    big = np.abs(grad) > 1e-6
    expect = g0 - lr * np.sign(grad)
    assert big.sum() > 100
    assert np.max(np.abs(g1[big] - expect[big])) < 1e-6


def test_cache_training_tcgen05_matches_mma_sync(ctx):
    # 200,000 rows: 1,563 tiles, so each backward CTA (two per SM) sums the
    # weight gradients of several tiles in tensor memory before adding them
    # to the FP32 array once.  Same samples, same weights: the two paths
    # differ only in FP32 summation order and where an FP32 sum rounds to
    # another FP16 operand.
    n = 200000
    q = _queries(n, 11)
    t = np.random.default_rng(12).uniform(0.1, 1.0, (n, 3)).astype(np.float32)
    d_q, d_t = ctx.to_device(q), ctx.to_device(t)
    out = {}
    for tc in (True, False):
        c, W, G = _cache(ctx, seed=13)
        c.set_tcgen05(tc)
        loss = c.train_step(d_q, d_t, n, update=False, want_loss=True)
        out[tc] = (loss, c.params(1).astype(np.float64), c.params(3).astype(np.float64))
        c.close()
    assert ctx.status() == 0
    assert abs(out[True][0] - out[False][0]) < 1e-3 * out[False][0]
    for k in (1, 2):
        a, b = out[True][k], out[False][k]
        assert np.all(np.isfinite(a))
        cos = a @ b / (np.linalg.norm(a) * np.linalg.norm(b))
        assert cos > 0.9999, (k, cos)
        assert abs(np.linalg.norm(a) / np.linalg.norm(b) - 1.0) < 0.01


def test_cache_learns_a_smooth_function(ctx):
    c = RadianceCache(ctx, default_config(log2_table=16, seed=7, lr_grid=1e-2, lr_mlp=1e-3))
    q = _queries(8192, 8)
    p = q[:, :3]
    t = np.stack([0.5 + 0.4 * np.sin(6 * p[:, 0]) * np.cos(4 * p[:, 1]), 0.3 + 0.2 * p[:, 2],
                  0.2 + 0.5 * p[:, 0] * p[:, 1]], axis=1).astype(np.float32)
    d_q, d_t = ctx.to_device(q), ctx.to_device(t)
    first = c.train_step(d_q, d_t, len(q), want_loss=True)
    for _ in range(300):
        c.train_step(d_q, d_t, len(q))
    last = c.train_step(d_q, d_t, len(q), want_loss=True)
    assert last < first / 20, (first, last)
    d_o = ctx.alloc(12 * len(q))
    c.infer(d_q, len(q), d_o)
    y = d_o.download(np.float32, (len(q), 3))
    assert np.sqrt(np.mean((y - t) ** 2)) < 0.05


def _rmse(a, b):
    return float(np.sqrt(np.mean((a - b) ** 2)))


def test_cache_experiment_reference_converges_to_fp64(ctx, blue_noise):
    # The radiance-cache experiment's reference (bench.py --workload
    # radiance_cache): 4096 plain frames of the heightfield scene at
    # 1920x1080 (8 bounces, roulette after 2) against the FP64 oracle's
    # 4096 samples per pixel on a 16 x 32 crop: both are Monte Carlo
    # estimates of the same pixels, so they agree to within their noise
    from minotert_gb300 import scene, workloads
    from minotert_gb300.pathtracer import Camera, Pathtracer, TraceSettings
    base = workloads.heightfield_boxes_256()
    W, H = 1920, 1080
    c0 = base.camera
    cam = Camera((W, H), c0.verticalFov, c0.nearPlane, c0.position, c0.yaw, c0.pitch)
    mesh = base.mesh()
    bvh = scene.build_bvh8(mesh)
    ds = scene.DeviceScene.triangles(ctx, mesh, bvh)
    ctx.blue_noise(blue_noise)
    pt = Pathtracer(ctx, ds, full_gbuffer=False)
    stream = ctx.stream()
    sky = base.sky
    col = ctx.alloc(12 * W * H)
    for f in range(4096):
        pt.frame_counter = (1 << 20) + f
        gb = pt.primaryRays((W, H), cam, cam, stream)
        pt.secondaryRays(gb, cam, sky, blue_noise, TraceSettings(1, 8, 2, 1, True, f), color=col, stream=stream)
    ref = col.download(np.float32, (H, W, 3), stream)
    assert ctx.status() == 0
    import oracle as orc
    y0, y1, x0, x1 = 600, 616, 900, 932
    consts = orc.camera_consts(cam.position, cam.yaw, cam.pitch, cam.verticalFov, cam.nearPlane, W, H)
    p = orc.primary(consts, W, H, bvh.nodes, bvh.tris, mesh.mats, y0=y0, y1=y1)
    sd = np.asarray(sky.sun_dir, np.float64)
    sd = (sd / np.linalg.norm(sd)).astype(np.float32)
    prm = orc.params_array(4096, 8, 2, 1, 1, sun=sd, sun_e=sky.sun_irradiance, sky=sky.radiance)
    crop64, _, _ = orc.pathtrace(bvh.nodes, bvh.tris, mesh.mats, consts, W, H, p["visibility"], p["hit_t"],
                                 blue_noise, prm, precision=64, y0=y0, y1=y1)
    a, b = ref[y0:y1, x0:x1], crop64[y0:y1, x0:x1]
    rel = float(np.sqrt(np.mean((a - b) ** 2)) / max(float(b.mean()), 1e-9))
    print(f"reference crop vs FP64: relative RMSE {rel:.4f}")
    assert rel < 0.01


def test_cache_frame_training_overlapped_with_tracing(ctx, hf_workload, blue_noise):
    # The same cache frames with the training on the context's second stream
    # (overlapped with the frame's ray tracing, joined before the cache is
    # queried) and first on the caller's stream: the same computations in
    # the same order, so the images agree up to the training's FP32 atomic
    # summation order.
    from minotert_gb300.pathtracer import Pathtracer, TraceSettings, camera_consts
    from minotert_gb300.scene import DeviceScene
    wl, mesh, bvh = hf_workload
    ds = DeviceScene.triangles(ctx, mesh, bvh)
    pt = Pathtracer(ctx, ds, full_gbuffer=False)
    ctx.blue_noise(blue_noise)
    W, H = wl.width, wl.height
    stream = ctx.stream()
    imgs = {}
    for overlap in (True, False):
        cache = RadianceCache(ctx, default_config(train_paths=16384, train_steps=4, query_vertex=1, seed=21),
                              bounds=(mesh.lo, mesh.hi))
        cache.set_overlap(overlap)
        col = ctx.alloc(12 * W * H)
        for f in range(6):
            pt.frame_counter = f
            gb = pt.primaryRays((W, H), wl.camera, wl.camera, stream)
            params = TraceSettings(1, 1, 2, 1, True, f).params(wl.sky)
            cache.frame(ds, gb, camera_consts(wl.camera, wl.camera, f), params, col, train=True, stream=stream)
        ctx.sync(stream)
        imgs[overlap] = col.download(np.float32, (H, W, 3))
        cache.close()
    assert ctx.status() == 0
    a, b = imgs[True], imgs[False]
    assert np.isfinite(a).all()
    assert _rmse(a, b) < 2e-3 * max(1e-3, float(np.mean(np.abs(b)))) + 1e-4, _rmse(a, b)


@pytest.mark.parametrize("query_vertex", [1, 0])
def test_trained_cache_beats_plain_path_tracing_at_equal_frames(ctx, hf_workload, blue_noise, query_vertex):
    # 128x128 heightfield scene; reference: plain path tracer, 1024 frames of
    # 1 spp.  After 48 training frames, 8 frames of cache-terminated paths
    # must be closer to the reference than 8 frames of the plain tracer.
    from minotert_gb300 import workloads
    from minotert_gb300.pathtracer import Pathtracer, TraceSettings, camera_consts
    from minotert_gb300.scene import DeviceScene
    wl = workloads.heightfield_boxes_256(size=128)
    mesh = hf_workload[1]
    ds = DeviceScene.triangles(ctx, mesh, hf_workload[2])
    pt = Pathtracer(ctx, ds, full_gbuffer=False)
    W, H = wl.width, wl.height
    ctx.blue_noise(blue_noise)
    plain_settings = TraceSettings(samples=1, bounces=6, rr_start=2, rng_mode=1)

    def accumulate(frames, fn, start=0):
        col = ctx.alloc(12 * W * H)
        for f in range(frames):
            pt.frame_counter = start + f
            gb = pt.primaryRays((W, H), wl.camera, wl.camera)
            fn(gb, col, f)
        return col.download(np.float32, (H, W, 3))

    def plain(gb, col, f):
        s = TraceSettings(1, 6, 2, 1, True, f)
        pt.secondaryRays(gb, wl.camera, wl.sky, blue_noise, s, color=col)

    ref = accumulate(1024, plain, start=10000)
    plain8 = accumulate(8, plain, start=0)
    cache = RadianceCache(ctx, default_config(train_paths=16384, train_steps=4, train_bounces=6,
                                              query_vertex=query_vertex),
                          bounds=(mesh.lo, mesh.hi))

    def learned(train):
        def fn(gb, col, f):
            consts = camera_consts(wl.camera, wl.camera, pt.frame_counter)
            params = TraceSettings(1, 1, 2, 1, True, f).params(wl.sky)
            cache.frame(ds, gb, consts, params, col, train=train)
        return fn

    accumulate(48, learned(True), start=20000)  # online training
    learned8 = accumulate(8, learned(True), start=0)
    assert ctx.status() == 0
    r_plain, r_learned = _rmse(plain8, ref), _rmse(learned8, ref)
    print(f"RMSE after 8 frames: plain {r_plain:.4f}, learned (query vertex {query_vertex}) {r_learned:.4f}")
    assert np.isfinite(learned8).all()
    assert r_learned < r_plain


def test_cache_against_plain_path_tracing_at_equal_gpu_time(ctx, hf_workload, blue_noise):
    # 480x270 view of the heightfield scene; reference: plain path tracer
    # (8 bounces, roulette after 2), 1024 frames.  The learned path (paths end
    # at the first bounce's hit, online training every frame, from an
    # untrained cache) and the plain path each get the same GPU time, the
    # learned path's 24 frames timed with CUDA events, training included.
    # The cache lowers each frame's variance but costs more per frame than
    # the bounces it replaces, so in this scene it does not beat the plain
    # tracer at equal time (the bench's radiance_cache workload gives the
    # bounds).  The test checks that it stays within 2x of the plain
    # tracer's RMSE at equal time and reports the ratio.
    from minotert_gb300.pathtracer import Camera, Pathtracer, TraceSettings, camera_consts
    from minotert_gb300.scene import DeviceScene
    wl, mesh, bvh = hf_workload
    W, H = 480, 270
    c = wl.camera
    cam = Camera((W, H), c.verticalFov, c.nearPlane, c.position, c.yaw, c.pitch)
    ds = DeviceScene.triangles(ctx, mesh, bvh)
    pt = Pathtracer(ctx, ds, full_gbuffer=False)
    ctx.blue_noise(blue_noise)
    stream = ctx.stream()

    def accumulate(frames, fn, start):
        col = ctx.alloc(12 * W * H)
        a, b = ctx.event(), ctx.event()
        ctx.record(a, stream)
        for f in range(frames):
            pt.frame_counter = start + f
            gb = pt.primaryRays((W, H), cam, cam, stream)
            fn(gb, col, f)
        ctx.record(b, stream)
        ctx.sync(stream)
        return col.download(np.float32, (H, W, 3)), ctx.elapsed_ms(a, b)

    def plain(gb, col, f):
        pt.secondaryRays(gb, cam, wl.sky, blue_noise, TraceSettings(1, 8, 2, 1, True, f), color=col, stream=stream)

    ref, _ = accumulate(1024, plain, start=10000)
    accumulate(4, plain, start=500)  # kernels loaded before anything is timed
    cache = RadianceCache(ctx, default_config(query_vertex=1), bounds=(mesh.lo, mesh.hi))

    def learned(gb, col, f):
        params = TraceSettings(1, 1, 2, 1, True, f).params(wl.sky)
        cache.frame(ds, gb, camera_consts(cam, cam, pt.frame_counter), params, col, train=True, stream=stream)

    warm = RadianceCache(ctx, default_config(query_vertex=1), bounds=(mesh.lo, mesh.hi))
    col = ctx.alloc(12 * W * H)
    gb = pt.primaryRays((W, H), cam, cam, stream)
    warm.frame(ds, gb, camera_consts(cam, cam, 0), TraceSettings(1, 1, 2, 1, True, 0).params(wl.sky), col,
               train=True, stream=stream)
    ctx.sync(stream)
    warm.close()
    img_l, ms_l = accumulate(24, learned, start=0)
    # plain frames in the same GPU time (per-frame time from 16 timed frames)
    _, ms16 = accumulate(16, plain, start=2000)
    n_plain = max(1, int(ms_l / (ms16 / 16)))
    img_p, ms_p = accumulate(n_plain, plain, start=0)
    cache.close()
    assert ctx.status() == 0
    assert np.isfinite(img_l).all()
    r_l, r_p = _rmse(img_l, ref), _rmse(img_p, ref)
    print(f"equal GPU time: learned 24 frames {ms_l:.2f} ms RMSE {r_l:.4f}; plain {n_plain} frames {ms_p:.2f} ms "
          f"RMSE {r_p:.4f}; RMSE ratio {r_l / r_p:.2f}")
    assert abs(ms_p - ms_l) < 0.25 * ms_l
    assert r_l < 2.0 * r_p
