"""CPU checks of the post-processing oracle (oracle/post.cpp,
orc_reproject in oracle/oracle.cpp): properties the reference's shaders
have by construction -- the bilateral filter keeps flat regions and stops
at depth edges, the tonemappers are monotonic with the sRGB end points,
reprojection with a still camera is an exact running mean."""
import numpy as np

from oracle import post


def _half(a):
    return np.asarray(a, np.float32).astype(np.float16).view(np.uint16)


def _planes(h, w, depth=0.5):
    z = np.full((h, w), depth, np.float32)
    n = np.zeros((h, w, 4), np.float32)
    n[..., 2] = 1.0
    return _half(z), _half(n)


def test_bilateral_keeps_a_flat_image():
    z, n = _planes(40, 48)
    col = np.full((40, 48, 3), 0.37, np.float32)
    out = post.bilateral(col, z, n, dither=False)
    assert np.allclose(out, 0.37, rtol=1e-6, atol=0)


def test_bilateral_dither_is_the_reference_pcg():
    z, n = _planes(8, 8)
    col = np.zeros((8, 8, 3), np.float32)
    out = post.bilateral(col, z, n, frame=3, dither=True)
    # bilateral.comp:68-70: randomFloat(x*709 + y*1153 + frame*1361) * 0.005
    from oracle import random_float
    for (y, x) in [(0, 0), (5, 2), (7, 7)]:
        f, _ = random_float((x * 709 + y * 1153 + 3 * 1361) & 0xFFFFFFFF)
        assert np.allclose(out[y, x], np.float32(f) * np.float32(0.005), rtol=0, atol=0)


def test_bilateral_stops_at_depth_edges():
    h, w = 32, 64
    z = np.full((h, w), 0.5, np.float32)
    z[:, w // 2:] = 0.05  # ten times farther
    n = np.zeros((h, w, 4), np.float32)
    n[..., 2] = 1.0
    col = np.zeros((h, w, 3), np.float32)
    col[:, w // 2:] = 1.0
    out = post.bilateral(col, _half(z), _half(n), dither=False)
    assert np.abs(out[:, : w // 2 - 1]).max() < 1e-6
    assert np.abs(out[:, w // 2 + 1:] - 1.0).max() < 1e-6


def test_bilateral_smooths_noise():
    rng = np.random.default_rng(0)
    z, n = _planes(64, 64)
    col = rng.exponential(0.5, size=(64, 64, 3)).astype(np.float32)
    out = post.bilateral(col, z, n, dither=False)
    assert out.std() < 0.25 * col.std()
    assert abs(out.mean() - col.mean()) < 0.05 * col.mean()


def test_tonemap_end_points_and_monotonic():
    ramp = np.linspace(0.0, 20.0, 4001, dtype=np.float32)
    col = np.repeat(ramp[:, None], 3, axis=1)
    for mode in post.TONEMAP_MODES:
        out = post.tonemap(col, mode)
        assert out[0, 0] == 0 and (out[:, 3] == 255).all()
        assert (np.diff(out[:, 0].astype(int)) >= 0).all(), mode
    lin = post.tonemap(np.array([[1.0, 0.5, 0.0031308 * 0.5]], np.float32), "linear")[0]
    # sRGB: 1 -> 255; 0.5 -> 1.055 * 0.5^(1/2.4) - 0.055 = 0.7354 -> 188;
    # below 0.0031308 linear: 12.92 * 0.0015654 = 0.0202 -> 5
    assert lin[0] == 255 and lin[1] == 188 and lin[2] == 5


def _gbuffer(wl, bvh, mesh, cam, prev, w, h):
    import oracle
    from conftest import oracle_consts
    c = oracle_consts(cam, prev=prev)
    return c, oracle.primary(c, w, h, nodes=bvh.nodes, tris=bvh.tris, mats=mesh.mats)


def test_reprojection_still_camera_is_a_running_mean(hf_workload):
    wl, mesh, bvh = hf_workload
    w, h = 96, 64
    cam = wl.camera
    cam = type(cam)((w, h), cam.verticalFov, cam.nearPlane, cam.position, cam.yaw, cam.pitch)
    c, g = _gbuffer(wl, bvh, mesh, cam, cam, w, h)
    rng = np.random.default_rng(5)
    sample = rng.random((h, w, 3), np.float32)
    hist = rng.random((h, w, 3), np.float32)
    hist_len = np.full((h, w), 3.0, np.float32)
    out, out_len = post.reproject(c, w, h, g["visibility"], g["hit_t"], g["normal"], g["motion"], g["visibility"],
                                  g["depth"], g["normal"], sample, hist, hist_len)
    sky = g["visibility"] == 0xFFFFFFFF
    assert np.array_equal(out[sky], sample[sky]) and (out_len[sky] == 1.0).all()
    hit = ~sky
    assert hit.mean() > 0.3
    # the previous-frame position is the pixel centre itself: one tap
    assert (out_len[hit] == 4.0).mean() > 0.99
    keep = hit & (out_len == 4.0)
    expect = hist + (sample - hist) * np.float32(0.25)
    assert np.array_equal(out[keep], expect[keep])


def test_reprojection_resets_on_disocclusion(hf_workload):
    wl, mesh, bvh = hf_workload
    w, h = 96, 64
    cam = wl.camera
    cam = type(cam)((w, h), cam.verticalFov, cam.nearPlane, cam.position, cam.yaw, cam.pitch)
    c, g = _gbuffer(wl, bvh, mesh, cam, cam, w, h)
    pvis = np.full_like(g["visibility"], 0xFFFFFFFF)  # the previous frame saw only sky
    rng = np.random.default_rng(6)
    sample = rng.random((h, w, 3), np.float32)
    out, out_len = post.reproject(c, w, h, g["visibility"], g["hit_t"], g["normal"], g["motion"], pvis, g["depth"],
                                  g["normal"], sample, np.ones((h, w, 3), np.float32), np.full((h, w), 9.0, np.float32))
    assert np.array_equal(out, sample) and (out_len == 1.0).all()


def test_reprojection_follows_camera_motion(hf_workload):
    # a small yaw: history taps come from the neighbouring pixels the motion
    # vectors point to, and the history length grows where they agree
    wl, mesh, bvh = hf_workload
    w, h = 96, 64
    cam0 = wl.camera
    cam0 = type(cam0)((w, h), cam0.verticalFov, cam0.nearPlane, cam0.position, cam0.yaw, cam0.pitch)
    cam1 = type(cam0)((w, h), cam0.verticalFov, cam0.nearPlane, cam0.position, cam0.yaw + 0.01, cam0.pitch)
    c0, g0 = _gbuffer(wl, bvh, mesh, cam0, cam0, w, h)
    c1, g1 = _gbuffer(wl, bvh, mesh, cam1, cam0, w, h)
    motion = g1["motion"].view(np.float16).astype(np.float32)
    hit = g1["visibility"] != 0xFFFFFFFF
    assert np.abs(motion[hit]).max() > 0.5  # the camera turned by about a pixel
    const = np.full((h, w, 3), 0.25, np.float32)
    out, out_len = post.reproject(c1, w, h, g1["visibility"], g1["hit_t"], g1["normal"], g1["motion"],
                                  g0["visibility"], g0["depth"], g0["normal"], const, const,
                                  np.full((h, w), 5.0, np.float32))
    assert (out_len[hit] == 6.0).mean() > 0.9
    assert np.allclose(out, 0.25, rtol=1e-6)


def test_exp_cw_accuracy():
    # the shared exponential is within 2 ulp of e^x over the float range it
    # serves, flushes below 2^-126 and saturates above 88
    rng = np.random.default_rng(9)
    x = np.concatenate([rng.uniform(-87.0, 88.0, 3000), rng.uniform(-1.0, 1.0, 3000),
                        [0.0, -0.0, 1.0, -1.0, 1e-8, -1e-8, 88.0, -86.9]]).astype(np.float32)
    got = post.exp_cw(x).astype(np.float64)
    ref = np.exp(x.astype(np.float64))
    ulp = np.spacing(ref.astype(np.float32)).astype(np.float64)
    normal = ref >= 2.0 ** -126
    assert (np.abs(got - ref)[normal] <= 2.0 * ulp[normal]).all()
    assert post.exp_cw(np.float32(0.0)) == 1.0
    assert post.exp_cw(np.float32(-100.0)) == 0.0 and np.isinf(post.exp_cw(np.float32(89.0)))
