"""GPU parity of the post-processing kernels (mrt_cuda_bilateral,
mrt_cuda_tonemap, mrt_cuda_reproject) against the CPU oracle.

Bars: reprojection and the bilateral filter bit-identical (explicitly
rounded + - * / on both sides, and the filter's weights through the shared
exp_cw); tonemap within one 8-bit step with at least 99.9% of channels
identical (CUDA's powf / expf in the curves and the sRGB encode).
"""
import ctypes as C

import numpy as np
import pytest

from conftest import oracle_consts
from minotert_gb300._lib import MRT_ERANGE, BilateralParams as BP_C, lib, ptr
from minotert_gb300.pathtracer import Camera, Pathtracer, Sky, TraceSettings, camera_consts
from minotert_gb300.post import (AMDParams, BilateralParams, Denoiser, ReprojectParams, Tonemapper, UchimuraParams,
                                 reproject)
from minotert_gb300.scene import DeviceScene
from oracle import post

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def hf_frame(ctx, hf_workload, blue_noise):
    """A 1-spp path-traced frame of the heightfield scene with a full
    g-buffer, at an odd size that is not a multiple of the 16x16 tiles."""
    wl, mesh, bvh = hf_workload
    W, H = 250, 130
    cam = wl.camera
    cam = Camera((W, H), cam.verticalFov, cam.nearPlane, cam.position, cam.yaw, cam.pitch)
    ds = DeviceScene.triangles(ctx, mesh, bvh)
    pt = Pathtracer(ctx, ds, full_gbuffer=True)
    gb = pt.primaryRays((W, H), cam, cam)
    col = pt.secondaryRays(gb, cam, Sky(), blue_noise, TraceSettings(samples=1, bounces=2, rng_mode=1))
    return cam, ds, pt, gb, col, W, H


@pytest.mark.parametrize("sigma,k_sigma,dither,thr", [(5.0, 2.0, True, 0.12), (2.0, 1.5, False, 0.12),
                                                      (8.0, 3.0, False, 0.12), (4.0, 2.0, False, 0.05),
                                                      (1.0, 0.4, True, 0.3)])
def test_bilateral_vs_oracle(ctx, hf_frame, sigma, k_sigma, dither, thr):
    # threshold 0.05 puts the weights' exponent beyond 88, the kernel form
    # that keeps the exponential's range handling (the shader's weights then
    # overflow where neighbours agree, giving inf / NaN like the oracle's;
    # NaN payloads differ between machines, so those pixels compare by
    # class); sigma 1 x 0.4 rounds to radius 0 (the centre tap alone)
    cam, ds, pt, gb, col, W, H = hf_frame
    out = Denoiser(ctx).bilateral(col, gb, cam, BilateralParams(sigma, k_sigma, thr), frame_counter=7,
                                  dither=dither)
    got = out.download(np.float32, (H, W, 3))
    g = gb.download()
    src = col.download(np.float32, (H, W, 3))
    ref = post.bilateral(src, g["depth"], g["normal"], sigma, k_sigma, thr, cam.nearPlane, 7, dither)
    fin = np.isfinite(ref)
    if thr >= 0.1:
        assert fin.all()
    assert np.array_equal(np.isfinite(got), fin) and np.array_equal(np.isnan(got), np.isnan(ref))
    assert np.array_equal(got[fin].view(np.uint32), ref[fin].view(np.uint32))
    assert fin.mean() > 0.01


def test_bilateral_smooths_a_flat_surface(ctx):
    # noise on one plane at constant depth: every tap agrees in depth and
    # normal, so the filter is the plain Gaussian and removes most noise
    from minotert_gb300.pathtracer import GBuffer
    W, H = 96, 80
    rng = np.random.default_rng(4)
    noisy = rng.exponential(0.5, size=(H, W, 3)).astype(np.float32)
    depth = np.full((H, W), 0.25, np.float16).view(np.uint16)
    nrm = np.zeros((H, W, 4), np.float16)
    nrm[..., 2] = 1.0
    gb = GBuffer(W, H, ctx.alloc(4 * W * H), ctx.alloc(4 * W * H), ctx.to_device(depth),
                 ctx.to_device(nrm.view(np.uint16)), None)
    cam = Camera((W, H), 1.0, 0.1, (0.0, 0.0, 0.0), 0.0, 0.0)
    out = Denoiser(ctx).bilateral(ctx.to_device(noisy), gb, cam, dither=False)
    got = out.download(np.float32, (H, W, 3))
    ref = post.bilateral(noisy, depth, nrm.view(np.uint16), near_plane=0.1, dither=False)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    inner = got[12:-12, 12:-12]
    assert inner.std() < 0.15 * noisy.std()


def test_bilateral_radius_limit(ctx, hf_frame):
    cam, ds, pt, gb, col, W, H = hf_frame
    p = BP_C()
    lib().mrt_bilateral_defaults(C.byref(p))
    p.sigma, p.k_sigma = 10.0, 3.0  # radius 30 > 24
    out = ctx.alloc(12 * W * H)
    rc = lib().mrt_cuda_bilateral(ctx.handle, C.byref(gb.c()), ptr(col), C.byref(p), ptr(out), None)
    assert rc == MRT_ERANGE


@pytest.mark.parametrize("mode", ["linear", "reinhard", "hable", "aces", "uchimura", "amd"])
def test_tonemap_vs_oracle(ctx, mode):
    rng = np.random.default_rng(21)
    n = 1 << 16
    col = np.concatenate([rng.exponential(0.6, size=(n - 6, 3)),
                          [[0, 0, 0], [1, 1, 1], [0.18, 0.18, 0.18], [30, 2, 0.1], [1e-5, 0, 0], [5, 5, 5]]])
    col = np.ascontiguousarray(col, np.float32)
    d_col = ctx.to_device(col)
    tm = Tonemapper(ctx)
    W, H = n, 1
    exposure = 1.3
    if mode == "uchimura":
        out = tm.uchimura(d_col, W, H, exposure, UchimuraParams())
    elif mode == "amd":
        out = tm.amd(d_col, W, H, exposure, AMDParams())
    elif mode == "reinhard":
        out = tm.reinhard(d_col, W, H, exposure, 8.0)
    else:
        out = getattr(tm, mode)(d_col, W, H, exposure)
    got = out.download(np.uint8, (n, 4))
    ref = post.tonemap(col, mode, post.tonemap_params(exposure=exposure))
    diff = np.abs(got.astype(int) - ref.astype(int))
    assert diff.max() <= 1
    assert (diff == 0).mean() > 0.999
    assert (got[:, 3] == 255).all()


def test_reprojection_bit_exact_under_camera_motion(ctx, hf_workload, blue_noise):
    wl, mesh, bvh = hf_workload
    W, H = 250, 130
    c0 = wl.camera
    cam0 = Camera((W, H), c0.verticalFov, c0.nearPlane, c0.position, c0.yaw, c0.pitch)
    cam1 = Camera((W, H), c0.verticalFov, c0.nearPlane, (c0.position[0] + 0.3, c0.position[1], c0.position[2]),
                  c0.yaw + 0.012, c0.pitch - 0.004)
    ds = DeviceScene.triangles(ctx, mesh, bvh)
    pt0, pt1 = Pathtracer(ctx, ds), Pathtracer(ctx, ds)
    gb0 = pt0.primaryRays((W, H), cam0, cam0)
    pt1.frame_counter = 1
    gb1 = pt1.primaryRays((W, H), cam1, cam0)
    rng = np.random.default_rng(8)
    sample = rng.random((H, W, 3), np.float32)
    hist = rng.random((H, W, 3), np.float32)
    hist_len = rng.integers(1, 20, size=(H, W)).astype(np.float32)
    d_s, d_h, d_l = ctx.to_device(sample), ctx.to_device(hist), ctx.to_device(hist_len)
    d_o, d_ol = ctx.alloc(12 * W * H), ctx.alloc(4 * W * H)
    consts = camera_consts(cam1, cam0, 1)
    prm = ReprojectParams(max_history=16.0, normal_cos=0.9, depth_rel=0.05)
    reproject(ctx, gb1, gb0, consts, d_s, d_h, d_l, d_o, d_ol, prm)
    got, got_len = d_o.download(np.float32, (H, W, 3)), d_ol.download(np.float32, (H, W))
    g0, g1 = gb0.download(), gb1.download()
    oc = oracle_consts(cam1, frame=1, prev=cam0)
    ref, ref_len = post.reproject(oc, W, H, g1["visibility"], g1["hit_t"], g1["normal"], g1["motion"],
                                  g0["visibility"], g0["depth"], g0["normal"], sample, hist, hist_len, 16.0, 0.9,
                                  0.05)
    assert np.array_equal(got_len, ref_len)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    hit = g1["visibility"] != 0xFFFFFFFF
    assert (got_len[hit] > 1.0).mean() > 0.8  # most of the history survives the move
