"""The headless renderer (mrt_renderer_*) against the same chain of C-ABI
calls made one by one: the reference's frame (atmosphere sky, 8 x 8
secondary samples, bilateral denoiser, AMD tonemapper) on scene 0, and a
reprojected accumulation under camera motion on the triangle scene.  The
kernels are deterministic, so the outputs must be identical."""
import numpy as np
import pytest

from minotert_gb300.pathtracer import Camera, Pathtracer, Sky as ConstSky, TraceSettings, camera_consts
from minotert_gb300.post import BilateralParams, Denoiser, ReprojectParams, Tonemapper, reproject
from minotert_gb300.renderer import (ACCUM_REPROJECT, DENOISE_NONE, SKY_CONSTANT, RenderSettings, Renderer,
                                     write_pfm, write_ppm)
from minotert_gb300.scene import DeviceScene, reference_spheres
from minotert_gb300.sky import Atmosphere, Sky

pytestmark = pytest.mark.gpu


def test_reference_frame_matches_the_call_chain(ctx, reference_blue_noise, tmp_path):
    # the reference's scene with its own blue-noise texture, as
    # Renderer_impl's constructor loads it
    W, H = 192, 108
    ds = DeviceScene.from_spheres(ctx, reference_spheres())
    cam = Camera.reference(W, H)
    r = Renderer(ctx, ds, W, H, blue_noise=reference_blue_noise)
    frames = 2
    for f in range(frames):
        r.draw(cam)
    rgba, hdr = r.read()
    assert (rgba[..., 3] == 255).all() and rgba[..., :3].std() > 5

    # the same frame (frame counter 1) call by call
    atmo = Atmosphere(ctx)
    view = Sky().createView(atmo, np.array(cam.position, np.float32))
    pt = Pathtracer(ctx, ds)
    pt.frame_counter = frames - 1
    gb = pt.primaryRays((W, H), cam, cam)
    col = pt.secondaryRays(gb, cam, ConstSky(radiance=(0.0, 0.0, 0.0), sun_dir=None), reference_blue_noise,
                           TraceSettings(samples=8, bounces=8), skyView=view)
    den = Denoiser(ctx).bilateral(col, gb, cam, BilateralParams(), frame_counter=frames - 1)
    out = Tonemapper(ctx).amd(den, W, H, 1.0)
    assert np.array_equal(hdr, den.download(np.float32, (H, W, 3)))
    assert np.array_equal(rgba, out.download(np.uint8, (H, W, 4)))

    write_ppm(tmp_path / "frame.ppm", rgba)
    data = (tmp_path / "frame.ppm").read_bytes()
    assert data.startswith(b"P6\n192 108\n255\n") and len(data) == len(b"P6\n192 108\n255\n") + W * H * 3
    write_pfm(tmp_path / "frame.pfm", hdr)
    pf = (tmp_path / "frame.pfm").read_bytes()
    head = b"PF\n192 108\n-1.0\n"
    assert pf.startswith(head)
    back = np.frombuffer(pf[len(head):], np.float32).reshape(H, W, 3)[::-1]
    assert np.array_equal(back, hdr)
    r.close()


def test_reprojected_accumulation_matches_the_call_chain(ctx, hf_workload, blue_noise):
    wl, mesh, bvh = hf_workload
    W, H = 200, 120
    c = wl.camera
    cams = [Camera((W, H), c.verticalFov, c.nearPlane, (c.position[0] + 0.2 * k, c.position[1], c.position[2]),
                   c.yaw + 0.01 * k, c.pitch) for k in range(3)]
    ds = DeviceScene.triangles(ctx, mesh, bvh)
    s = RenderSettings.defaults()
    s.trace.samples, s.trace.max_bounces, s.trace.rng_mode = 1, 2, 1
    s.sky_mode, s.accumulation, s.denoise = SKY_CONSTANT, ACCUM_REPROJECT, DENOISE_NONE
    for k in range(3):
        s.trace.sky_radiance[k] = (0.25, 0.32, 0.45)[k]
    r = Renderer(ctx, ds, W, H, blue_noise=blue_noise)
    for cam in cams:
        r.draw(cam, s)
    rgba, hdr = r.read()

    # call by call: frame 0 starts the history, frames 1-2 reproject it
    pt = Pathtracer(ctx, ds)
    prm = ReprojectParams(32.0, 0.9, 0.05)
    hist = hist_len = gb_prev = None
    for f, cam in enumerate(cams):
        prev = cams[f - 1] if f else cam
        pt_f = Pathtracer(ctx, ds)
        pt_f.frame_counter = f
        gb = pt_f.primaryRays((W, H), cam, prev)
        col = pt_f.secondaryRays(gb, cam, ConstSky(radiance=(0.25, 0.32, 0.45), sun_dir=None), blue_noise,
                                 TraceSettings(samples=1, bounces=2, rng_mode=1))
        consts = camera_consts(cam, prev, f)
        out, out_len = ctx.alloc(12 * W * H), ctx.alloc(4 * W * H)
        if hist is None:
            h0, l0 = ctx.alloc(12 * W * H), ctx.alloc(4 * W * H)
            h0.upload(col.download(np.float32, (H, W, 3)))
            l0.upload(np.zeros((H, W), np.float32))
            reproject(ctx, gb, gb, consts, col, h0, l0, out, out_len, prm)
        else:
            reproject(ctx, gb, gb_prev, consts, col, hist, hist_len, out, out_len, prm)
        hist, hist_len, gb_prev = out, out_len, gb
        pt = pt_f  # keep this frame's g-buffer alive
        gb_keep = gb
    ref = hist.download(np.float32, (H, W, 3))
    assert np.array_equal(hdr, ref)
    lens = hist_len.download(np.float32, (H, W))
    vis = gb_keep.download()["visibility"]
    assert (lens[vis != 0xFFFFFFFF] == 3.0).mean() > 0.8
