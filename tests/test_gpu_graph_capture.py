"""A whole frame (primary + secondary rays; with the default schedule the
shadow rays fork to the context's second stream and join back) captured
into a CUDA graph by the caller in relaxed capture mode, replayed, gives the
directly launched frame's image bit for bit.  The capture and replay go
through PyTorch's graph API on a PyTorch stream whose handle the C ABI
receives.  (The global and thread-local capture modes reject a call of the
secondary pass; the primary pass captures in global mode too.)"""
import numpy as np
import pytest

from minotert_gb300.pathtracer import Pathtracer, TraceSettings
from minotert_gb300.scene import DeviceScene

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("overlap", [1, 0])
def test_frame_captured_in_a_graph(ctx, hf_workload, blue_noise, overlap):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device for PyTorch")
    wl, mesh, bvh = hf_workload
    ds = DeviceScene.triangles(ctx, mesh, bvh)
    saved = int(ctx.tuning().overlap_shadow)
    ctx.set_tuning(overlap_shadow=overlap)  # 1: the fork / join is part of what is captured
    pt = Pathtracer(ctx, ds, full_gbuffer=False)
    W, H = wl.width, wl.height
    color = ctx.alloc(12 * W * H)
    settings = TraceSettings(samples=1, bounces=4, rr_start=2, rng_mode=1)
    ts = torch.cuda.Stream()
    sh = ts.cuda_stream

    def frame():
        pt.frame_counter = 9
        gb = pt.primaryRays((W, H), wl.camera, wl.camera, sh)
        pt.secondaryRays(gb, wl.camera, wl.sky, blue_noise, settings, color=color, stream=sh)

    frame()  # allocates the wavefront buffers and g-buffer outside the capture
    ts.synchronize()
    ref = color.download(np.float32, (H, W, 3)).copy()
    color.zero()
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=ts, capture_error_mode="relaxed"):
        frame()
    ts.synchronize()
    assert not color.download(np.float32, (H, W, 3)).any()  # capture records, does not run
    g.replay()
    torch.cuda.synchronize()
    img = color.download(np.float32, (H, W, 3))
    ctx.set_tuning(overlap_shadow=saved)
    assert np.array_equal(img.view(np.uint32), ref.view(np.uint32))
    assert ctx.status() == 0
