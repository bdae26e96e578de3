"""Camera windows (an off-centre projection rendering a sub-window of the
viewport's frustum) on the host: the window's rays are the full frame's
rays of the same pixels, and the narrowed projection stays the inverse of
the narrowed inverse projection."""
import math

import numpy as np

from minotert_gb300.pathtracer import Camera, camera_consts, primary_rays_host


def _cam(window=None):
    return Camera((192, 128), math.radians(60.0), 0.01, (18.0, 6.0, 11.0), math.atan2(-6.0, -18.0), -0.5,
                  window=window)


def test_window_rays_are_the_full_frames_rays(built_lib):
    full = primary_rays_host(_cam(), 192, 128).reshape(128, 192)
    for x0, y0, w, h in [(40, 24, 64, 48), (0, 0, 32, 32), (160, 96, 32, 32), (7, 13, 100, 20)]:
        sub = primary_rays_host(_cam((x0, y0, w, h)), w, h).reshape(h, w)
        crop = full[y0:y0 + h, x0:x0 + w]
        assert np.array_equal(sub["org"], crop["org"])
        assert np.abs(sub["dir"] - crop["dir"]).max() < 3e-7


def test_window_projection_is_consistent(built_lib):
    c = camera_consts(_cam((40, 24, 64, 48)))
    P = np.array(c.projection[:], np.float64).reshape(4, 4).T
    Pi = np.array(c.inv_projection[:], np.float64).reshape(4, 4).T
    err = np.abs(P @ Pi - np.eye(4)).max()
    assert err < 1e-5, err
    full = camera_consts(_cam())
    # depth (NDC z) and the homogeneous w row are those of the full frustum
    Pf = np.array(full.projection[:], np.float64).reshape(4, 4).T
    assert np.allclose(P[2:], Pf[2:])
