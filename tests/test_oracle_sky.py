"""CPU checks of the sky / atmosphere oracle (oracle/post.cpp) and of the
library's host-side atmosphere parameters.  The reference ships no golden
sky images (its shaders need Vulkan), so these are properties of the
restated algorithm: value ranges, monotonicity of the transmittance LUT,
the sun disc, and the azimuthal symmetry of the sky-view parameterisation.
"""
import numpy as np
import pytest

from oracle import post

SUN = np.array([-0.435286462, 0.818654716, 0.374606609], np.float32)  # sky.ixx:186
E = np.array([8.0, 8.0, 8.0], np.float32)
CAM = np.array([0.0, 0.0, 0.5], np.float32)


@pytest.fixture(scope="module")
def luts():
    a = post.earth()
    t = post.sky_transmittance(a)
    m = post.sky_multiscatter(a, t)
    v = post.sky_view(a, t, m, CAM, SUN, E)
    return a, t, m, v


def test_earth_params_match_library(built_lib):
    from minotert_gb300.sky import Atmosphere
    assert np.array_equal(Atmosphere.earth(), post.earth())


def test_transmittance_lut(luts):
    a, t, m, v = luts
    rgb = t[..., :3]
    assert np.isfinite(rgb).all() and (rgb > 0).all() and (rgb <= 1.0).all()
    assert (t[..., 3] == 1.0).all()
    # along a row the path to the atmosphere's top gets longer: transmittance
    # falls (x_mu = 0 looks straight up, x_mu = 1 grazes the horizon)
    assert (np.diff(rgb, axis=1) <= 1e-6).all()
    # blue is attenuated most (Rayleigh ~ lambda^-4)
    assert (rgb[..., 2] <= rgb[..., 0] + 1e-6).all()
    # near the top of the atmosphere looking up almost nothing is in the way
    assert (rgb[-1, 0] > 0.9999).all()


def test_multiscatter_lut(luts):
    a, t, m, v = luts
    assert np.isfinite(m).all() and (m[..., :3] >= 0).all()
    # sun well above the horizon (u > 0.6): multiple scattering is non-zero
    assert (m[:, 24:, :3] > 0).all()
    # sun far below the horizon at the ground: no light
    assert (m[0, :4, :3] < 1e-6).all()


def test_sky_view_lut(luts):
    a, t, m, v = luts
    assert np.isfinite(v).all() and (v[..., :3] >= 0).all()
    assert v[..., :3].max() > 0.1


def test_sun_disc_and_sky(luts):
    a, t, m, v = luts
    c_sun = post.sky_color(a, t, v, CAM, SUN, E, SUN)[0]
    assert (c_sun > 1e4).all()  # limb-darkened disc at ~120000 lux x transmittance
    rng = np.random.default_rng(3)
    d = rng.normal(size=(4096, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    away = d @ SUN < 0.99
    c = post.sky_color(a, t, v, CAM, SUN, E, d)
    assert np.isfinite(c).all() and (c >= 0).all()
    assert c[away].max() < 10.0
    # the clear sky is blue above the horizon
    up = (d[:, 2] > 0.3) & away
    assert (c[up, 2] > c[up, 0]).mean() > 0.95


def test_sky_is_symmetric_about_the_sun_plane(luts):
    # the sky view is parameterised by zenith angle and the cosine of the
    # azimuth to the sun, so mirroring a direction across the vertical
    # plane through the sun leaves its radiance unchanged
    a, t, m, v = luts
    up = np.array([0.0, 0.0, 1.0])
    sh = SUN.astype(np.float64) - (SUN @ up) * up
    sh /= np.linalg.norm(sh)
    nrm = np.cross(up, sh)  # normal of the mirror plane
    rng = np.random.default_rng(4)
    d = rng.normal(size=(512, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    dm = d - 2.0 * (d @ nrm)[:, None] * nrm[None, :]
    keep = (np.abs(d @ nrm) > 0.05) & (d @ SUN < 0.99)
    c1 = post.sky_color(a, t, v, CAM, SUN, E, d[keep].astype(np.float32))
    c2 = post.sky_color(a, t, v, CAM, SUN, E, dm[keep].astype(np.float32))
    assert np.allclose(c1, c2, rtol=1e-3, atol=1e-6)
