import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


def _has_gpu() -> bool:
    """Asks the CUDA driver directly (no torch import needed)."""
    import ctypes
    try:
        cuda = ctypes.CDLL("libcuda.so.1")
    except OSError:
        return False
    if cuda.cuInit(0) != 0:
        return False
    n = ctypes.c_int(0)
    return cuda.cuDeviceGetCount(ctypes.byref(n)) == 0 and n.value > 0


def pytest_collection_modifyitems(config, items):
    if _has_gpu():
        return
    skip = pytest.mark.skip(reason="no GPU in this environment")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def built_lib():
    from minotert_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def ctx(built_lib):
    from minotert_gb300._lib import Context
    c = Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def hf_workload(built_lib):
    """heightfield + boxes scene (8,576 triangles), 256x256, with its BVH."""
    from minotert_gb300 import scene, workloads
    wl = workloads.heightfield_boxes_256()
    mesh = wl.mesh()
    bvh = scene.build_bvh8(mesh)
    return wl, mesh, bvh


@pytest.fixture(scope="session")
def ico_workload(built_lib):
    """icosphere field (1,034,240 triangles), 1920x1080, with its BVH."""
    from minotert_gb300 import scene, workloads
    wl = workloads.icospheres_1080p()
    mesh = wl.mesh()
    bvh = scene.build_bvh8(mesh)
    return wl, mesh, bvh


def asset_blue_noise() -> np.ndarray:
    """The reference's blue-noise texture (assets/blue_noise.png, 256 x 256
    RGBA8), decoded into the committed fixture by golden/make_blue_noise.py."""
    return np.load(ROOT / "tests" / "golden" / "blue_noise_asset.npz")["rgba"]


@pytest.fixture(scope="session")
def blue_noise(built_lib):
    """The measured configurations' 64 x 64 tile: the asset's top-left crop."""
    from minotert_gb300 import scene
    return scene.blue_noise_tile(asset_blue_noise(), 64)


@pytest.fixture(scope="session")
def reference_blue_noise(built_lib):
    """The whole 256 x 256 asset, fetched at Gid % 256 like secondaryRays.comp:125."""
    return asset_blue_noise()


def oracle_consts(camera, frame=0, prev=None):
    import oracle
    w, h = camera.viewport
    pv = None if prev is None else (prev.position, prev.yaw, prev.pitch)
    return oracle.camera_consts(camera.position, camera.yaw, camera.pitch, camera.verticalFov, camera.nearPlane, w,
                                h, prev=pv, frame=frame)


def random_rays(n, lo, hi, seed=0, margin=2.0):
    from minotert_gb300._lib import RAY_DTYPE
    rng = np.random.default_rng(seed)
    rays = np.zeros(n, RAY_DTYPE)
    rays["org"] = rng.uniform(np.asarray(lo) - margin, np.asarray(hi) + margin, size=(n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays["dir"] = d.astype(np.float32)
    rays["tmin"] = 0.0
    rays["tmax"] = np.inf
    return rays
