"""The measured workloads: seeded scenes, cameras, lights and trace settings.

heightfield_boxes_256   64x64-cell sine-octave heightfield (8,192 tris) +
                        32 boxes (384 tris); 256x256 pinhole, 1 spp, one
                        cosine-weighted diffuse bounce, 64x64 blue-noise
                        tile, albedo U[0.2,0.8], one directional light
icospheres_1080p        200 Perlin-displaced icospheres (4 subdivisions,
                        5,120 tris each, radius log-uniform[0.2,5]) on a
                        10,240-tri ground plane (1,034,240 tris); 1920x1080,
                        1 spp, 4 bounces, Russian roulette after bounce 2
"""
from __future__ import annotations

import math
from dataclasses import dataclass

from . import scene as _scene
from .pathtracer import Camera, Sky, TraceSettings


@dataclass
class Workload:
    name: str
    width: int
    height: int
    camera: Camera
    sky: Sky
    settings: TraceSettings
    mesh_fn: object
    seed: int = 1

    def mesh(self):
        return self.mesh_fn(self.seed)


SUN = (0.45, -0.35, 0.82)


def heightfield_boxes_256(seed: int = 1, size: int = 256) -> Workload:
    cam = Camera((size, size), math.radians(60.0), 0.01, (0.0, -27.0, 13.0), math.radians(90.0), math.radians(-28.0))
    return Workload("heightfield_boxes_256", size, size, cam, Sky((0.25, 0.32, 0.45), SUN, (2.5, 2.5, 2.5)),
                    TraceSettings(samples=1, bounces=1, rr_start=0),
                    lambda s: _scene.heightfield_boxes(s, 64, 32), seed)


def icospheres_1080p(seed: int = 1, width: int = 1920, height: int = 1080) -> Workload:
    cam = Camera((width, height), math.radians(60.0), 0.05, (0.0, -62.0, 40.0), math.radians(90.0),
                 math.radians(-36.0))
    return Workload("icospheres_1080p", width, height, cam, Sky((0.25, 0.32, 0.45), SUN, (2.5, 2.5, 2.5)),
                    TraceSettings(samples=1, bounces=4, rr_start=2),
                    lambda s: _scene.icospheres(s, 200, 4, 0.2, 5.0, 10240), seed)


@dataclass
class BatchScene:
    kind: str         # "heightfield" or "icospheres"
    target_tris: int
    rays: int         # width * height of the scene's camera
    width: int
    height: int
    seed: int

    def mesh(self):
        from ._lib import lib
        if self.kind == "heightfield":
            return _scene.heightfield_boxes(self.seed, lib().mrt_heightfield_grid_for(self.target_tris), 0)
        if self.target_tris >= 5120:
            return _scene.icospheres(self.seed, max(1, round(self.target_tris / 5120)), 4, 0.2, 5.0, 0)
        level = max(0, int(math.floor(math.log(max(self.target_tris, 20) / 20.0, 4))))
        return _scene.icospheres(self.seed, max(1, round(self.target_tris / (20 * 4 ** level))), level, 0.2, 5.0, 0)

    def rays_for(self, mesh):
        return _scene.pinhole_rays(mesh.lo, mesh.hi, self.width, self.height, seed=self.seed)


@dataclass
class BatchWorkload:
    name: str
    scenes: list
    settings: TraceSettings
    sky: Sky


def batched64(seed: int = 1, count: int = 64, tri_range=(1_000, 500_000), ray_range=(16_000, 2_000_000),
              bounces: int = 3) -> BatchWorkload:
    """`count` independent scenes alternating heightfields and icosphere
    clusters, triangle counts log-uniform in tri_range, ray counts uniform
    in ray_range (square pinhole images), closest-hit bounce loop of
    `bounces` diffuse bounces."""
    import numpy as np
    rng = np.random.default_rng(seed)
    scenes = []
    for s in range(count):
        t = int(round(math.exp(rng.uniform(math.log(tri_range[0]), math.log(tri_range[1])))))
        r = int(rng.uniform(*ray_range))
        w = max(1, int(round(math.sqrt(r))))
        scenes.append(BatchScene("heightfield" if s % 2 == 0 else "icospheres", t, w * w, w, w, seed * 1000 + s))
    return BatchWorkload(f"batched{count}", scenes, TraceSettings(samples=1, bounces=bounces, rr_start=0),
                         Sky((0.6, 0.7, 0.9), None))


WORKLOADS = {"heightfield_boxes_256": heightfield_boxes_256, "icospheres_1080p": icospheres_1080p,
             "batched64": batched64}
