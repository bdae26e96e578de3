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


WORKLOADS = {"heightfield_boxes_256": heightfield_boxes_256, "icospheres_1080p": icospheres_1080p}
