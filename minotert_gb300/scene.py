"""Host-side scene modules: procedural meshes, the BVH8 builder and the
device upload (mrt_host.h / mrt_cuda_scene_upload_*)."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from ._lib import (MAT_DTYPE, NODE_DTYPE, SPHERE_DTYPE, TRI_DTYPE, Bvh8_C, BvhBuildParams, Context, Mesh_C, MrtError,
                   lib, ptr)


@dataclass
class Mesh:
    verts: np.ndarray   # (n, 9) float32: v0 v1 v2
    mats: np.ndarray    # (n,) MAT_DTYPE: unit normal + RGBA8 albedo
    lo: np.ndarray
    hi: np.ndarray

    @property
    def tri_count(self) -> int:
        return int(self.verts.shape[0])

    def albedo(self) -> np.ndarray:
        a = self.mats["albedo"]
        return np.stack([(a >> s) & 0xFF for s in (0, 8, 16)], axis=1).astype(np.float32) / np.float32(255.0)


def _take_mesh(m: Mesh_C) -> Mesh:
    n = m.tri_count
    verts = np.ctypeslib.as_array(m.verts, shape=(n * 9,)).reshape(n, 9).copy()
    mats = np.frombuffer((C.c_char * (n * 16)).from_address(m.materials), dtype=MAT_DTYPE, count=n).copy()
    mesh = Mesh(verts, mats, np.array(m.bounds_lo[:], np.float32), np.array(m.bounds_hi[:], np.float32))
    lib().mrt_mesh_free(C.byref(m))
    return mesh


def heightfield_boxes(seed: int = 1, grid: int = 64, boxes: int = 32) -> Mesh:
    """Heightfield (grid x grid cells, 4 sine octaves) + axis-aligned boxes."""
    m = Mesh_C()
    rc = lib().mrt_scene_heightfield_boxes(seed, grid, boxes, C.byref(m))
    if rc:
        raise MrtError(rc, "mrt_scene_heightfield_boxes")
    return _take_mesh(m)


def icospheres(seed: int = 1, spheres: int = 200, levels: int = 4, rmin: float = 0.2, rmax: float = 5.0,
               ground_tris: int = 10240) -> Mesh:
    """Perlin-displaced icospheres on a ground plane."""
    m = Mesh_C()
    rc = lib().mrt_scene_icospheres(seed, spheres, levels, rmin, rmax, ground_tris, C.byref(m))
    if rc:
        raise MrtError(rc, "mrt_scene_icospheres")
    return _take_mesh(m)


def concat(meshes) -> Mesh:
    verts = np.concatenate([m.verts for m in meshes])
    mats = np.concatenate([m.mats for m in meshes])
    return Mesh(verts, mats, verts.reshape(-1, 3).min(0), verts.reshape(-1, 3).max(0))


@dataclass
class Bvh8:
    nodes: np.ndarray   # NODE_DTYPE
    tris: np.ndarray    # TRI_DTYPE (leaf order)
    depth: int
    leaf_count: int
    build_ms: float


def build_bvh8(mesh_or_verts, bins: int = 64, threads: int = 0, trav_cost: float = 0.5, collapse: int = 0,
               prim_cost: float = 0.3) -> Bvh8:
    """SAH BVH2 collapsed to BVH8: collapse 0 = greedy largest-area
    opening (default), 1 = SAH-optimal (dynamic programming, with prim_cost
    the cost of a triangle test relative to an 8-wide node visit)."""
    verts = mesh_or_verts.verts if isinstance(mesh_or_verts, Mesh) else np.asarray(mesh_or_verts)
    verts = np.ascontiguousarray(verts, dtype=np.float32).reshape(-1, 9)
    out = Bvh8_C()
    params = BvhBuildParams(bins, 3, threads, int(round(trav_cost * 100)), collapse, int(round(prim_cost * 100)))
    rc = lib().mrt_bvh8_build(ptr(verts), verts.shape[0], C.byref(params), C.byref(out))
    if rc:
        raise MrtError(rc, "mrt_bvh8_build")
    nodes = np.frombuffer((C.c_char * (out.node_count * 128)).from_address(out.nodes), dtype=NODE_DTYPE).copy()
    tris = np.frombuffer((C.c_char * (out.tri_count * 48)).from_address(out.tris), dtype=TRI_DTYPE).copy()
    res = Bvh8(nodes, tris, out.depth, out.leaf_count, out.build_ms)
    lib().mrt_bvh8_free(C.byref(out))
    return res


def reference_spheres() -> np.ndarray:
    """The reference's 5 spheres (src/gpu/scene.glsl:4-11)."""
    s = np.zeros(5, dtype=SPHERE_DTYPE)
    lib().mrt_scene_reference(ptr(s))
    return s


def load_png(path_or_bytes) -> np.ndarray:
    """RGBA8 image (h, w, 4) from a PNG file or its bytes, decoded like the
    reference's asset loader (renderer.ixx:101-110, lodepng to RGBA8)."""
    w, h = C.c_uint32(0), C.c_uint32(0)
    if isinstance(path_or_bytes, (bytes, bytearray)):
        data = np.frombuffer(bytes(path_or_bytes), np.uint8)
        call = lambda out, n: lib().mrt_png_decode_rgba8(ptr(data), data.nbytes, out, n, C.byref(w), C.byref(h))
    else:
        path = str(path_or_bytes).encode()
        call = lambda out, n: lib().mrt_png_load_rgba8(path, out, n, C.byref(w), C.byref(h))
    rc = call(None, 0)
    if rc:
        raise MrtError(rc, "PNG decode")
    out = np.zeros((h.value, w.value, 4), np.uint8)
    rc = call(ptr(out), out.nbytes)
    if rc:
        raise MrtError(rc, "PNG decode")
    return out


def blue_noise_tile(rgba: np.ndarray, size: int = 64) -> np.ndarray:
    """The top-left size x size crop of an RGBA8 blue-noise texture: the tile
    the measured workloads sample at Gid % size (the reference samples its
    whole 256 x 256 texture at Gid % 256, secondaryRays.comp:125; kernels
    read channels R and G)."""
    return np.ascontiguousarray(rgba[:size, :size])


def blue_noise(seed: int = 1, size: int = 64) -> np.ndarray:
    """size x size x 4 RGBA8 blue-noise tile (void-and-cluster)."""
    out = np.zeros((size, size, 4), dtype=np.uint8)
    rc = lib().mrt_blue_noise_generate(seed, size, ptr(out))
    if rc:
        raise MrtError(rc, "mrt_blue_noise_generate")
    return out


def accumulate_copies(ctx: Context, acc, x, groups: int, copies: int, count: int, scale: float, stream=None):
    """acc[g][i] += scale * sum_c x[g][c][i] on the device (float32 buffers,
    count a multiple of 4): per-pixel sample means of ray copies laid out
    [scene][copy][pixel]."""
    ctx.check(lib().mrt_cuda_accumulate_copies(ctx.handle, ptr(acc), ptr(x), groups, copies, count, float(scale),
                                               ptr(stream)), "accumulate_copies")


class DeviceBatch:
    """Many scenes concatenated into one device BVH (mrt_batch): rays of all
    scenes trace in one persistent launch.  Hit ids are batch-wide:
    scene s's local id = prim - tri_offsets[s]."""

    def __init__(self, ctx: Context, scenes):
        """scenes: list of (Mesh, Bvh8)."""
        self.ctx = ctx
        self.meshes = [m for m, _ in scenes]
        self.bvhs = [b for _, b in scenes]
        n = len(scenes)
        self._keep = [np.ascontiguousarray(b.nodes) for b in self.bvhs] + [np.ascontiguousarray(b.tris)
                                                                           for b in self.bvhs]
        self._keep += [np.ascontiguousarray(m.mats) for m in self.meshes]
        node_ptrs = (C.c_void_p * n)(*[b.nodes.ctypes.data for b in self.bvhs])
        tri_ptrs = (C.c_void_p * n)(*[b.tris.ctypes.data for b in self.bvhs])
        mat_ptrs = (C.c_void_p * n)(*[m.mats.ctypes.data for m in self.meshes])
        node_counts = np.array([len(b.nodes) for b in self.bvhs], np.uint32)
        tri_counts = np.array([len(b.tris) for b in self.bvhs], np.uint32)
        self.tri_offsets = np.concatenate([[0], np.cumsum(tri_counts)]).astype(np.uint64)
        h = C.c_void_p()
        ctx.check(lib().mrt_cuda_batch_create(ctx.handle, n, node_ptrs, ptr(node_counts), tri_ptrs, ptr(tri_counts),
                                              mat_ptrs, C.byref(h)), "batch_create")
        self._h = h

    @property
    def handle(self):
        return self._h

    def trace(self, rays, ray_offsets: np.ndarray, hits, any_hit: bool = False, stream=None):
        off = np.ascontiguousarray(ray_offsets, np.uint32)
        self.ctx.check(lib().mrt_cuda_batch_trace(self.ctx.handle, self._h, ptr(rays), ptr(off), ptr(hits),
                                                  int(any_hit), ptr(stream)), "batch_trace")

    def pathtrace(self, rays, ray_offsets: np.ndarray, params, frame: int, radiance, use_graph: bool = True,
                  stream=None):
        off = np.ascontiguousarray(ray_offsets, np.uint32)
        self.ctx.check(lib().mrt_cuda_batch_pathtrace(self.ctx.handle, self._h, ptr(rays), ptr(off),
                                                      C.byref(params), frame, ptr(radiance), int(use_graph),
                                                      ptr(stream)), "batch_pathtrace")

    def accumulate(self, acc, radiance, groups: int, copies: int, count: int, scale: float, stream=None):
        """acc[g][i] += scale * sum_c radiance[g][c][i] (mrt_cuda_accumulate_copies)."""
        accumulate_copies(self.ctx, acc, radiance, groups, copies, count, scale, stream)

    def close(self):
        if self._h and self.ctx.handle:
            lib().mrt_cuda_batch_destroy(self.ctx.handle, self._h)
        self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def pinhole_rays(lo, hi, width: int, height: int, seed: int = 0, fov_deg: float = 50.0) -> np.ndarray:
    """width x height camera rays looking at the centre of the box [lo, hi]
    from a seeded direction above it (RAY_DTYPE, tmin 0, tmax inf)."""
    from ._lib import RAY_DTYPE
    lo, hi = np.asarray(lo, np.float64), np.asarray(hi, np.float64)
    c = 0.5 * (lo + hi)
    r = 0.5 * np.linalg.norm(hi - lo) + 1e-3
    rng = np.random.default_rng(seed)
    az, el = rng.uniform(0, 2 * np.pi), np.radians(rng.uniform(20, 60))
    eye = c + 1.6 * r / np.tan(np.radians(fov_deg) / 2) * 0.6 * np.array(
        [np.cos(el) * np.cos(az), np.cos(el) * np.sin(az), np.sin(el)])
    fwd = c - eye
    fwd /= np.linalg.norm(fwd)
    right = np.cross(fwd, [0.0, 0.0, 1.0])
    right /= np.linalg.norm(right)
    up = np.cross(right, fwd)
    th = np.tan(np.radians(fov_deg) / 2)
    xs = ((np.arange(width) + 0.5) / width * 2 - 1) * th * width / height
    ys = (1 - (np.arange(height) + 0.5) / height * 2) * th
    d = fwd[None, None, :] + xs[None, :, None] * right[None, None, :] + ys[:, None, None] * up[None, None, :]
    d /= np.linalg.norm(d, axis=2, keepdims=True)
    rays = np.zeros(width * height, RAY_DTYPE)
    rays["org"] = eye.astype(np.float32)
    rays["dir"] = d.reshape(-1, 3).astype(np.float32)
    rays["tmin"] = 0.0
    rays["tmax"] = np.inf
    return rays


class DeviceScene:
    """A scene uploaded to one context (mrt_scene)."""

    def __init__(self, ctx: Context, handle: C.c_void_p, kind: str, mesh: Mesh | None = None,
                 bvh: Bvh8 | None = None, spheres: np.ndarray | None = None):
        self.ctx, self._h, self.kind = ctx, handle, kind
        self.mesh, self.bvh, self.spheres = mesh, bvh, spheres

    @property
    def handle(self):
        return self._h

    @classmethod
    def triangles(cls, ctx: Context, mesh: Mesh, bvh: Bvh8 | None = None) -> "DeviceScene":
        bvh = bvh or build_bvh8(mesh)
        h = C.c_void_p()
        ctx.check(lib().mrt_cuda_scene_upload_triangles(ctx.handle, ptr(bvh.nodes), len(bvh.nodes), ptr(bvh.tris),
                                                         len(bvh.tris), ptr(mesh.mats), len(mesh.mats), C.byref(h)),
                  "scene_upload_triangles")
        return cls(ctx, h, "triangles", mesh=mesh, bvh=bvh)

    @classmethod
    def from_spheres(cls, ctx: Context, spheres: np.ndarray) -> "DeviceScene":
        spheres = np.ascontiguousarray(spheres, dtype=SPHERE_DTYPE)
        h = C.c_void_p()
        ctx.check(lib().mrt_cuda_scene_upload_spheres(ctx.handle, ptr(spheres), len(spheres), C.byref(h)),
                  "scene_upload_spheres")
        return cls(ctx, h, "spheres", spheres=spheres)

    def close(self):
        if self._h and self.ctx.handle:
            lib().mrt_cuda_scene_destroy(self.ctx.handle, self._h)
        self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
