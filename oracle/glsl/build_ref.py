"""Build recipe: the reference's own compute shaders, compiled for the host.

Test infrastructure and the CPU baseline of the reference's own code only.
Reads the shader sources where they lie in the reference tree (src/gpu/ of
MinoteRT), rewrites each into C++ against glsl.hpp (translate.py), appends
the entry-point shim from this folder and compiles everything with g++ into
oracle/_ref/libglsl_ref.so.  Outputs go to oracle/_ref/ only (git-ignored,
carried to the GPU host with the rest of the tree, where the translation is
compiled again for its CPU).  Nothing here is copied into the repository:
with neither the reference tree nor a translation `build()` returns None
and the tests fall back to the committed vectors in tests/golden/.

Compiler settings that make the C++ evaluate the GLSL as written:
-ffp-contract=off (no fused multiply-add), -fsingle-precision-constant
(floating literals are binary32, as in GLSL) and
-ftrivial-auto-var-init=zero (the shaders read some locals they never
assign, e.g. Intersection.t of a primary ray that misses; GLSL leaves those
undefined, here they read 0).
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

from . import translate

HERE = Path(__file__).resolve().parent
OUT = HERE.parent / "_ref"
REF_GPU = Path(os.environ.get("MRT_REFERENCE", "/root/reference")) / "src" / "gpu"

# (translation unit, shader source relative to src/gpu, shim, defines before
# the header, defines before the shim, specialisation constants).  The LUT
# sizes are the ones the reference's sky module creates its images with
# (src/gfx/modules/sky.ixx): transmittance 256 x 64, multiple scattering
# 32 x 32, sky view 192 x 108.
_CW = "#define GLSL_EXP_CW\n"
UNITS = [
    ("funcs", None, "shim_funcs.inc", "", "", {}),
    ("primary", "primaryRay.comp", "shim_primary.inc", "", "", {}),
    ("secondary", "secondaryRays.comp", "shim_secondary.inc", "", "", {}),
    ("sky_transmittance", "sky/genTransmittance.comp", "shim_sky.inc", _CW, "#define REF_SKY_TRANSMITTANCE\n",
     {"TransmittanceSizeWidth": 256, "TransmittanceSizeHeight": 64}),
    ("sky_multiscatter", "sky/genMultiScattering.comp", "shim_sky.inc", _CW, "#define REF_SKY_MULTISCATTER\n",
     {"MultiScatteringWidth": 32, "MultiScatteringHeight": 32}),
    ("sky_view", "sky/genView.comp", "shim_sky.inc", _CW, "#define REF_SKY_VIEW\n",
     {"ViewSizeWidth": 192, "ViewSizeHeight": 108}),
    ("bilateral", "denoise/bilateral.comp", "shim_bilateral.inc", _CW, "", {}),
] + [(f"tonemap_{n}", f"tonemap/{n}.comp", "shim_tonemap.inc", "", f"#define REF_TONEMAP_ENTRY ref_tonemap_{n}\n", {})
     for n in ("linear", "reinhard", "hable", "aces", "uchimura", "amd")]

_PROLOGUE = """// generated by oracle/glsl/build_ref.py from {src}; do not edit
{pre}#include <cstring>
#include "glsl.hpp"
namespace {{
using namespace glsl;
using glsl::uint;
{usings}
"""
_BUILTINS = ("abs sign floor ceil round fract mod min max clamp mix step smoothstep sqrt inversesqrt pow exp exp2 "
             "log log2 sin cos tan asin acos atan dot cross length distance normalize reflect greaterThanEqual "
             "greaterThan lessThan any all imageSize imageStore textureSize texelFetch textureLod texture "
             "barrier").split()
_FLAGS = ["-std=gnu++20", "-O1", "-fPIC", "-pthread", "-ffp-contract=off", "-fsingle-precision-constant",
          "-ftrivial-auto-var-init=zero", "-w", f"-I{HERE}"]


def available() -> bool:
    return (REF_GPU / "primaryRay.comp").is_file()


def _unit_source(name: str, rel: str | None, shim: str, pre: str, defines: str, spec: dict) -> str:
    if rel is None:  # the pure helper files, through a stub that includes them
        stub = OUT / "glsl" / "funcs.glsl"
        stub.write_text(f'#include "{REF_GPU / "random.glsl"}"\n#include "{REF_GPU / "intersect.glsl"}"\n')
        body, src = translate.translate(stub), "random.glsl, intersect.glsl, util.glsl"
    else:
        body, src = translate.translate(REF_GPU / rel, spec), rel
    usings = "\n".join(f"using glsl::{b};" for b in _BUILTINS)
    return (_PROLOGUE.format(src=src, pre=pre, usings=usings) + body + "\n} // namespace\n" + defines +
            (HERE / shim).read_text())


def build(force: bool = False) -> Path | None:
    """Compile the shaders; returns the library path, or None when neither the
    reference tree nor an earlier translation (oracle/_ref/glsl/*.cpp, which
    travels with the rest of oracle/_ref) is there."""
    (OUT / "glsl").mkdir(parents=True, exist_ok=True)
    if available():
        srcs = {u[0]: _unit_source(*u) for u in UNITS}
    else:
        files = {u[0]: OUT / "glsl" / f"{u[0]}.cpp" for u in UNITS}
        if not all(f.is_file() for f in files.values()):
            return None
        srcs = {n: f.read_text() for n, f in files.items()}
    key = hashlib.sha256(("".join(srcs[n] for n in sorted(srcs)) + (HERE / "glsl.hpp").read_text() +
                          " ".join(_FLAGS)).encode()).hexdigest()[:16]
    lib = OUT / "libglsl_ref.so"
    stamp = OUT / "libglsl_ref.key"
    if not force and lib.exists() and stamp.exists() and stamp.read_text() == key:
        return lib

    def compile_one(name):
        cpp = OUT / "glsl" / f"{name}.cpp"
        cpp.write_text(srcs[name])
        obj = OUT / "glsl" / f"{name}.o"
        r = subprocess.run(["g++", *_FLAGS, "-c", str(cpp), "-o", str(obj)], capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"compiling {name}:\n{r.stderr[-4000:]}")
        return obj

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(compile_one, list(srcs)))
    r = subprocess.run(["g++", "-shared", "-pthread", "-o", str(lib), *map(str, objs)], capture_output=True,
                       text=True)
    if r.returncode:
        raise RuntimeError(r.stderr[-4000:])
    stamp.write_text(key)
    return lib


_lib = None


def lib() -> C.CDLL | None:
    """The compiled reference shaders (None without the reference tree)."""
    global _lib
    if _lib is None:
        path = build()
        if path is None:
            return None
        L = C.CDLL(str(path))
        f, u, i, vp = C.c_float, C.c_uint32, C.c_int, C.c_void_p
        fp, up = C.POINTER(f), C.POINTER(u)
        L.ref_pcg.argtypes, L.ref_pcg.restype = [up], u
        L.ref_random_float.argtypes, L.ref_random_float.restype = [up], f
        L.ref_random_sphere_point.argtypes = [f, f, fp]
        L.ref_ray_at.argtypes = [fp, fp, f, fp]
        L.ref_ray_sphere.argtypes, L.ref_ray_sphere.restype = [fp, fp, fp, f], f
        L.ref_srgb_encode.argtypes = [fp, fp]
        L.ref_reversible_tonemap.argtypes = [fp, fp, i]
        L.ref_primary_rays.argtypes, L.ref_primary_rays.restype = [vp, i, i, vp, vp, vp, vp], i
        L.ref_secondary_rays.argtypes = [vp, i, i, vp, vp, vp, vp, i, i, vp, i, i, vp, i, i, vp, vp]
        L.ref_secondary_rays.restype = i
        L.ref_dispatch_threads.argtypes, L.ref_dispatch_threads.restype = [i], i
        L.ref_secondary_rays_rows.argtypes = [vp, i, i, vp, vp, vp, vp, i, i, vp, i, i, vp, i, i, vp, vp, i, i]
        L.ref_secondary_rays_rows.restype = i
        L.ref_sky_transmittance.argtypes, L.ref_sky_transmittance.restype = [vp, vp], i
        L.ref_sky_multiscatter.argtypes, L.ref_sky_multiscatter.restype = [vp, vp, vp], i
        L.ref_sky_view.argtypes, L.ref_sky_view.restype = [vp, vp, vp, vp, vp, vp, vp], i
        L.ref_bilateral.argtypes, L.ref_bilateral.restype = [vp, vp, vp, i, i, vp, vp], i
        for n in ("linear", "reinhard", "hable", "aces", "uchimura", "amd"):
            fn = getattr(L, f"ref_tonemap_{n}")
            fn.argtypes, fn.restype = [vp, i, i, vp, i, vp], i
        _lib = L
    return _lib
