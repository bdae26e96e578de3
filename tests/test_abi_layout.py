"""The ctypes mirrors of the C ABI's structs (minotert_gb300/_lib.py) have
the C layout: a small C program compiled with gcc against include/*.h
prints each struct's size and every field's offset, and the mirrors must
agree (a field added on one side only -- the tuning struct grows with the
launch schedule's knobs -- fails here, without a GPU)."""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import pytest

from minotert_gb300 import _lib

ROOT = Path(__file__).resolve().parents[1]

PAIRS = {
    "mrt_camera_consts": _lib.CameraConsts, "mrt_gbuffer": _lib.GBuffer, "mrt_trace_params": _lib.TraceParams,
    "mrt_frame_stats": _lib.FrameStats, "mrt_tuning": _lib.Tuning, "mrt_cache_config": _lib.CacheConfig,
    "mrt_device_info": _lib.DeviceInfo, "mrt_camera": _lib.Camera_C, "mrt_mesh": _lib.Mesh_C,
    "mrt_bvh_build_params": _lib.BvhBuildParams, "mrt_bvh8": _lib.Bvh8_C,
    "mrt_bilateral_params": _lib.BilateralParams, "mrt_tonemap_params": _lib.TonemapParams,
    "mrt_reproject_params": _lib.ReprojectParams,
}


def test_ctypes_mirrors_match_the_headers(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "mrt_host.h"', "int main(void) {"]
    for cname, py in PAIRS.items():
        lines.append(f'    printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'    printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run([cc, "-std=c11", f"-I{ROOT / 'include'}", str(src), "-o", str(exe)], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr  # a field the mirror names but the header lacks fails to compile
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        name, field, value = line.split()
        got[(name, field)] = int(value)
    for cname, py in PAIRS.items():
        assert got[(cname, "size")] == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)
