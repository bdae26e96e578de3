"""In-tree build of libmrt.so: the C++ host modules (g++) and the sm_103a
CUDA kernels + C ABI (nvcc), compiled in parallel, linked with nvcc.

    python -m minotert_gb300.build            # incremental
    python -m minotert_gb300.build --force    # rebuild everything
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libmrt.so"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
    f"-I{INCLUDE}", f"-I{CSRC / 'cuda'}", "--expt-relaxed-constexpr",
]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread", f"-I{INCLUDE}"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmrt.so")


def _sources():
    host = sorted((CSRC / "host").glob("*.cpp"))
    cuda = sorted((CSRC / "cuda").glob("*.cu"))
    return host, cuda


def _headers():
    return list(INCLUDE.glob("*.h")) + list((CSRC / "cuda").glob("*.cuh")) + list((CSRC / "cuda").glob("*.hpp"))


def _stale(obj: Path, src: Path, deps) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return src.stat().st_mtime > t or any(d.stat().st_mtime > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    host, cuda = _sources()
    deps = _headers()
    jobs = []
    objs = []
    for src in host:
        obj = BUILD / (src.stem + ".host.o")
        objs.append(obj)
        if force or _stale(obj, src, deps):
            jobs.append(["g++", *CXX_FLAGS, "-c", str(src), "-o", str(obj)])
    for src in cuda:
        obj = BUILD / (src.stem + ".cu.o")
        objs.append(obj)
        if force or ptxas_info or _stale(obj, src, deps):
            extra = ["-Xptxas", "-v"] if ptxas_info else []
            jobs.append([nvcc, *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for out in ex.map(_run, jobs):
                if verbose and out.strip():
                    print(out)
    if jobs or not LIB.exists():
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lpthread"])
    return LIB


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--ptxas-info", action="store_true", help="print register/spill/smem usage")
    a = ap.parse_args(argv)
    lib = build(force=a.force, verbose=True, ptxas_info=a.ptxas_info)
    print(lib)


if __name__ == "__main__":
    sys.exit(main())
