"""Builds the CPU oracle (test infrastructure) into oracle/_build/liboracle.so.

The oracle is plain C++17 with no dependencies.  It is compiled with
-ffp-contract=off so every FMA is an explicit std::fma; on x86-64 hosts
whose CPU has FMA units -mfma makes those single instructions (the result
is the same either way: fma is correctly rounded).
"""
from __future__ import annotations

import platform
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build" / "liboracle.so"


def _has_fma() -> bool:
    if platform.machine() not in ("x86_64", "AMD64"):
        return False
    try:
        return " fma " in (" " + Path("/proc/cpuinfo").read_text().replace("\n", " ") + " ")
    except OSError:
        return False


def build(force: bool = False) -> Path:
    srcs = [HERE / "oracle.cpp", HERE / "post.cpp"]
    OUT.parent.mkdir(exist_ok=True)
    if not force and OUT.exists() and all(OUT.stat().st_mtime > s.stat().st_mtime for s in srcs):
        return OUT
    cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-math-errno", "-pthread"]
    if _has_fma():
        cmd.append("-mfma")
    cmd += [str(x) for x in srcs] + ["-o", str(OUT)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    return OUT


if __name__ == "__main__":
    print(build(force=True))
