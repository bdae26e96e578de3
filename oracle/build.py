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
    src = HERE / "oracle.cpp"
    OUT.parent.mkdir(exist_ok=True)
    if not force and OUT.exists() and OUT.stat().st_mtime > src.stat().st_mtime:
        return OUT
    cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-math-errno", "-pthread"]
    if _has_fma():
        cmd.append("-mfma")
    cmd += [str(src), "-o", str(OUT)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    return OUT


if __name__ == "__main__":
    print(build(force=True))
