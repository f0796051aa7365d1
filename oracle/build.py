"""Build recipe of the CPU oracle (test infrastructure): oracle/libfjsph_oracle.so.

g++ with -ffp-contract=off so that the only fused multiply-adds are the explicit std::fma calls
of the restated distance metric; OpenMP for the timed CPU baseline.
"""
from __future__ import annotations

import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "libfjsph_oracle.so"
SRC = HERE / "oracle.cpp"


def build(verbose: bool = False) -> Path:
    deps = [SRC, HERE / "oracle.h", HERE.parent / "include" / "fjsph_gb300.h"]
    if LIB.exists() and LIB.stat().st_mtime >= max(p.stat().st_mtime for p in deps):
        return LIB
    cxx = shutil.which("g++") or "c++"
    cmd = [cxx, "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", str(SRC), "-o", str(LIB)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stderr}")
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
