"""The integer FP64 -> FP32 rounding used by the packing kernels (fjsph_gb300/csrc/split.cuh)
agrees bit for bit with the compiler's conversions: hi = fl32(x), lo = fl32(x - hi), over 16M
doubles of every exponent with ties, near-ties and exponent carries.  The same header is compiled
for the device, where the conversions it replaces run on the FP64 pipe."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_split_matches_conversions(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "split_check"
    subprocess.run([gxx, "-O2", "-o", str(exe), str(ROOT / "tests" / "native" / "split_check.cpp")], check=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "0 mismatches" in res.stdout
