"""The mixed update's float<->double conversions (rocflu_gb300/csrc/
convert.cuh, integer instructions) against the host's C casts: every float
through f2d, and d2f on every double exponent with rounding-boundary
mantissas and on random bit patterns.  tests/convert_check.cpp is compiled
with the host C++ compiler and run (about 15 s); the device comparison with
the hardware conversions is tests/test_gpu_parity.py's."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "rocflu_gb300", "csrc")


def test_conversions_match_c_casts(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "convert_check")
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", CSRC, os.path.join(HERE, "convert_check.cpp"), "-o", exe],
                   check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip().endswith("ok")
