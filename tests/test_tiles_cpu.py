"""The mixed mode's tile plan (rocflu_gb300/csrc/tiles.h, host code): every
stencil member and face neighbour's 16-bit local id resolves to its cell,
halo lists hold each cell once, bank-aligned slots keep the low three bits
of the cell id and remove the stencil loop's bank conflicts on a
Morton-ordered box, and compact slots are taken when the aligned buffers
would cost occupancy.  tests/tiles_check.cpp is compiled with the host C++
compiler and run."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "rocflu_gb300", "csrc")


def test_tile_plan(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "tiles_check")
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", CSRC, os.path.join(HERE, "tiles_check.cpp"), "-o", exe],
                   check=True)
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip().endswith("ok")
