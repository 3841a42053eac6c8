"""The device-buffer argument rules of rflu_gpu_residual_static
(rocflu_gb300/csrc/args.h, host code): a buffer on another GPU than the
context's, host memory, and a call made while another device is current are
refused before anything is launched; device memory on the context's GPU and
managed memory are accepted.  tests/args_check.cpp is compiled with the host
C++ compiler and run (a one-GPU machine cannot place a buffer on a second GPU)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "rocflu_gb300", "csrc")


def test_device_argument_rules(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "args_check")
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", CSRC, os.path.join(HERE, "args_check.cpp"), "-o", exe],
                   check=True)
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip().endswith("ok")
