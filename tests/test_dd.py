"""Double-float arithmetic (mahakala_gb300/csrc/mk_dd.cuh) on the host:
add, sub, mul, div and rsqrt against long double over random operands.
Bar: 1e-13 relative (the pairs carry ~44-48 bits)."""

import os
import shutil
import subprocess

import pytest

from conftest import ROOT


def test_double_float_accuracy(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = tmp_path / "dd_check"
    subprocess.run([nvcc, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "mahakala_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "dd_check.cu"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    errs = [float(x) for x in out]
    names = ["add", "sub", "mul", "div", "rsqrt"]
    for n, e in zip(names, errs):
        assert e < 1e-13, f"{n}: {e:.3e}"
