"""Double-float arithmetic (mahakala_gb300/csrc/mk_dd.cuh) on the host:
add, sub, mul, div and rsqrt against long double over random operands
(bar: 1e-13 relative, the pairs carry ~44-48 bits), and the null
renormalisation and camera rays built on it (renull_k0_dd and
camera_ray_pair in mk_kerr.cuh)."""

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


def test_double_float_null_renormalisation(tmp_path):
    """renull_k0_dd (mk_kerr.cuh), the near-hole phase's renormalisation at
    radial turning points, against the quadratic's nearer root in long
    double: 1e-11 relative away from the surface g00 = 0, 1e-9 within
    |g00| < 1e-2 (the nearer root there loses digits in any precision)."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = tmp_path / "renull_check"
    subprocess.run([nvcc, "-O2", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I", os.path.join(ROOT, "mahakala_gb300", "csrc"), "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "renull_check.cu"), "-o", str(exe)], check=True)
    worst, worst_g00, near = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    assert int(near) > 100
    assert float(worst) < 1e-11, worst
    assert float(worst_g00) < 1e-9, worst_g00


def test_double_float_camera_rays(tmp_path):
    """camera_ray_pair (mk_kerr.cuh), the mixed forms' camera rays in
    double-float, against the reference's construction in long double over
    4 spins x 7 inclinations (0-180 deg) x 3 fields of view x 3 distances x
    2 grid sizes: positions within 1e-13 and wavevectors within 1e-11 of
    their norms, and NaN exactly where the reference has no direction (the
    centre of an odd grid)."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = tmp_path / "camera_pair_check"
    subprocess.run([nvcc, "-O2", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I", os.path.join(ROOT, "mahakala_gb300", "csrc"), "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "camera_pair_check.cu"), "-o", str(exe)], check=True)
    worst_x, worst_k, rays, nan_ok = subprocess.run([str(exe)], check=True, capture_output=True,
                                                    text=True).stdout.split()
    assert int(rays) > 700000
    assert float(worst_x) < 1e-13, worst_x
    assert float(worst_k) < 1e-11, worst_k
    assert nan_ok == "1"
