"""Shared test fixtures.

Markers: ``gpu`` tests need a CUDA device (GB300) and call the C-ABI
library; everything else runs on the CPU.  The oracle (``oracle/``) is the
checker: a C restatement of the reference built here with gcc.
"""

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built sm_103a library")


def golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def tiny_arrays():
    """The tiny synthetic snapshot stored in tests/golden/snapshot.npz."""
    from mahakala_gb300.grmhd.synthetic import SnapshotArrays
    d = golden("snapshot")
    return SnapshotArrays(uov=d["uov"], B=d["B"], x1v=d["x1v"], x2v=d["x2v"], x3v=d["x3v"], x1f=d["x1f"],
                          x2f=d["x2f"], x3f=d["x3f"], LogicalLocations=d["LogicalLocations"],
                          Levels=d["Levels"], bhspin=0.9, fluid_gamma=13. / 9)


def amr_arrays(case):
    """Multi-level synthetic mesh `case` (0 or 1) stored in tests/golden/amr.npz."""
    from mahakala_gb300.grmhd.synthetic import SnapshotArrays
    d = golden("amr")
    p = f"case{case}_"
    return SnapshotArrays(uov=d[p + "uov"], B=d[p + "B"], x1v=d[p + "x1v"], x2v=d[p + "x2v"], x3v=d[p + "x3v"],
                          x1f=d[p + "x1f"], x2f=d[p + "x2f"], x3f=d[p + "x3f"],
                          LogicalLocations=d[p + "LogicalLocations"], Levels=d[p + "Levels"], bhspin=0.94,
                          fluid_gamma=13. / 9)


@pytest.fixture(scope="session")
def cuda():
    """Skip without a GPU; with one, build (if needed) and load the library."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mahakala_gb300 import _lib, build
    build.build()
    _lib.load()
    return torch.device("cuda", 0)


def rel_err(x, ref, floor=0.0):
    x = np.asarray(x, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    den = np.maximum(np.abs(ref), floor)
    with np.errstate(all="ignore"):
        e = np.abs(x - ref) / np.where(den > 0, den, 1.0)
    e = np.where((x == ref) | (np.isnan(x) & np.isnan(ref)), 0.0, e)
    return e
