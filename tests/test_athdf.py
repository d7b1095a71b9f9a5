"""The h5py-free .athdf reader and writer (mahakala_gb300/grmhd/hdf5.py).

* The reader against an HDF5 file written by the HDF5 library itself:
  scipy's MATLAB 7.3 test file (a 512-byte user block, superblock 0,
  symbol-table root group, one float64 dataset with a string attribute),
  whose contents scipy's own tests state (pi/4 * arange(9)).  Skipped
  where scipy's test data is not installed.
* write_athdf -> load_athdf round trips of the tiny golden snapshot and of
  a multi-level mesh, contiguous and chunked per meshblock with deflate:
  every dataset and VariableNames bit-identical.
* The path-based call of the reference (AthenakFluidModel(path)) builds
  the same oracle snapshot as the arrays.
* Not HDF5 and unsupported parts are refused with HDF5Error.
"""

import os

import numpy as np
import pytest

from conftest import amr_arrays

MAT = None
try:
    import scipy.io.matlab as _m
    MAT = os.path.join(os.path.dirname(_m.__file__), "tests", "data", "testhdf5_7.4_GLNX86.mat")
except ImportError:  # pragma: no cover
    pass

FIELDS = ("x1v", "x2v", "x3v", "x1f", "x2f", "x3f", "uov", "B", "LogicalLocations", "Levels")


@pytest.mark.skipif(not (MAT and os.path.exists(MAT)), reason="scipy's MATLAB test data is not installed")
def test_reader_on_a_file_written_by_the_hdf5_library():
    from mahakala_gb300.grmhd.hdf5 import File
    f = File(MAT)
    assert f.keys() == ["testdouble"]
    a = f["testdouble"]
    assert a.dtype == np.float64 and a.shape == (9, 1)
    assert np.array_equal(a.ravel(), np.pi / 4 * np.arange(9, dtype=float))
    assert bytes(f.dataset_attrs("testdouble")["MATLAB_class"]) == b"double"


def _same(a, b):
    for k in FIELDS:
        x, y = np.asarray(getattr(a, k)), np.asarray(getattr(b, k))
        assert x.shape == y.shape and np.array_equal(x, y), k
    assert tuple(a.VariableNames) == tuple(b.VariableNames)


@pytest.mark.parametrize("chunked", [False, True])
def test_roundtrip_tiny_snapshot(tmp_path, tiny_arrays, chunked):
    from mahakala_gb300.grmhd.athenak import load_athdf
    from mahakala_gb300.grmhd.hdf5 import File, write_athdf
    path = str(tmp_path / "tiny.athdf")
    write_athdf(path, tiny_arrays, chunk_blocks=chunked, deflate=chunked)
    got = load_athdf(path)
    _same(got, tiny_arrays)
    assert got.uov.dtype == np.float32 and got.Levels.dtype == np.asarray(tiny_arrays.Levels).dtype
    assert sorted(File(path).keys()) == sorted(FIELDS)


@pytest.mark.parametrize("case", [0, 1])
def test_roundtrip_multilevel_mesh(tmp_path, case):
    from mahakala_gb300.grmhd.athenak import load_athdf
    from mahakala_gb300.grmhd.hdf5 import write_athdf
    arrs = amr_arrays(case)
    path = str(tmp_path / f"amr{case}.athdf")
    write_athdf(path, arrs, chunk_blocks=arrs.uov.shape[1] <= 64, deflate=True)
    _same(load_athdf(path), arrs)


def test_path_call_builds_the_same_oracle_snapshot(tmp_path, orc, tiny_arrays):
    from mahakala_gb300.grmhd.athenak import load_athdf
    from mahakala_gb300.grmhd.hdf5 import write_athdf
    path = str(tmp_path / "tiny.athdf")
    write_athdf(path, tiny_arrays)
    arrs = load_athdf(path)
    a, b = orc.OracleSnapshot(tiny_arrays), orc.OracleSnapshot(arrs, bhspin=tiny_arrays.bhspin,
                                                                fluid_gamma=tiny_arrays.fluid_gamma)
    assert np.array_equal(a.all_meshblocks, b.all_meshblocks)


def test_not_hdf5_and_unsupported_parts_are_refused(tmp_path, tiny_arrays):
    from mahakala_gb300.grmhd.hdf5 import File, HDF5Error, write_athdf
    junk = tmp_path / "junk.athdf"
    junk.write_bytes(b"not an hdf5 file" * 64)
    with pytest.raises(HDF5Error):
        File(str(junk))
    path = tmp_path / "tiny.athdf"
    write_athdf(str(path), tiny_arrays)
    raw = bytearray(path.read_bytes())
    raw[8] = 7  # superblock version 7 does not exist
    bad = tmp_path / "bad.athdf"
    bad.write_bytes(bytes(raw))
    with pytest.raises(HDF5Error):
        File(str(bad))


def test_malformed_files_fail_with_an_error(tmp_path, tiny_arrays):
    """Truncated files and self-referencing structures raise HDF5Error; the
    reader never loops or returns short data."""
    from mahakala_gb300.grmhd.hdf5 import File, HDF5Error, write_athdf
    path = tmp_path / "tiny.athdf"
    write_athdf(str(path), tiny_arrays)
    raw = path.read_bytes()
    for cut in (40, 200, len(raw) // 2, len(raw) - 100):
        bad = tmp_path / f"cut{cut}.athdf"
        bad.write_bytes(raw[:cut])
        with pytest.raises(HDF5Error):
            f = File(str(bad))
            for k in f.keys():
                f[k]
