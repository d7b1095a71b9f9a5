"""The C-ABI library loads without a GPU and exports every symbol the public
header declares, with the struct layouts the Python binding assumes."""

import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "mahakala_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*(mk_[a-z0-9_]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from mahakala_gb300 import _lib, build
    build.build()
    return _lib.load()


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("mk_render", "mk_integrate", "mk_camera_init", "mk_fluid_scalars", "mk_synchrotron",
              "mk_solve_intensity", "mk_snapshot_build", "mk_shadow_pass"):
        assert n in names


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header(lib):
    from mahakala_gb300 import _lib
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_struct_layouts(lib):
    from mahakala_gb300 import _lib
    for name, cls in (("mk_step_policy", _lib.StepPolicy), ("mk_camera", _lib.Camera),
                      ("mk_snapshot_view", _lib.SnapshotView), ("mk_request", _lib.Request)):
        assert lib.mk_sizeof(name.encode()) == ctypes.sizeof(cls)


def test_version_and_workspace(lib):
    assert lib.mk_abi_version() == 1
    assert b"sm_103a" in lib.mk_version()
    assert lib.mk_render_workspace_bytes(100, 0) == 256
    assert lib.mk_render_workspace_bytes(100, 1) > 256 + 2 * 100 * 100
    assert lib.mk_snapshot_bytes(8, 8) == 8 * 10 ** 3 * 32 + 8 * 32


def test_argument_errors_without_gpu(lib):
    """Argument validation happens before any CUDA call."""
    from mahakala_gb300 import _lib
    with pytest.raises(_lib.MKError) as e:
        _lib.call("mk_render", None, 1, 10, None, 1, 0, None, 256, None)
    assert e.value.code == _lib.MK_ERR_ARG
    assert b"null" in lib.mk_last_error()
    with pytest.raises(_lib.MKError):
        _lib.call("mk_camera_init", None, None, None)
