"""The C-ABI library loads without a GPU and exports every symbol the public
header declares, with the struct layouts the Python binding assumes; a C
program includes the header and links the library."""

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
                      ("mk_snapshot_view", _lib.SnapshotView), ("mk_mesh_desc", _lib.MeshDesc),
                      ("mk_request", _lib.Request)):
        assert lib.mk_sizeof(name.encode()) == ctypes.sizeof(cls)


def test_version_and_workspace(lib):
    assert lib.mk_abi_version() == 1
    assert b"sm_103a" in lib.mk_version()
    assert lib.mk_render_workspace_bytes(100, 0) == 256
    assert lib.mk_snapshot_bytes(8, 8) == 8 * 10 ** 3 * 32 + 8 * 32
    # mixed forms: two queues of 160-byte records, plus 64 bytes a ray of
    # camera states once the launch exceeds one wave of 4 blocks x 128
    # threads per SM (the SM count the library reports; 1 without a GPU)
    from mahakala_gb300 import _lib
    wave = lib.mk_device_sm_count() * 4 * 128
    for n in (100, wave, wave + 1, 4 * wave):
        for prec in (_lib.MK_MIXED, _lib.MK_MIXED_STRICT, _lib.MK_MIXED_DF):
            assert lib.mk_render_workspace_bytes(n, prec) == 256 + 320 * n + (64 * n if n > wave else 0)
        assert lib.mk_render_workspace_bytes(n, _lib.MK_FP64) == 256


def test_argument_errors_without_gpu(lib):
    """Argument validation happens before any CUDA call."""
    from mahakala_gb300 import _lib
    with pytest.raises(_lib.MKError) as e:
        _lib.call("mk_render", None, 1, 10, None, 1, 0, None, 256, None)
    assert e.value.code == _lib.MK_ERR_ARG
    assert b"null" in lib.mk_last_error()
    with pytest.raises(_lib.MKError):
        _lib.call("mk_camera_init", None, None, None)


def test_tuning_switches_validate_without_gpu(lib):
    """The measurement switches accept their documented values and refuse
    others (no GPU call is made)."""
    from mahakala_gb300 import _lib
    for name, good, bad in ((b"fp64_rays_per_warp", (1, 32), (3, 64)), (b"fp64_zone", (0, 1), (2,)),
                            (b"phase_events", (1, 0), (5,)), (b"f32_blocks_per_sm", (0, 3, 4, 5), (2, 6)),
                            (b"zone_wait_test", (1, 0), (2,)), (b"zone_wait_ns", (5, 1_000_000_000), (0,))):
        for v in good:
            _lib.call("mk_set_tuning", name, v)
        for v in bad:
            with pytest.raises(_lib.MKError) as e:
                _lib.call("mk_set_tuning", name, v)
            assert e.value.code == _lib.MK_ERR_ARG
    _lib.call("mk_set_tuning", b"fp64_rays_per_warp", 32)
    _lib.call("mk_set_tuning", b"fp64_zone", 1)
    _lib.call("mk_set_tuning", b"phase_events", 0)
    _lib.call("mk_set_tuning", b"f32_blocks_per_sm", 0)
    _lib.call("mk_set_tuning", b"zone_wait_test", 0)
    _lib.call("mk_set_tuning", b"zone_wait_ns", 1_000_000_000)
    with pytest.raises(_lib.MKError):
        _lib.call("mk_set_tuning", b"no_such_knob", 1)


def test_mixed_request_limit_without_gpu(lib):
    """A mixed-form launch refuses more requests than its shared-memory
    request table holds, before touching the device."""
    import ctypes as c
    from mahakala_gb300 import _lib
    n = _lib.MK_MAX_REQUESTS_MIXED + 1
    ws = (c.c_uint8 * 16)()
    with pytest.raises(_lib.MKError) as e:
        _lib.call("mk_render", c.addressof(ws), n, 10, c.addressof(ws), 1, _lib.MK_MIXED, c.addressof(ws),
                  lib.mk_render_workspace_bytes(10, _lib.MK_MIXED), None)
    assert e.value.code == _lib.MK_ERR_LIMIT


def test_c_host_compiles_links_and_calls(lib, tmp_path):
    """The header as C11 (-pedantic -Werror) in a C program linked against
    the library: struct layouts as a C compiler lays them out equal the
    library's, and the GPU-free entry points answer (tests/abi_c_check.c)."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not available")
    build_dir = os.path.join(ROOT, "mahakala_gb300", "_build")
    exe = tmp_path / "abi_c_check"
    subprocess.run([gcc, "-std=c11", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "abi_c_check.c"), "-L", build_dir, "-lmahakala_gb300",
                    f"-Wl,-rpath,{build_dir}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout + out.stderr
