"""ctypes binding of ``libmahakala_gb300.so`` (include/mahakala_gb300.h).

The library is the product: every compute call goes through it.  There is
no CPU fallback; a missing library or a missing GPU raises immediately.
"""

import ctypes
import os

import numpy as np

from . import build as _build

_c = ctypes
_VP = _c.c_void_p
_I32 = _c.c_int32
_I64 = _c.c_int64
_D = _c.c_double
_SZ = _c.c_size_t

MK_OK, MK_ERR_ARG, MK_ERR_CUDA, MK_ERR_LIMIT, MK_ERR_UNSUPPORTED, MK_ERR_TIMEOUT = 0, 1, 2, 3, 4, 5
MK_RAY_ACTIVE, MK_RAY_CAPTURED, MK_RAY_ESCAPED, MK_RAY_MAXSTEPS, MK_RAY_NAN = 0, 1, 2, 3, 4
MK_FP64, MK_MIXED, MK_MIXED_DF, MK_MIXED_STRICT = 0, 1, 2, 3
MK_POLICY_REFERENCE, MK_POLICY_FIXED = 0, 1
MK_CAMERA_GRID, MK_CAMERA_EQUATOR = 0, 1
MK_MAX_NU = 4
MK_PROBE_FFMA2 = 100
MK_MATH_RSQRT, MK_MATH_RCP, MK_MATH_SQRT, MK_MATH_LIB_RSQRT, MK_MATH_LIB_RCP, MK_MATH_LIB_SQRT = range(6)
NOALLOC_WORKSPACE_BYTES = 16 << 20
NOALLOC_MAX_MIXED_RAYS = (NOALLOC_WORKSPACE_BYTES - 256) // 320
MK_WS_STEPS, MK_WS_SAMPLES, MK_WS_MAX_TAU, MK_WS_TO_FP64, MK_WS_FP32_QUEUE, MK_WS_STEPS_FP64 = 1, 2, 3, 4, 6, 8
MK_WS_TO_FP32 = 14
MK_WS_SAMPLES_FP64 = 10
MK_WS_ZONE_RUN_MAX = 11
MK_WS_STEPS_B, MK_WS_SAMPLES_B = 12, 13
MK_WS_STEPS_C, MK_WS_SAMPLES_C = 15, 16
MK_WS_ERROR = 17
MK_MAX_REQUESTS_MIXED = 128


class MKError(RuntimeError):
    """A C-ABI call returned a non-zero mk_status."""

    def __init__(self, code, msg):
        super().__init__(f"[mk_status {code}] {msg}")
        self.code = code


class StepPolicy(_c.Structure):
    _fields_ = [("kind", _I32), ("nmax", _I32), ("div", _D), ("tol", _D), ("hfrac", _D), ("hmin", _D),
                ("hmax", _D), ("capture", _D), ("r_escape", _D)]


class Camera(_c.Structure):
    _fields_ = [("kind", _I32), ("pixels", _I32), ("bhspin", _D), ("cos_inc", _D), ("sin_inc", _D),
                ("distance", _D), ("fov_lower", _D), ("fov_upper", _D)]


class SnapshotView(_c.Structure):
    _fields_ = [("blocks", _VP), ("geom", _VP), ("geom_f32", _VP), ("faces", _VP), ("table", _VP),
                ("blocks64", _VP), ("block64", _VP), ("nmb", _I32), ("n", _I32),
                ("nb", _I32 * 3), ("pad0", _I32), ("lo", _D * 3), ("width", _D * 3)]


class MeshDesc(_c.Structure):
    _fields_ = [("uov", _VP), ("B", _VP), ("locs", _VP), ("levels", _VP), ("keys", _VP), ("key_block", _VP),
                ("geom", _VP), ("faces", _VP), ("table", _VP), ("blocks64", _VP), ("block64", _VP),
                ("nmb", _I32), ("n", _I32), ("n64", _I32), ("pad0", _I32), ("nb", _I32 * 3), ("pad1", _I32),
                ("lo", _D * 3), ("width", _D * 3)]


def mesh_key(level, i, j, k):
    """MK_MESH_KEY of include/mahakala_gb300.h (NumPy arrays or ints)."""
    return (np.int64(level) << 54) | (np.int64(i) << 36) | (np.int64(j) << 18) | np.int64(k)


class Request(_c.Structure):
    _fields_ = [("camera", Camera), ("policy", StepPolicy), ("fluid_gamma", _D), ("r_low", _D), ("r_high", _D),
                ("electron_gamma_m1", _D), ("ion_gamma_m1", _D), ("Ne_unit", _D), ("B_unit", _D),
                ("L_unit", _D), ("cos_fallback_pitch", _D), ("sigma_cut", _D), ("nnu", _I32),
                ("snapshot", _I32), ("nu", _D * MK_MAX_NU), ("image", _VP), ("nsteps", _VP), ("status", _VP),
                ("ray_offset", _I64), ("rows_em", _VP), ("rows_ab", _VP), ("rows_dt", _VP), ("rows", _I64)]


class Job(_c.Structure):
    _fields_ = [("nreq", _I32), ("nsnap", _I32), ("total_rays", _I64)]


# name -> (restype, argtypes); the declarations of include/mahakala_gb300.h
SIGNATURES = {
    "mk_version": (_c.c_char_p, []),
    "mk_abi_version": (_I32, []),
    "mk_last_error": (_c.c_char_p, []),
    "mk_device_sm_count": (_I32, []),
    "mk_camera_init": (_c.c_int, [_c.POINTER(Camera), _VP, _VP]),
    "mk_camera_points": (_c.c_int, [_VP, _VP, _I64, _D, _D, _D, _D, _VP, _VP]),
    "mk_integrate": (_c.c_int, [_VP, _I64, _D, _c.POINTER(StepPolicy), _VP, _VP, _VP, _VP, _VP, _VP]),
    "mk_radius_cal": (_c.c_int, [_VP, _I64, _I64, _D, _VP, _VP]),
    "mk_shadow_pass": (_c.c_int, [_VP, _VP, _VP, _I64, _D, _D, _D, _D, _I32, _VP, _VP, _VP, _VP, _VP, _VP,
                                  _VP]),
    "mk_snapshot_bytes": (_SZ, [_I32, _I32]),
    "mk_snapshot_build": (_c.c_int, [_c.POINTER(MeshDesc), _VP, _SZ, _c.POINTER(SnapshotView), _VP]),
    "mk_fluid_scalars": (_c.c_int, [_c.POINTER(SnapshotView), _D, _VP, _I64, _D, _VP, _VP]),
    "mk_fluid_prims": (_c.c_int, [_c.POINTER(SnapshotView), _VP, _I64, _VP, _VP, _VP]),
    "mk_rlow_rhigh": (_c.c_int, [_VP, _VP, _VP, _I64, _D, _D, _D, _D, _VP, _VP]),
    "mk_synchrotron": (_c.c_int, [_VP, _VP, _VP, _VP, _VP, _I64, _I32, _D, _VP, _VP, _VP]),
    "mk_solve_intensity": (_c.c_int, [_VP, _VP, _VP, _I64, _I64, _D, _VP, _VP, _VP]),
    "mk_attenuated_emissivity": (_c.c_int, [_VP, _VP, _VP, _I64, _I64, _D, _VP, _VP]),
    "mk_render_workspace_bytes": (_SZ, [_I64, _I32]),
    "mk_render": (_c.c_int, [_VP, _I32, _I64, _VP, _I32, _I32, _VP, _SZ, _VP]),
    "mk_render_noalloc": (_c.c_int, [_VP, _I32, _I64, _VP, _I32, _I32, _VP]),
    "mk_render_job": (_c.c_int, [_VP, _VP, _VP, _I32, _I64, _VP, _SZ, _VP]),
    "mk_sizeof": (_SZ, [_c.c_char_p]),
    "mk_probe_fma": (_c.c_int, [_I32, _I32, _I32, _I64, _VP, _VP]),
    "mk_probe_math": (_c.c_int, [_I32, _VP, _I64, _VP, _VP]),
    "mk_set_tuning": (_c.c_int, [_c.c_char_p, _I64]),
    "mk_render_phase_ms": (_c.c_int, [_VP, _VP]),
}

_LIB = None


def library_path():
    return _build.LIB


def load():
    """Load the library (no GPU needed to load it) and declare signatures."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not os.path.exists(path):
        raise RuntimeError(
            f"mahakala_gb300: the CUDA library {path} is not built; run "
            "`python -c 'import __graft_entry__ as g; g.build()'` (there is no CPU fallback)")
    lib = _c.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    for name, cls in (("mk_step_policy", StepPolicy), ("mk_camera", Camera),
                      ("mk_snapshot_view", SnapshotView), ("mk_mesh_desc", MeshDesc), ("mk_request", Request)):
        n = lib.mk_sizeof(name.encode())
        if n != _c.sizeof(cls):
            raise RuntimeError(f"ABI mismatch: sizeof({name}) C={n} ctypes={_c.sizeof(cls)}")
    _LIB = lib
    return lib


def check(code):
    if code != MK_OK:
        raise MKError(code, load().mk_last_error().decode(errors="replace"))
    return code


def call(name, *args):
    return check(getattr(load(), name)(*args))
