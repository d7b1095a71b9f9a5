"""Camera and geodesic entry points with the reference's call surface.

Mirrors ``mahakala/geodesics.py``: same names, positional order and
defaults.  Arrays come back as float64 CUDA tensors (the reference returns
jax device arrays); the compute runs in the sm_103a kernels of
``libmahakala_gb300.so``.
"""

import numpy as np
import torch

from . import _lib
from ._device import device, f64, ptr, stream_ptr

__all__ = ["initialize_geodesics_at_camera", "geodesic_integrator", "radius_cal", "radius_EH",
           "find_shadow_bisection", "find_shadow_bisection_angles", "select_photons_integrator",
           "trace", "make_camera", "step_policy"]


def radius_EH(a_spin):
    """Outer horizon radius (geodesics.py:350-351)."""
    return 1 + np.sqrt(1 - a_spin ** 2)


def _cos_sin(inclination):
    i = inclination * np.pi / 180  # geodesics.py:205
    return float(np.cos(i)), float(np.sin(i))


def make_camera(bhspin, inclination, distance, fov_lower, fov_upper, pixels_per_side, camera_type="grid"):
    kind = camera_type.lower()
    if kind not in ("grid", "equator"):
        raise ValueError(f'Unexpected camera type "{camera_type}". Please choose either "grid" or "equator"')
    ci, si = _cos_sin(inclination)
    cam = _lib.Camera()
    cam.kind = _lib.MK_CAMERA_GRID if kind == "grid" else _lib.MK_CAMERA_EQUATOR
    cam.pixels = int(pixels_per_side)
    cam.bhspin, cam.cos_inc, cam.sin_inc = float(bhspin), ci, si
    cam.distance, cam.fov_lower, cam.fov_upper = float(distance), float(fov_lower), float(fov_upper)
    return cam


def camera_pixels(cam):
    return cam.pixels * cam.pixels if cam.kind == _lib.MK_CAMERA_GRID else cam.pixels


def initialize_geodesics_at_camera(bhspin, inclination, distance, fov_lower, fov_upper, pixels_per_side,
                                   camera_type="grid"):
    """geodesics.py:29-55 -> (npx, 8) float64 CUDA tensor, pixel ix*n + iy."""
    cam = make_camera(bhspin, inclination, distance, fov_lower, fov_upper, pixels_per_side, camera_type)
    if cam.pixels <= 0:
        raise ValueError("pixels_per_side must be positive")
    s0 = torch.empty((camera_pixels(cam), 8), dtype=torch.float64, device=device())
    _lib.call("mk_camera_init", _lib.ctypes.byref(cam), ptr(s0), stream_ptr())
    return s0


def step_policy(N, div=40.0, tol=1e-4, kind="reference", hfrac=0.05, hmin=0.01, hmax=10.0, capture=1.01,
                r_escape=1000.0):
    pol = _lib.StepPolicy()
    pol.kind = _lib.MK_POLICY_REFERENCE if kind == "reference" else _lib.MK_POLICY_FIXED
    pol.nmax = int(N)
    pol.div, pol.tol = float(div), float(tol)
    pol.hfrac, pol.hmin, pol.hmax = float(hfrac), float(hmin), float(hmax)
    pol.capture, pol.r_escape = float(capture), float(r_escape)
    return pol


def trace(s0, bhspin, policy, rows=False):
    """Integrate every ray to its stop; returns dict(K, why, state[, S, dt]).

    Reference policy: K = first stopped step (N if none), state = state after
    K steps; with rows=True also the full (N, npx, 8) rows and (N, npx) dt.
    Fixed policy: K = steps taken, state = final state."""
    s0 = f64(s0)
    if s0.ndim != 2 or s0.shape[1] != 8:
        raise ValueError("s0 must have shape (npx, 8)")
    npx = s0.shape[0]
    dev = s0.device
    K = torch.empty(npx, dtype=torch.int32, device=dev)
    why = torch.empty(npx, dtype=torch.int32, device=dev)
    state = torch.empty((npx, 8), dtype=torch.float64, device=dev)
    S = dt = None
    if rows:
        S = torch.empty((policy.nmax, npx, 8), dtype=torch.float64, device=dev)
        dt = torch.empty((policy.nmax, npx), dtype=torch.float64, device=dev)
    _lib.call("mk_integrate", ptr(s0), npx, float(bhspin), _lib.ctypes.byref(policy), ptr(S), ptr(dt), ptr(K),
              ptr(why), ptr(state), stream_ptr())
    out = dict(K=K, why=why, state=state)
    if rows:
        out["S"], out["dt"] = S, dt
    return out


def trimmed_rows(K, N):
    """Rows geodesic_integrator keeps (geodesics.py:275-281): the first row
    where every ray has dt == 0, plus 2, or all N rows."""
    K = K.to("cpu") if isinstance(K, torch.Tensor) else np.asarray(K)
    if len(K) and bool((K < N).all()):
        F = int(K.max())
        if F >= 1:
            return min(F + 2, N)
    return N


def geodesic_integrator(N, s0, div, tol, bhspin):
    """geodesics.py:233-281 -> (S[N_t, npx, 8], dt[N_t, npx]) CUDA tensors."""
    r = trace(s0, bhspin, step_policy(N, div, tol), rows=True)
    nt = trimmed_rows(r["K"], N)
    return r["S"][:nt], r["dt"][:nt]


def radius_cal(x, bhspin):
    """geodesics.py:284-291 over the last axis (>= 4 components)."""
    x = f64(x)
    shape = x.shape[:-1]
    flat = x.reshape(-1, x.shape[-1]).contiguous()
    r = torch.empty(flat.shape[0], dtype=torch.float64, device=x.device)
    _lib.call("mk_radius_cal", ptr(flat), flat.shape[0], flat.shape[1], float(bhspin), ptr(r), stream_ptr())
    return r.reshape(shape)


def select_photons_integrator(inc, angle, radius, bhspin, distance=1000, max_steps=2000):
    """geodesics.py:354-378: radius_cal at row argmax(dt) - 1 of each ray's
    trimmed trajectory (div 40, tol 1e-2)."""
    angle = np.atleast_1d(np.asarray(angle, dtype=np.float64))
    radius = np.broadcast_to(np.asarray(radius, dtype=np.float64), angle.shape)
    return _shadow_pass(inc, np.cos(angle), np.sin(angle), radius, bhspin, distance, max_steps)


def _shadow_pass(inc, ca, sa, mid, bhspin, distance, max_steps):
    dev = device()
    n = len(mid)
    ci, si = _cos_sin(inc)
    cat, sat, midt = f64(ca, dev), f64(sa, dev), f64(mid, dev)
    K = torch.empty(n, dtype=torch.int32, device=dev)
    best = torch.empty(n, dtype=torch.int32, device=dev)
    best_dt, r_km1, r_best, r_last = (torch.empty(n, dtype=torch.float64, device=dev) for _ in range(4))
    _lib.call("mk_shadow_pass", ptr(cat), ptr(sat), ptr(midt), n, float(bhspin), ci, si, float(distance),
              int(max_steps), ptr(K), ptr(best), ptr(best_dt), ptr(r_km1), ptr(r_best), ptr(r_last),
              stream_ptr())
    K, best = K.cpu().numpy(), best.cpu().numpy()
    best_dt, r_km1, r_best, r_last = (t.cpu().numpy() for t in (best_dt, r_km1, r_best, r_last))
    N = int(max_steps)
    # argmax(dt) over the trimmed rows: a stopped ray's rows from K on hold
    # dt == 0, and K always lies inside the trimmed range, so argmax is K
    # unless an accepted step had dt > 0; a ray that never stopped keeps all
    # N rows and argmax is its largest dt.
    out = np.empty(n)
    for p in range(n):
        if K[p] < N:
            am = best[p] if (best[p] >= 0 and best_dt[p] > 0) else K[p]
        else:
            am = best[p]
        row = am - 1
        if row < 0:
            out[p] = r_last[p]          # row -1 wraps to the last kept row
        elif am == K[p]:
            out[p] = r_km1[p]
        else:
            out[p] = r_best[p]
    return out


def find_shadow_bisection_angles(bhspin, inc, angles, max_steps=2000, error_allowed=0.001, max_it=40):
    """geodesics.py:405-435: bisection on 'fell in' (r < 100) per angle."""
    angles = np.asarray(angles, dtype=np.float64)
    ca, sa = np.cos(angles), np.sin(angles)
    inner = np.zeros_like(angles) + 0.5
    outer = np.zeros_like(angles) + 10
    error = outer - inner
    counter = 0
    while np.max(error) > error_allowed and counter < max_it:
        mid = (outer - inner) / 2 + inner
        final_mid = _shadow_pass(inc, ca, sa, mid, bhspin, 1000, max_steps)
        fell = np.where(final_mid < 100)
        got_away = np.where(final_mid >= 100)
        inner[fell] = (outer[fell] - inner[fell]) / 2 + inner[fell]
        outer[got_away] = (outer[got_away] - inner[got_away]) / 2 + inner[got_away]
        error = outer - inner
        counter += 1
    return inner


def find_shadow_bisection(bhspin, inc, num_angles, max_steps=2000, error_allowed=0.001, max_it=40):
    """geodesics.py:381-402."""
    angles = np.arange(num_angles) / num_angles * 2. * np.pi
    radii = find_shadow_bisection_angles(bhspin, inc, angles, max_it=max_it, error_allowed=error_allowed,
                                         max_steps=max_steps)
    return np.append(angles, angles[0]), np.append(radii, radii[0])
