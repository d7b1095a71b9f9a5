"""CPU oracle for the per-ray imaging path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU baseline
(and its ``--impl reference`` arm) may import this package, and only as the
checker or the timed CPU restatement of the reference; the shipped package
never does.

It restates the reference (Mahakala, Python+JAX) in plain C (``mk_oracle.c``)
plus NumPy for the pieces the reference itself runs in NumPy (camera grid,
ghost fill).  Every function names the reference file:line it follows.  It
is pinned against golden vectors produced by executing the unmodified
reference (``tests/golden/make_golden.py``) and against the reference's own
shadow fixture (``tests/data/shadow_data.npy`` re-saved as
``tests/golden/shadow.npz``).
"""

import ctypes
import math
import os

import numpy as np

from . import build as _build

_LIB = None

# cgs constants (mahakala/constants.py:22-31; MP from electrons.py:25)
EE = 4.8032e-10
KB = 1.3807e-16
CL = 2.99792458e10
ME = 9.1094e-28
MP = 1.6726e-24
HPL = 6.6261e-27
GNEWT = 6.6743e-8
Msun = 1.989e33

ST_ACTIVE, ST_CAPTURED, ST_ESCAPED, ST_MAXSTEPS, ST_NAN = 0, 1, 2, 3, 4

_D = ctypes.POINTER(ctypes.c_double)
_F = ctypes.POINTER(ctypes.c_float)
_I = ctypes.POINTER(ctypes.c_int32)


class _RenderParams(ctypes.Structure):
    _fields_ = [("bhspin", ctypes.c_double), ("div", ctypes.c_double), ("tol", ctypes.c_double),
                ("N", ctypes.c_int), ("fluid_gamma", ctypes.c_double), ("r_low", ctypes.c_double),
                ("r_high", ctypes.c_double), ("gem1", ctypes.c_double), ("gim1", ctypes.c_double),
                ("Ne_unit", ctypes.c_double), ("B_unit", ctypes.c_double),
                ("L_unit", ctypes.c_double), ("cos_fallback", ctypes.c_double),
                ("c2_11_12", ctypes.c_double), ("sigma_cut", ctypes.c_double),
                ("nnu", ctypes.c_int), ("nu", ctypes.c_double * 4)]


def lib():
    global _LIB
    if _LIB is None:
        _LIB = ctypes.CDLL(_build.build())
        _LIB.orc_radius_cal.restype = ctypes.c_double
        _LIB.orc_lookup.restype = ctypes.c_int
    return _LIB


def _p(a, kind=_D):
    return a.ctypes.data_as(kind)


def _c(a, dtype=np.float64):
    return np.ascontiguousarray(a, dtype=dtype)


# ---------------------------------------------------------------- camera
def _jnp_linspace(start, stop, num):
    """jnp.linspace (used by the equator camera, geodesics.py:185)."""
    start, stop = np.float64(start), np.float64(stop)
    div = num - 1
    step = np.arange(div, dtype=np.float64) / np.float64(div)
    out = start * (1.0 - step) + stop * step
    return np.concatenate([out, [stop]])


def camera_grid_list(fov_lower, fov_upper, pixels_per_side):
    """Pixel centres, ``np.linspace(lo, hi, 2n+1)[1::2]`` (geodesics.py:160)."""
    return np.linspace(fov_lower, fov_upper, 2 * pixels_per_side + 1)[1::2]


def inclination_cos_sin(inclination):
    i = inclination * np.pi / 180  # geodesics.py:205
    return float(np.cos(i)), float(np.sin(i))


def initialize_geodesics_at_camera(bhspin, inclination, distance, fov_lower, fov_upper,
                                   pixels_per_side, camera_type="grid"):
    """geodesics.py:29-55 -> (npx, 8)."""
    ci, si = inclination_cos_sin(inclination)
    if camera_type.lower() == "grid":
        g = _c(camera_grid_list(fov_lower, fov_upper, pixels_per_side))
        n = len(g)
        s0 = np.empty((n * n, 8))
        lib().orc_camera_grid(_p(g), ctypes.c_int(n), ctypes.c_double(ci), ctypes.c_double(si),
                              ctypes.c_double(distance), ctypes.c_double(bhspin), _p(s0))
        return s0
    if camera_type.lower() == "equator":
        g = _jnp_linspace(fov_lower, fov_upper, 2 * pixels_per_side + 1)[1::2]
        n = len(g)
        s0 = np.zeros((n, 8))
        s0[:, 1] = distance
        s0[:, 2] = g
        s0[:, 4] = 1.0
        s0[:, 5] = 1.0
        out = np.empty_like(s0)
        # nullify only (orc_camera_polar would rebuild the direction)
        for p in range(n):
            out[p] = _nullify_py(s0[p], bhspin)
        return out
    raise ValueError(f'Unexpected camera type "{camera_type}"')


def _metric_py(x, a):
    aa = a * a
    zz = x[3] * x[3]
    kk = 0.5 * (x[1] * x[1] + x[2] * x[2] + zz - aa)
    rr = math.sqrt(kk * kk + aa * zz) + kk
    r = math.sqrt(rr)
    f = (2.0 * rr * r) / (rr * rr + aa * zz)
    l = np.array([1.0, (r * x[1] + a * x[2]) / (rr + aa), (r * x[2] - a * x[1]) / (rr + aa), x[3] / r])
    return np.diag([-1.0, 1.0, 1.0, 1.0]) + f * np.outer(l, l)


def _nullify_py(s, a):
    """_Nullify with p=1 (geodesics.py:58-85) for one ray."""
    x, v = s[:4], s[4:].copy()
    g = _metric_py(x, a)
    A = (v[0] * g[0, 0]) * v[0]
    b = ((v[1] * g[1, 0] + v[2] * g[2, 0]) + v[3] * g[3, 0]) * v[0]
    w = [(v[1] * g[1, 1 + j] + v[2] * g[2, 1 + j]) + v[3] * g[3, 1 + j] for j in range(3)]
    C = (w[0] * v[1] + w[1] * v[2]) + w[2] * v[3]
    bb, AC = b * b, A * C
    dd = 0.0 if abs(bb - AC) <= 1e-8 + 1e-5 * abs(AC) else bb - AC
    bs = 0.0 if b < 0 else 1.0
    with np.errstate(all="ignore"):
        D = -(b + bs * np.sqrt(dd))
        x1, x2 = D / A, C / D
    if np.isnan(x1) or np.isnan(x2):
        d1 = d2 = np.nan
    else:
        d1, d2 = min(x1, x2), max(x1, x2)
    S = d1 if d1 > 0 else (d2 if d2 > 0 else np.nan)
    out = s.copy()
    out[5:] = v[1:] / S
    return out


# ------------------------------------------------------------ geodesics
def radius_cal(x, bhspin):
    """geodesics.py:284-291 (vectorised)."""
    x = np.asarray(x)
    R = np.sqrt(x[..., 1] ** 2 + x[..., 2] ** 2 + x[..., 3] ** 2)
    return np.sqrt((R ** 2 - bhspin ** 2 + np.sqrt((R ** 2 - bhspin ** 2) ** 2
                                                    + 4 * bhspin ** 2 * x[..., 3] ** 2)) / 2)


def radius_EH(a):
    return 1 + np.sqrt(1 - a ** 2)


def integrate(s0, N, div, tol, bhspin, full=False):
    """Per-ray integration with the reference step rule.

    Returns dict(K, why, state[, S, dt]) where K is the first frozen step (N if
    the ray never froze) and state the ray's state after K steps."""
    s0 = _c(s0)
    npx = s0.shape[0]
    K = np.empty(npx, np.int32)
    why = np.empty(npx, np.int32)
    state = np.empty((npx, 8))
    S = np.empty((N, npx, 8)) if full else None
    dt = np.empty((N, npx)) if full else None
    lib().orc_integrate(_p(s0), ctypes.c_int(npx), ctypes.c_int(N), ctypes.c_double(div),
                        ctypes.c_double(tol), ctypes.c_double(bhspin),
                        _p(S) if full else None, _p(dt) if full else None,
                        _p(K, _I), _p(why, _I), _p(state))
    out = dict(K=K, why=why, state=state)
    if full:
        out["S"], out["dt"] = S, dt
    return out


def perturbed(s0, eps=1e-12, direction=0):
    """s0 with a rounding-sized change of the initial wavevector: direction 0
    scales its spatial part by (1 + eps); 1, 2, 3 tilt it by eps |k| along
    x, y, z.  Probes of how strongly each ray amplifies such a change."""
    s = np.array(s0, dtype=np.float64, copy=True)
    if direction == 0:
        s[:, 5:8] *= (1.0 + eps)
    else:
        s[:, 4 + direction] += eps * np.linalg.norm(s[:, 5:8], axis=1)
    return s


def amplification(state, state_pert, eps=1e-12, floor=1e-3):
    """Per ray: relative end-state change (floor 1e-3 for components near
    zero) per unit relative change eps of the initial wavevector.  Rounding
    differences of two FP64 evaluation orders (~1e-13 accumulated over a
    ray) reach the end state multiplied by this factor; rays near the
    critical curve reach 1e5 and more."""
    with np.errstate(all="ignore"):
        d = np.abs(state - state_pert) / np.maximum(np.abs(state), floor)
    d = np.where(np.isnan(d), np.inf, d)
    return d.reshape(d.shape[0], -1).max(axis=1) / eps


def conditioning(run, s0, key_state="state", key_steps="K", eps=1e-12):
    """Per-ray amplification, the largest over the four probe directions of
    perturbed(); inf where a probe changes the ray's step count.  Returns
    (unperturbed result, amplification)."""
    base = run(s0)
    amp = np.zeros(len(s0))
    for d in range(4):
        pr = run(perturbed(s0, eps, d))
        a = amplification(base[key_state], pr[key_state], eps)
        amp = np.maximum(amp, np.where(base[key_steps] != pr[key_steps], np.inf, a))
    return base, amp


def trimmed_rows(K, N):
    """Number of trajectory rows geodesic_integrator keeps (geodesics.py:275-281)."""
    if np.all(K < N):
        F = int(np.max(K))
        if F >= 1:
            return min(F + 2, N)
    return N


def geodesic_integrator(N, s0, div, tol, bhspin):
    """geodesics.py:233-281 -> (S[N_t, npx, 8], dt[N_t, npx])."""
    r = integrate(s0, N, div, tol, bhspin, full=True)
    nt = trimmed_rows(r["K"], N)
    return r["S"][:nt], r["dt"][:nt]


def end_state(K, state_after_K, s_rows=None):
    """Last trajectory row: the state after min(K, N-1) steps."""
    return state_after_K


def find_shadow_bisection_angles(bhspin, inc, angles, max_steps=2000, error_allowed=0.001,
                                 max_it=40, distance=1000.0):
    """geodesics.py:405-435."""
    angles = _c(angles)
    ca, sa = _c(np.cos(angles)), _c(np.sin(angles))
    ci, si = inclination_cos_sin(inc)
    out = np.empty(len(angles))
    lib().orc_shadow_bisection(_p(ca), _p(sa), ctypes.c_int(len(angles)), ctypes.c_double(ci),
                               ctypes.c_double(si), ctypes.c_double(bhspin),
                               ctypes.c_double(distance), ctypes.c_int(max_steps),
                               ctypes.c_double(error_allowed), ctypes.c_int(max_it), _p(out))
    return out


def trace_fixed(s0, N, bhspin, hfrac=0.05, hmin=0.01, hmax=10.0, capture=1.01, r_escape=1000.0):
    """Vacuum trace with the fixed-fraction step policy (not in the reference)."""
    s0 = _c(s0)
    npx = s0.shape[0]
    state = np.empty((npx, 8))
    nsteps = np.empty(npx, np.int32)
    why = np.empty(npx, np.int32)
    lib().orc_trace_fixed(_p(s0), ctypes.c_int(npx), ctypes.c_int(N), ctypes.c_double(bhspin),
                          ctypes.c_double(hfrac), ctypes.c_double(hmin), ctypes.c_double(hmax),
                          ctypes.c_double(capture), ctypes.c_double(r_escape), _p(state),
                          _p(nsteps, _I), _p(why, _I))
    return dict(state=state, nsteps=nsteps, why=why)


# ------------------------------------------------------- emission/transfer
def rlow_rhigh_model(dens, u, beta, r_low=1, r_high=40, electron_gamma=4. / 3, ion_gamma=5. / 3):
    """electrons.py:32-50."""
    dens, u, beta = np.broadcast_arrays(_c(dens), _c(u), _c(beta))
    dens, u, beta = _c(dens), _c(u), _c(beta)
    out = np.empty(dens.shape)
    lib().orc_rlow_rhigh(_p(dens), _p(u), _p(beta), ctypes.c_int64(dens.size),
                         ctypes.c_double(r_low), ctypes.c_double(r_high),
                         ctypes.c_double(electron_gamma - 1.), ctypes.c_double(ion_gamma - 1.),
                         _p(out))
    return out


def synchrotron_coefficients(Ne, Theta_e, B, pitch_angle, nu, invariant=True, rescale_nu=1.):
    """transfer.py:30-86."""
    arrs = np.broadcast_arrays(*[_c(v) for v in (Ne, Theta_e, B, pitch_angle, nu)])
    arrs = [_c(v) for v in arrs]
    em = np.empty(arrs[0].shape)
    ab = np.empty(arrs[0].shape)
    lib().orc_synchrotron(*[_p(v) for v in arrs], ctypes.c_int64(em.size), ctypes.c_int(int(bool(invariant))),
                          ctypes.c_double(rescale_nu), ctypes.c_double(2.0 ** (11. / 12)),
                          _p(em), _p(ab))
    return em, ab


def solve_specific_intensity(emissivity, absorptivity, dt, L_unit, dIs=False):
    """transfer.py:89-119."""
    em, ab, dt = _c(emissivity), _c(absorptivity), _c(dt)
    nsteps, npx = em.shape
    I = np.empty(npx)
    d = np.empty((max(nsteps - 1, 0), npx)) if dIs else None
    lib().orc_solve_intensity(_p(em), _p(ab), _p(dt), ctypes.c_int(nsteps), ctypes.c_int(npx),
                              ctypes.c_double(L_unit), _p(I), _p(d) if dIs else None)
    return (I, d) if dIs else I


def solve_attenuated_emissivity(emissivity, absorptivity, dt, L_unit):
    """transfer.py:122-144."""
    em, ab, dt = _c(emissivity), _c(absorptivity), _c(dt)
    nsteps, npx = em.shape
    out = np.empty((max(nsteps - 1, 0), npx))
    lib().orc_attenuated_emissivity(_p(em), _p(ab), _p(dt), ctypes.c_int(nsteps), ctypes.c_int(npx),
                                    ctypes.c_double(L_unit), _p(out))
    return out


def get_units(M_BH, mass_scale):
    """grmhd/grmhd.py:40-55."""
    L_unit = GNEWT * M_BH / CL ** 2
    T_unit = L_unit / CL
    dens_unit = mass_scale / L_unit ** 3
    Ne_unit = dens_unit / (MP + ME)
    B_unit = CL * np.sqrt(4. * np.pi * dens_unit)
    return dict(L_unit=L_unit, T_unit=T_unit, dens_unit=dens_unit, Ne_unit=Ne_unit, B_unit=B_unit)


# --------------------------------------------------------------- snapshot
class OracleSnapshot:
    """Ghost-filled meshblocks + geometry, as AthenakFluidModel holds them.

    ``all_meshblocks`` is ``(nmb, 8, n+2, n+2, n+2)`` float64 indexed
    ``[mb, prim, k, j, i]`` (athenak.py:124-127, 145).  Single-level meshes
    take the same-level ghost copy of athenak.py:217-233 (zero ghosts at the
    domain edge); multi-level meshes the full fill of athenak.py:160-525
    (``oracle.amr``), with the literal O(nmb) lookup."""

    def __init__(self, arrs, bhspin=None, fluid_gamma=None, fast_lookup=True):
        uov, B = arrs.uov, arrs.B
        nprim, nmb, nk, nj, ni = uov.shape
        if not (nk == nj == ni):
            raise NotImplementedError("cubic meshblocks only")
        levels = np.asarray(arrs.Levels)
        multilevel = bool(np.any(levels != levels[0]))
        n = ni
        self.n, self.nmb = n, nmb
        self.bhspin = float(arrs.bhspin if bhspin is None else bhspin)
        self.fluid_gamma = float(arrs.fluid_gamma if fluid_gamma is None else fluid_gamma)
        locs = np.asarray(arrs.LogicalLocations)
        data = np.concatenate([uov, B], axis=0)  # (8, nmb, k, j, i)
        if multilevel:
            from .amr import multilevel_meshblocks
            mbs = multilevel_meshblocks(data, locs, levels)
            fast_lookup = False
        else:
            index = {tuple(int(v) for v in locs[m]): m for m in range(nmb)}
            mbs = np.zeros((nmb, 8, n + 2, n + 2, n + 2), dtype=np.float64)
            mbs[:, :, 1:-1, 1:-1, 1:-1] = data.transpose(1, 0, 2, 3, 4)
            for m in range(nmb):
                ti, tj, tk = (int(v) for v in locs[m])
                for di in (-1, 0, 1):
                    for dj in (-1, 0, 1):
                        for dk in (-1, 0, 1):
                            if di == dj == dk == 0:
                                continue
                            nb = index.get((ti + di, tj + dj, tk + dk))
                            if nb is None:
                                continue
                            src = [0 if d == 1 else (-1 if d == -1 else slice(0, n)) for d in (di, dj, dk)]
                            tgt = [-1 if d == 1 else (0 if d == -1 else slice(1, n + 1)) for d in (di, dj, dk)]
                            mbs[m, :, tgt[2], tgt[1], tgt[0]] = data[:, nb, src[2], src[1], src[0]]
        self.all_meshblocks = mbs
        self.ext = _c(np.stack([arrs.x1f[:, 0], arrs.x1f[:, -1], arrs.x2f[:, 0], arrs.x2f[:, -1],
                                arrs.x3f[:, 0], arrs.x3f[:, -1]], axis=1))
        self.left = _c(np.stack([arrs.x1v[:, 0], arrs.x2v[:, 0], arrs.x3v[:, 0]], axis=1))
        self.dx = _c(np.stack([arrs.x1v[:, 1] - arrs.x1v[:, 0], arrs.x2v[:, 1] - arrs.x2v[:, 0],
                               arrs.x3v[:, 1] - arrs.x3v[:, 0]], axis=1))
        self.faces = None
        self.nb = None
        self.table = None
        if fast_lookup:
            nbx = [int(locs[:, c].max()) + 1 for c in range(3)]
            if nbx[0] * nbx[1] * nbx[2] == nmb:
                faces = []
                for c, (f, v) in enumerate(((arrs.x1f, 0), (arrs.x2f, 1), (arrs.x3f, 2))):
                    fa = np.empty(nbx[c] + 1)
                    for m in range(nmb):
                        fa[locs[m, c]] = f[m, 0]
                        fa[locs[m, c] + 1] = f[m, -1]
                    faces.append(_c(fa))
                table = np.empty((nbx[2], nbx[1], nbx[0]), np.int32)
                for m in range(nmb):
                    table[locs[m, 2], locs[m, 1], locs[m, 0]] = m
                self.faces, self.nb, self.table = faces, np.array(nbx, np.int32), _c(table, np.int32)

    def _args(self):
        f = self.faces
        return (_p(self.all_meshblocks), ctypes.c_int(self.nmb), ctypes.c_int(self.n),
                _p(self.ext), _p(self.left), _p(self.dx),
                _p(f[0]) if f else None, _p(f[1]) if f else None, _p(f[2]) if f else None,
                _p(self.nb, _I) if f else None, _p(self.table, _I) if f else None,
                ctypes.c_double(self.bhspin))

    def get_fluid_scalars_from_geodesics(self, S, fallback_pitch_angle=np.pi / 3.):
        """athenak.py:639-812 -> dict(dens, u, pitch_angle, kdotu, b)."""
        S = _c(S)
        shape = S.shape[:-1]
        npts = int(np.prod(shape))
        out = np.empty((npts, 5))
        lib().orc_fluid_scalars(*self._args(), _p(S), ctypes.c_int64(npts),
                                ctypes.c_double(np.cos(fallback_pitch_angle)), _p(out))
        out = out.reshape(shape + (5,))
        return dict(dens=out[..., 0], u=out[..., 1], pitch_angle=out[..., 2], kdotu=out[..., 3],
                    b=out[..., 4])

    def get_prims_from_geodesics(self, S):
        """athenak.py:527-637 -> dict of the 8 primitives (+ block ids)."""
        S = _c(S)
        shape = S.shape[:-1]
        npts = int(np.prod(shape))
        out = np.empty((npts, 8))
        blk = np.empty(npts, np.int32)
        lib().orc_fluid_prims(*self._args(), _p(S), ctypes.c_int64(npts), _p(out), _p(blk, _I))
        out = out.reshape(shape + (8,))
        names = ("dens", "U1", "U2", "U3", "u", "B1", "B2", "B3")
        d = {k: out[..., i] for i, k in enumerate(names)}
        d["block"] = blk.reshape(shape)
        return d


def _render_params(snapshot, mass_scale, M_bh, r_high, freqs, max_nsteps, r_low, div, tol):
    units = get_units(M_bh, mass_scale)
    P = _RenderParams()
    P.bhspin, P.div, P.tol, P.N = snapshot.bhspin, div, tol, int(max_nsteps)
    P.fluid_gamma, P.r_low, P.r_high = snapshot.fluid_gamma, r_low, r_high
    P.gem1, P.gim1 = 4. / 3 - 1., 5. / 3 - 1.
    P.Ne_unit, P.B_unit, P.L_unit = units["Ne_unit"], units["B_unit"], units["L_unit"]
    P.cos_fallback = float(np.cos(np.pi / 3.))
    P.c2_11_12 = 2.0 ** (11. / 12)
    P.sigma_cut = 100.
    P.nnu = len(freqs)
    for i, f in enumerate(freqs):
        P.nu[i] = f
    return P


def render_rays(snapshot, s0, mass_scale=1.e26, M_bh=6.2e9 * Msun, r_high=40, observing_frequency=230.e9,
                max_nsteps=10000, r_low=1, div=40, tol=1e-4):
    """make_image's per-ray work (images.py:79-120) for the rays s0 (npx, 8):
    returns (intensity (nnu, npx), steps (npx))."""
    freqs = np.atleast_1d(np.asarray(observing_frequency, dtype=np.float64))
    if len(freqs) > 4:
        raise ValueError("at most 4 frequencies")
    P = _render_params(snapshot, mass_scale, M_bh, r_high, freqs, max_nsteps, r_low, div, tol)
    s0 = _c(s0)
    npx = s0.shape[0]
    img = np.empty((len(freqs), npx))
    steps = np.empty(npx, np.int32)
    lib().orc_render(ctypes.byref(P), *snapshot._args()[:-1], s0.ctypes.data_as(_D), ctypes.c_int(npx),
                     _p(img), _p(steps, _I))
    return img, steps


def make_image(snapshot, camera_inclination=60, camera_distance=1000, mass_scale=1.e26,
               M_bh=6.2e9 * Msun, r_high=40, observing_frequency=230.e9, fov=20, resolution=160,
               max_nsteps=10000, r_low=1, div=40, tol=1e-4, return_steps=False, bhspin=None):
    """images.py:30-144, one ray at a time; ``observing_frequency`` may be a
    list (one image per frequency, same rays).  Returns (res, res) or
    (nnu, res, res)."""
    a = snapshot.bhspin if bhspin is None else bhspin
    s0 = initialize_geodesics_at_camera(a, camera_inclination, camera_distance, -fov / 2.,
                                        fov / 2., resolution)
    snap = snapshot if bhspin is None else _with_spin(snapshot, a)
    img, steps = render_rays(snap, s0, mass_scale, M_bh, r_high, observing_frequency, max_nsteps, r_low, div, tol)
    img = img.reshape(-1, resolution, resolution)
    if np.ndim(observing_frequency) == 0:
        img = img[0]
    return (img, steps.reshape(resolution, resolution)) if return_steps else img


def _with_spin(snapshot, a):
    import copy
    s = copy.copy(snapshot)
    s.bhspin = float(a)
    return s


def image_parity(img, steps, ref_img, ref_steps, pert_img, pert_steps, floor_frac=1e-4, ill_tol=1e-10,
                 bar=1e-8):
    """Checker of an FP64 image against the oracle's render of the same rays.

    img, ref_img, pert_img: (nnu, n) intensities of the same n rays -- the
    image under test, the oracle, and the oracle with each ray's initial
    wavevector perturbed by 1e-12 (``perturbed``); steps, ref_steps,
    pert_steps: (n,) accepted steps per ray.  A ray is ill-conditioned when
    the perturbed oracle run changes its step count or moves any channel by
    more than ``ill_tol`` relative (floor ``floor_frac`` of the channel's
    maximum): two FP64 evaluation orders then legitimately differ by more
    than rounding.  On the conditioned rays the steps must be equal, every
    pixel within ``bar`` relative and the summed flux within ``bar``.
    Returns a dict of the counts and errors and ``ok``."""
    img, ref, pert = (np.atleast_2d(np.asarray(x, dtype=np.float64)) for x in (img, ref_img, pert_img))
    steps, ref_steps, pert_steps = (np.asarray(x).reshape(-1) for x in (steps, ref_steps, pert_steps))
    floor = floor_frac * np.abs(ref).max(axis=1, keepdims=True)

    def rel(a, b):
        den = np.maximum(np.abs(b), floor)
        with np.errstate(all="ignore"):
            e = np.abs(a - b) / np.where(den > 0, den, 1.0)
        return np.where((a == b) | (np.isnan(a) & np.isnan(b)), 0.0, e)

    ill = (pert_steps != ref_steps) | (rel(pert, ref) > ill_tol).any(axis=0)
    ok_rays = ~ill
    n_ok = int(ok_rays.sum())
    steps_equal = bool(np.array_equal(steps[ok_rays], ref_steps[ok_rays]))
    err = rel(img, ref)
    max_pix = float(err[:, ok_rays].max()) if n_ok else 0.0
    fl, fl_ref = img[:, ok_rays].sum(axis=1), ref[:, ok_rays].sum(axis=1)
    with np.errstate(all="ignore"):
        flux = float(np.max(np.abs(fl - fl_ref) / np.where(fl_ref != 0, np.abs(fl_ref), 1.0)))
        flux_all = float(np.max(np.abs(img.sum(axis=1) - ref.sum(axis=1)) / np.abs(ref.sum(axis=1))))
    return {"rays": int(len(ref_steps)), "ill_conditioned": int(ill.sum()), "steps_equal": steps_equal,
            "max_pixel_rel_err": max_pix, "flux_rel_err": flux, "flux_rel_err_all_rays": flux_all,
            "max_pixel_rel_err_all_rays": float(err.max()), "bar": bar,
            "ok": bool(steps_equal and max_pix <= bar and flux <= bar and ill.mean() < 0.05)}
