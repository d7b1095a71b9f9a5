"""Generate golden vectors by executing the UNMODIFIED reference (Mahakala).

Run where the reference checkout exists, naming it in ``MAHAKALA_REF``::

    MAHAKALA_REF=<path to the Mahakala checkout> python tests/golden/make_golden.py [name ...]

jax is not installable offline, so ``jaxshim.install()`` provides a NumPy
stand-in for the jax subset the reference uses (see ``jaxshim.py``); the
reference's own ``.py`` files are imported in place and called through their
public API.  Each fixture is a small ``.npz`` beside this script.  The GPU
machine never runs this script; tests there only read the ``.npz`` files.

Fixtures:
  camera        initialize_geodesics_at_camera (grid and equator cameras)
  integrator    geodesic_integrator trajectories (geodesics.py:233-281)
  shadow        the reference's own tests/data/shadow_data.npy, re-saved
  synchrotron   synchrotron_coefficients (transfer.py:30-86)
  electrons     rlow_rhigh_model (electrons.py:32-50)
  transfer      solve_specific_intensity / solve_attenuated_emissivity
  units         GRMHDFluidModel.get_units (grmhd/grmhd.py:40-55)
  snapshot      AthenakFluidModel.load_athenak_meshblocks ghost fill on a
                tiny synthetic snapshot (grmhd/athenak.py:67-158)
  scalars       get_fluid_scalars_from_geodesics (grmhd/athenak.py:639-812)
  image         make_image (images.py:30-144) on the tiny snapshot
  amr           two multi-level meshes: ghost fill (grmhd/athenak.py:67-525),
                sampled primitives and scalars (:527-812), one image
"""

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("MAHAKALA_REF")
if not REF or not os.path.isdir(os.path.join(REF, "mahakala")):
    sys.exit("make_golden.py: set MAHAKALA_REF to the Mahakala checkout (the directory holding mahakala/)")

sys.path.insert(0, HERE)
sys.path.insert(0, REPO)
sys.path.insert(0, REF)

import jaxshim  # noqa: E402

jaxshim.install()

import mahakala as ma  # noqa: E402
from mahakala.electrons import rlow_rhigh_model  # noqa: E402
from mahakala.grmhd.grmhd import GRMHDFluidModel  # noqa: E402
from mahakala.grmhd.athenak import AthenakFluidModel  # noqa: E402
from mahakala.images import make_image  # noqa: E402
from mahakala.constants import Msun  # noqa: E402

from mahakala_gb300.grmhd.synthetic import make_synthetic_snapshot  # noqa: E402

J = jaxshim.JArray


def _save(name, **arrays):
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **arrays)
    print(f"wrote {path} ({os.path.getsize(path)} bytes)")


CAMERA_CASES = [
    # (bhspin, inclination, distance, fov_lower, fov_upper, pixels, camera)
    (0.94, 60.0, 1000.0, -10.0, 10.0, 8, "grid"),
    (0.5, 17.0, 1000.0, -25.0, 25.0, 6, "grid"),
    (0.0, 85.0, 1000.0, -10.0, 10.0, 5, "grid"),
    (0.9, 90.0, 500.0, -7.0, 3.0, 4, "grid"),
    (0.0, 60.0, 1000.0, -15.0, 15.0, 8, "Equator"),
]


def gen_camera():
    out = {}
    for n, case in enumerate(CAMERA_CASES):
        s0 = ma.initialize_geodesics_at_camera(*case[:6], camera_type=case[6])
        out[f"case{n}_params"] = np.array(case[:6], dtype=np.float64)
        out[f"case{n}_equator"] = np.array(case[6].lower() == "equator")
        out[f"case{n}_s0"] = np.asarray(s0)
    _save("camera", **out)


INTEGRATOR_CASES = [
    # (bhspin, inc, fov half-width, pixels, N, div, tol)
    (0.94, 60.0, 10.0, 4, 1500, 40.0, 1e-4),   # all rays stop before N
    (0.5, 17.0, 8.0, 3, 300, 40.0, 1e-2),      # N reached: trim to N rows
    (0.0, 85.0, 6.0, 3, 1200, 20.0, 1e-4),     # another divisor
]


def gen_integrator():
    out = {}
    for n, (a, inc, half, px, N, div, tol) in enumerate(INTEGRATOR_CASES):
        t0 = time.time()
        s0 = ma.initialize_geodesics_at_camera(a, inc, 1000.0, -half, half, px)
        S, dt = ma.geodesic_integrator(N, s0, div, tol, a)
        S = np.asarray(S)
        dt = np.asarray(dt)
        out[f"case{n}_params"] = np.array([a, inc, half, px, N, div, tol])
        out[f"case{n}_s0"] = np.asarray(s0)
        out[f"case{n}_rows"] = np.array(S.shape[0])
        out[f"case{n}_last"] = S[-1]
        out[f"case{n}_nsteps"] = (dt != 0).sum(axis=0)
        out[f"case{n}_dtsum"] = dt.sum(axis=0)
        # full trajectory of a few rays pins the per-step state and dt
        keep = np.arange(0, S.shape[1], max(1, S.shape[1] // 4))[:4]
        out[f"case{n}_keep"] = keep
        out[f"case{n}_S_keep"] = S[:, keep, :]
        out[f"case{n}_dt_keep"] = dt[:, keep]
        print(f"integrator case {n}: rows {S.shape[0]} in {time.time()-t0:.1f}s")
    _save("integrator", **out)


def gen_shadow():
    path = os.path.join(REF, "tests", "data", "shadow_data.npy")
    data = np.load(path, allow_pickle=True).item()
    out = {}
    for key in sorted(data):
        d = data[key]
        out[f"{key}_bhspin"] = np.array(float(d["bhspin"]))
        out[f"{key}_inclination"] = np.array(float(d["inclination"]))
        out[f"{key}_angles"] = np.asarray(d["angles"], dtype=np.float64)
        out[f"{key}_radii"] = np.asarray(d["radii"], dtype=np.float64)
    out["keys"] = np.array(sorted(data))
    # a short literal bisection run pins the exact iteration rule
    t0 = time.time()
    ang = np.asarray(data["test4"]["angles"][:3], dtype=np.float64)
    r = ma.find_shadow_bisection_angles(0.71, 13.0, ang, max_steps=2000,
                                        error_allowed=1e-3, max_it=6)
    out["short_angles"] = ang
    out["short_params"] = np.array([0.71, 13.0, 2000, 1e-3, 6])
    out["short_radii"] = np.asarray(r)
    print(f"short bisection in {time.time()-t0:.1f}s")
    _save("shadow", **out)


def _synchro_inputs(rng, n):
    Ne = 10 ** rng.uniform(2, 7, n)
    Theta = 10 ** rng.uniform(-1, 2.5, n)
    B = 10 ** rng.uniform(-1, 2.5, n)
    pitch = rng.uniform(0.01, np.pi - 0.01, n)
    nu = 10 ** rng.uniform(9.5, 12.5, n)
    # edge cases: Theta_e < 0.3 cut, X > 1e12 cut, Planck series branch,
    # NaN inputs, zero field, tiny pitch angle
    Theta[:8] = [0.1, 0.29, 0.3, 0.31, 1e-3, 1e4, 5e5, 2e6]
    B[8:12] = [0.0, 1e-12, 1e-9, 1e4]
    pitch[12:16] = [0.0, 1e-8, np.pi / 2, np.pi]
    Ne[16] = np.nan
    Theta[17] = np.nan
    nu[18:22] = [1e8, 1e6, 1e15, 1e17]
    Theta[22:26] = [3e4, 1e5, 1e6, 1e7]
    return Ne, Theta, B, pitch, nu


def gen_synchrotron():
    rng = np.random.Generator(np.random.PCG64(1234))
    n = 400
    Ne, Theta, B, pitch, nu = _synchro_inputs(rng, n)
    out = dict(Ne=Ne, Theta=Theta, B=B, pitch=pitch, nu=nu)
    with np.errstate(all="ignore"):
        em, ab = ma.synchrotron_coefficients(Ne.view(J), Theta.view(J),
                                             B.view(J), pitch.view(J), nu.view(J),
                                             invariant=True, rescale_nu=1. / 230e9)
        out["em_inv"] = np.asarray(em)
        out["ab_inv"] = np.asarray(ab)
        em, ab = ma.synchrotron_coefficients(Ne.view(J), Theta.view(J), B.view(J),
                                             pitch.view(J), nu.view(J),
                                             invariant=False)
        out["em_raw"] = np.asarray(em)
        out["ab_raw"] = np.asarray(ab)
        em, ab = ma.synchrotron_coefficients(Ne.view(J), Theta.view(J), B.view(J),
                                             pitch.view(J), nu.view(J),
                                             invariant=True, rescale_nu=1.)
        out["em_inv1"] = np.asarray(em)
        out["ab_inv1"] = np.asarray(ab)
    _save("synchrotron", **out)


def gen_electrons():
    rng = np.random.Generator(np.random.PCG64(99))
    n = 300
    dens = 10 ** rng.uniform(-4, 1, n)
    u = dens * 10 ** rng.uniform(-3, 0, n)
    beta = 10 ** rng.uniform(-3, 3, n)
    beta[:4] = [0.0, np.inf, np.nan, 1.0]
    out = dict(dens=dens, u=u, beta=beta)
    with np.errstate(all="ignore"):
        for tag, kw in [("default", {}), ("rhigh1", dict(r_high=1)),
                        ("rhigh10", dict(r_high=10)),
                        ("rhigh80_rlow3", dict(r_high=80, r_low=3)),
                        ("gammas", dict(electron_gamma=5. / 3, ion_gamma=4. / 3))]:
            out["theta_" + tag] = np.asarray(
                rlow_rhigh_model(dens.view(J), u.view(J), beta.view(J), **kw))
    _save("electrons", **out)


def gen_transfer():
    rng = np.random.Generator(np.random.PCG64(7))
    nsteps, npx = 40, 12
    em = 10 ** rng.uniform(-20, -14, (nsteps, npx))
    ab = 10 ** rng.uniform(-30, -22, (nsteps, npx))
    dt = -rng.uniform(0.01, 20.0, (nsteps, npx))
    dt[25:, :3] = 0.0      # rays that stopped early
    dt[5:9, 5] = 0.0       # a frozen stretch
    em[:, 7] = 0.0
    ab[10:20, 8] = 10 ** rng.uniform(-18, -17, 10)   # optically thick part
    L_unit = 9.152e14
    out = dict(em=em, ab=ab, dt=dt, L_unit=np.array(L_unit))
    out["I"] = np.asarray(ma.solve_specific_intensity(em.view(J), ab.view(J), dt.view(J), L_unit))
    I2, dIs = ma.solve_specific_intensity(em.view(J), ab.view(J), dt.view(J), L_unit, dIs=True)
    out["I_dIs"] = np.asarray(I2)
    out["dIs"] = np.asarray(dIs)
    out["att"] = np.asarray(ma.solve_attenuated_emissivity(em.view(J), ab.view(J), dt.view(J), L_unit))
    _save("transfer", **out)


def gen_units():
    m = GRMHDFluidModel()
    cases = [(6.2e9 * Msun, 1e26), (6.5e9 * Msun, 3.1e25), (4.1e6 * Msun, 1e19)]
    out = {}
    for n, (M, ms) in enumerate(cases):
        u = m.get_units(M, ms)
        out[f"case{n}_in"] = np.array([M, ms])
        out[f"case{n}_out"] = np.array([u["L_unit"], u["T_unit"], u["dens_unit"],
                                        u["Ne_unit"], u["B_unit"]])
    _save("units", **out)


TINY = dict(nblocks=2, cells_per_block=8, extent=20.0, bhspin=0.9, seed=5)


def _tiny_model(fluid_gamma=13. / 9):
    snap = make_synthetic_snapshot(**TINY)
    name = "tiny_synthetic.athdf"
    datasets = dict(uov=snap.uov, B=snap.B, x1v=snap.x1v, x2v=snap.x2v, x3v=snap.x3v,
                    x1f=snap.x1f, x2f=snap.x2f, x3f=snap.x3f,
                    LogicalLocations=snap.LogicalLocations, Levels=snap.Levels)
    attrs = {"VariableNames": np.array([v.encode() for v in snap.VariableNames])}
    jaxshim.register_h5(name, datasets, attrs)
    model = AthenakFluidModel(name, TINY["bhspin"], fluid_gamma=fluid_gamma)
    return snap, model


def gen_snapshot():
    snap, model = _tiny_model()
    mbs = np.asarray(model.all_meshblocks)
    assert np.array_equal(mbs.astype(np.float32).astype(np.float64), mbs)
    _save("snapshot", uov=snap.uov, B=snap.B, x1v=snap.x1v, x2v=snap.x2v,
          x3v=snap.x3v, x1f=snap.x1f, x2f=snap.x2f, x3f=snap.x3f,
          LogicalLocations=snap.LogicalLocations, Levels=snap.Levels,
          all_meshblocks=mbs.astype(np.float32),
          params=np.array([TINY["nblocks"], TINY["cells_per_block"], TINY["extent"],
                           TINY["bhspin"], TINY["seed"]]))


def _scalar_points(rng, nrows, npx, extent, a):
    """Sample positions: inside blocks, on block/domain faces, outside."""
    x = rng.uniform(-1.2 * extent, 1.2 * extent, (nrows, npx, 3))
    x[:5, :, :] = rng.uniform(-3, 3, (5, npx, 3))           # near/inside horizon
    h = extent / 2.0
    faces = np.array([-extent, -h, 0.0, h, extent])
    x[5:15, :, 0] = rng.choice(faces, (10, npx))             # exactly on x faces
    x[15:20, :, 1] = rng.choice(faces, (5, npx))
    x[20:25, :, 2] = rng.choice(faces, (5, npx))
    S = np.zeros((nrows, npx, 8))
    S[..., 1:4] = x
    S[..., 0] = rng.uniform(-50, 0, (nrows, npx))
    k = rng.normal(size=(nrows, npx, 3))
    S[..., 5:8] = k
    S[..., 4] = 1.0 + rng.uniform(0, 0.5, (nrows, npx))
    return S


def gen_scalars():
    snap, model = _tiny_model()
    rng = np.random.Generator(np.random.PCG64(21))
    S = _scalar_points(rng, 120, 10, TINY["extent"], TINY["bhspin"])
    with np.errstate(all="ignore"):
        sc = model.get_fluid_scalars_from_geodesics(S.view(J))
        pr = model.get_prims_from_geodesics(S.view(J))
    out = dict(S=S)
    for k in ("dens", "u", "pitch_angle", "kdotu", "b"):
        out["sc_" + k] = np.asarray(sc[k])
    for k in ("dens", "u", "U1", "U2", "U3", "B1", "B2", "B3"):
        out["pr_" + k] = np.asarray(pr[k])
    _save("scalars", **out)


IMAGE_CASES = [
    # kwargs for make_image on the tiny snapshot
    dict(camera_inclination=60, camera_distance=1000, mass_scale=1e27,
         M_bh=6.2e9 * Msun, r_high=3, observing_frequency=230e9, fov=30,
         resolution=6, max_nsteps=1500),
    dict(camera_inclination=20, camera_distance=1000, mass_scale=3e26,
         M_bh=6.5e9 * Msun, r_high=10, observing_frequency=86e9, fov=36,
         resolution=5, max_nsteps=1500, max_chunk_bytes=4 * 20 * 1500 * 10),
]


def gen_image():
    snap, model = _tiny_model()
    out = {}
    for n, kw in enumerate(IMAGE_CASES):
        t0 = time.time()
        with np.errstate(all="ignore"):
            img = make_image(model, **kw)
        out[f"case{n}_image"] = np.asarray(img)
        out[f"case{n}_kw"] = np.array([kw["camera_inclination"], kw["camera_distance"],
                                       kw["mass_scale"], kw["M_bh"], kw["r_high"],
                                       kw["observing_frequency"], kw["fov"],
                                       kw["resolution"], kw["max_nsteps"]])
        print(f"image case {n} in {time.time()-t0:.1f}s, max {np.max(img):.4e}")
    out["fluid_gamma"] = np.array(model.fluid_gamma)
    _save("image", **out)


AMR_CASES = [
    # three levels: a root block refined, one of its children refined again
    dict(nblocks=2, cells_per_block=4, extent=8.0, refine=((0, 0, 0, 0), (1, 0, 0, 0)), seed=5),
    # two refined root blocks meeting at an edge
    dict(nblocks=2, cells_per_block=4, extent=8.0, refine=((0, 0, 0, 0), (0, 1, 1, 1)), seed=6),
]
AMR_IMAGE = dict(camera_inclination=50, camera_distance=1000, mass_scale=1e27, M_bh=6.2e9 * Msun, r_high=10,
                 observing_frequency=230e9, fov=14, resolution=5, max_nsteps=1500)


def _amr_model(case, fluid_gamma=13. / 9):
    from mahakala_gb300.grmhd.synthetic import make_multilevel_snapshot
    snap = make_multilevel_snapshot(**case)
    name = "amr_synthetic_%d.athdf" % case["seed"]
    datasets = dict(uov=snap.uov, B=snap.B, x1v=snap.x1v, x2v=snap.x2v, x3v=snap.x3v,
                    x1f=snap.x1f, x2f=snap.x2f, x3f=snap.x3f,
                    LogicalLocations=snap.LogicalLocations, Levels=snap.Levels)
    attrs = {"VariableNames": np.array([v.encode() for v in snap.VariableNames])}
    jaxshim.register_h5(name, datasets, attrs)
    return snap, AthenakFluidModel(name, snap.bhspin, fluid_gamma=fluid_gamma)


def gen_amr():
    """Multi-level meshes: the reference's ghost fill (athenak.py:67-525),
    its lookup + interpolation on sample points (:527-812) and one image."""
    out = {}
    rng = np.random.Generator(np.random.PCG64(77))
    for c, case in enumerate(AMR_CASES):
        snap, model = _amr_model(case)
        ext = case["extent"]
        S = _scalar_points(rng, 40, 10, ext, snap.bhspin)
        faces = np.array([-ext, -ext / 2, -ext / 4, 0.0, ext / 4, ext / 2, ext])  # faces of every level
        S[25:35, :, 0] = rng.choice(faces, (10, 10))
        S[25:35, :, 1] = rng.choice(faces, (10, 10))
        with np.errstate(all="ignore"):
            sc = model.get_fluid_scalars_from_geodesics(S.view(J))
            pr = model.get_prims_from_geodesics(S.view(J))
        p = f"case{c}_"
        for k in ("uov", "B", "x1v", "x2v", "x3v", "x1f", "x2f", "x3f", "LogicalLocations", "Levels"):
            out[p + k] = getattr(snap, k)
        out[p + "all_meshblocks"] = np.asarray(model.all_meshblocks)
        out[p + "S"] = S
        for k in ("dens", "u", "pitch_angle", "kdotu", "b"):
            out[p + "sc_" + k] = np.asarray(sc[k])
        for k in ("dens", "u", "U1", "U2", "U3", "B1", "B2", "B3"):
            out[p + "pr_" + k] = np.asarray(pr[k])
        if c == 0:
            with np.errstate(all="ignore"):
                out[p + "image"] = np.asarray(make_image(model, **AMR_IMAGE))
            out[p + "image_kw"] = np.array([AMR_IMAGE[k] for k in ("camera_inclination", "camera_distance",
                                                                   "mass_scale", "M_bh", "r_high",
                                                                   "observing_frequency", "fov", "resolution",
                                                                   "max_nsteps")])
    out["params"] = np.array([[case["nblocks"], case["cells_per_block"], case["extent"], case["seed"]]
                              for case in AMR_CASES])
    _save("amr", **out)


GENERATORS = dict(camera=gen_camera, integrator=gen_integrator, shadow=gen_shadow,
                  synchrotron=gen_synchrotron, electrons=gen_electrons,
                  transfer=gen_transfer, units=gen_units, snapshot=gen_snapshot,
                  scalars=gen_scalars, image=gen_image, amr=gen_amr)


if __name__ == "__main__":
    names = sys.argv[1:] or list(GENERATORS)
    for name in names:
        GENERATORS[name]()
