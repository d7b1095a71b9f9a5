"""Per-step diagnostics from the fused FP64 render (images.step_diagnostics)
against the oracle's stage-by-stage make_image sequence (images.py:56-120:
geodesic_integrator, get_fluid_scalars_from_geodesics, beta/sigma,
rlow_rhigh_model, units, synchrotron_coefficients, sigma cut), then
solve_specific_intensity(dIs=True) and solve_attenuated_emissivity
(transfer.py:89-144) on the oracle's rows.

Bar: 1e-8 relative (floor 1e-4 of each array's maximum) on every
well-conditioned entry of the dt, emissivity, absorptivity, dIs and
attenuated-emissivity rows and of the image, with the zero pattern of dt
identical.  An entry is ill-conditioned when the oracle's own pipeline run
from initial wavevectors changed by 1e-12 (oracle.perturbed) moves it by
more than 1e-10, or changes the ray's step count (then the whole ray is);
such entries must stay under 5 % of those compared.
"""

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

BAR = 1e-8
ILL = 1e-10
FLOOR = 1e-4


def _oracle_rows(orc, snap, a, kw, s0):
    """The oracle's em, ab, dt rows, dIs, attenuated emissivity and image of
    the rays s0, in the order make_image computes them."""
    S, dt = orc.geodesic_integrator(kw["max_nsteps"], s0, 40, 1e-4, a)
    fs = snap.get_fluid_scalars_from_geodesics(S)
    with np.errstate(all="ignore"):
        bsq = fs["b"] * fs["b"]
        beta = fs["u"] * (snap.fluid_gamma - 1.) / bsq / 0.5
        sigma = bsq / fs["dens"]
    theta = orc.rlow_rhigh_model(fs["dens"], fs["u"], beta, r_high=kw["r_high"])
    units = orc.get_units(kw["M_bh"], kw["mass_scale"])
    nu = kw["observing_frequency"]
    em, ab = orc.synchrotron_coefficients(units["Ne_unit"] * fs["dens"], theta, units["B_unit"] * fs["b"],
                                          fs["pitch_angle"], -fs["kdotu"] * nu, invariant=True, rescale_nu=1. / nu)
    cut = sigma > 100.
    em = np.where(cut, 0., em)
    ab = np.where(cut, 0., ab)
    I, dIs = orc.solve_specific_intensity(em, ab, dt, units["L_unit"], dIs=True)
    att = orc.solve_attenuated_emissivity(em, ab, dt, units["L_unit"])
    K = orc.integrate(s0, kw["max_nsteps"], 40, 1e-4, a)["K"]
    return dict(em=em, ab=ab, dt=dt, dIs=dIs, attenuated=att, image=I, K=K)


def _pad_rows(x, n):
    """x with rows appended (zeros) up to n rows; the two runs may trim to
    different lengths."""
    if x.shape[0] >= n:
        return x[:n]
    return np.concatenate([x, np.zeros((n - x.shape[0],) + x.shape[1:])], axis=0)


def test_step_diagnostics_match_oracle(cuda, orc, tiny_arrays):
    from mahakala_gb300.grmhd.athenak import AthenakFluidModel
    from mahakala_gb300.images import step_diagnostics
    model = AthenakFluidModel(tiny_arrays, tiny_arrays.bhspin, fluid_gamma=13. / 9)
    kw = dict(camera_inclination=60, mass_scale=1e27, M_bh=6.2e9 * 1.989e33, r_high=3, observing_frequency=230e9,
              fov=30, resolution=12, max_nsteps=1500)
    d = step_diagnostics(model, **kw)
    a = tiny_arrays.bhspin
    snap = orc.OracleSnapshot(tiny_arrays)
    s0 = orc.initialize_geodesics_at_camera(a, kw["camera_inclination"], 1000, -kw["fov"] / 2., kw["fov"] / 2.,
                                            kw["resolution"])
    ref = _oracle_rows(orc, snap, a, kw, s0)
    pert = _oracle_rows(orc, snap, a, kw, orc.perturbed(s0))
    got = dict(em=d["em"][0].cpu().numpy(), ab=d["ab"][0].cpu().numpy(), dt=d["dt"].cpu().numpy(),
               dIs=d["dIs"][0].cpu().numpy(), attenuated=d["attenuated"][0].cpu().numpy(),
               image=d["image"][0].cpu().numpy().reshape(-1))
    K = d["nsteps"].reshape(-1).cpu().numpy()
    assert ref["em"].max() > 0
    # both runs keep max(K) + 2 rows (geodesics.py:275-281); only an
    # ill-conditioned ray can make the two lengths differ
    nrows = ref["em"].shape[0]
    for key in ("dt", "em", "ab", "dIs", "attenuated"):
        got[key] = _pad_rows(got[key], ref[key].shape[0])
    ray_ill = pert["K"] != ref["K"]
    assert np.array_equal(K[~ray_ill], ref["K"][~ray_ill])
    assert np.array_equal(got["dt"][:, ~ray_ill] == 0, ref["dt"][:, ~ray_ill] == 0)
    # rows the ray reached (later rows: the reference repeats the frozen
    # state's sample with dt = 0, the fused kernel leaves zeros; the
    # transfer weighs both by dt = 0)
    reached = np.arange(nrows)[:, None] <= ref["K"][None, :]
    compared, ill_total = 0, 0
    for key in ("dt", "em", "ab", "dIs", "attenuated", "image"):
        g, r = got[key], ref[key]
        p = _pad_rows(pert[key], r.shape[0]) if key != "image" else pert[key]
        floor = FLOOR * np.abs(r).max()
        ill = (rel_err(p, r, floor=floor) > ILL) | ray_ill
        if key in ("em", "ab"):
            mask = reached & ~ill
            ill = ill & reached
        else:
            mask = ~ill
        err = rel_err(g, r, floor=floor)
        assert np.max(err[mask], initial=0.0) <= BAR, (key, float(np.max(err[mask])))
        compared += mask.sum() + ill.sum()
        ill_total += ill.sum()
        if key in ("em", "ab"):
            assert np.all(g[~reached] == 0.0), key
    assert ill_total < 0.05 * compared, f"{ill_total} of {compared} entries ill-conditioned"


def test_step_diagnostics_multifrequency_rows_and_fp64_only(cuda, tiny_arrays):
    from mahakala_gb300.grmhd.athenak import AthenakFluidModel
    from mahakala_gb300.images import PreparedRender, RenderRequest, step_diagnostics
    model = AthenakFluidModel(tiny_arrays, tiny_arrays.bhspin, fluid_gamma=13. / 9)
    kw = dict(camera_inclination=25, mass_scale=3e26, r_high=10, fov=36, resolution=9, max_nsteps=1200)
    d = step_diagnostics(model, observing_frequency=[86e9, 345e9], **kw)
    for c, nu in enumerate((86e9, 345e9)):
        one = step_diagnostics(model, observing_frequency=nu, **kw)
        assert np.array_equal(d["em"][c].cpu().numpy(), one["em"][0].cpu().numpy())
        assert np.array_equal(d["attenuated"][c].cpu().numpy(), one["attenuated"][0].cpu().numpy())
    with pytest.raises(ValueError):
        PreparedRender([RenderRequest(model, rows=100, **kw)], precision="mixed")
