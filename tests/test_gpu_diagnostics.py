"""Per-step diagnostics from the fused FP64 render (images.step_diagnostics)
against the reference's stage-by-stage sequence run through this package's
stage kernels (images.py:56-144: geodesic_integrator, fluid scalars,
electrons, synchrotron, sigma cut), then solve_specific_intensity(dIs=True)
and solve_attenuated_emissivity (transfer.py:89-144) on both.

Bars (relative, floor 1e-6 of each array's maximum): dt rows within 1e-7
and zero at the same rows; emissivity and absorptivity within 1e-7 at
every row a ray reaches, zero beyond; dIs, the attenuated emissivity and
the image within 1e-7.  The two integrators agree to
~1e-13 per step (the fused kernel takes r from the metric evaluation, the
stage one from radius_cal); near the photon ring that difference grows
along the path, which the 1e-7 bar covers on this small case.
"""

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _stage_rows(model, kw):
    import mahakala_gb300 as ma
    from mahakala_gb300.electrons import rlow_rhigh_model
    a = model.bhspin
    s0 = ma.initialize_geodesics_at_camera(a, kw["camera_inclination"], 1000, -kw["fov"] / 2., kw["fov"] / 2.,
                                           kw["resolution"])
    S, dt = ma.geodesic_integrator(kw["max_nsteps"], s0, 40, 1e-4, a)
    fs = model.get_fluid_scalars_from_geodesics(S)
    bsq = fs["b"] * fs["b"]
    beta = fs["u"] * (model.fluid_gamma - 1.) / bsq / 0.5
    sigma = bsq / fs["dens"]
    theta = rlow_rhigh_model(fs["dens"], fs["u"], beta, r_high=kw["r_high"])
    units = model.get_units(kw["M_bh"], kw["mass_scale"])
    nu = kw["observing_frequency"]
    em, ab = ma.synchrotron_coefficients(units["Ne_unit"] * fs["dens"], theta, units["B_unit"] * fs["b"],
                                         fs["pitch_angle"], -fs["kdotu"] * nu, invariant=True, rescale_nu=1. / nu)
    cut = sigma > 100.
    em = em.masked_fill(cut, 0.)
    ab = ab.masked_fill(cut, 0.)
    return em, ab, dt, units["L_unit"]


def test_step_diagnostics_match_stage_sequence(cuda, tiny_arrays):
    from mahakala_gb300 import transfer
    from mahakala_gb300.grmhd.athenak import AthenakFluidModel
    from mahakala_gb300.images import step_diagnostics
    model = AthenakFluidModel(tiny_arrays, tiny_arrays.bhspin, fluid_gamma=13. / 9)
    kw = dict(camera_inclination=60, mass_scale=1e27, M_bh=6.2e9 * 1.989e33, r_high=3, observing_frequency=230e9,
              fov=30, resolution=12, max_nsteps=1500)
    d = step_diagnostics(model, **kw)
    em, ab, dt, L_unit = _stage_rows(model, kw)
    em, ab, dt = em.cpu().numpy(), ab.cpu().numpy(), dt.cpu().numpy()
    dem, dab, ddt = d["em"][0].cpu().numpy(), d["ab"][0].cpu().numpy(), d["dt"].cpu().numpy()
    assert dem.shape == em.shape and ddt.shape == dt.shape
    assert np.array_equal(ddt == 0, dt == 0)
    assert np.max(rel_err(ddt, dt, floor=1e-6 * np.abs(dt).max())) <= 1e-7
    K = d["nsteps"].reshape(-1).cpu().numpy()
    reached = np.arange(em.shape[0])[:, None] <= K[None, :]
    assert em.max() > 0
    for got, ref in ((dem, em), (dab, ab)):
        floor = 1e-6 * np.abs(ref).max()
        assert np.max(rel_err(got[reached], ref[reached], floor=floor)) <= 1e-7
        assert np.all(got[~reached] == 0.0)
    I_ref, dIs_ref = transfer.solve_specific_intensity(transfer_input(em), transfer_input(ab), transfer_input(dt),
                                                       L_unit, dIs=True)
    att_ref = transfer.solve_attenuated_emissivity(transfer_input(em), transfer_input(ab), transfer_input(dt),
                                                   L_unit).cpu().numpy()
    dIs_ref = dIs_ref.cpu().numpy()
    for got, ref in ((d["dIs"][0].cpu().numpy(), dIs_ref), (d["attenuated"][0].cpu().numpy(), att_ref)):
        assert got.shape == ref.shape
        assert np.max(rel_err(got, ref, floor=1e-6 * np.abs(ref).max())) <= 1e-7
    img = d["image"][0].cpu().numpy().reshape(-1)
    I_ref = I_ref.cpu().numpy()
    assert np.max(rel_err(img, I_ref, floor=1e-6 * np.abs(I_ref).max())) <= 1e-7


def transfer_input(a):
    import torch
    return torch.as_tensor(a, dtype=torch.float64, device="cuda")


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
