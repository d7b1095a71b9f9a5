"""Fused render kernel (mk_render) against the reference's make_image golden
images and the oracle.

Tolerance: 1e-8 relative per pixel (floor 1e-4 of the image maximum for
near-empty pixels), the FP64 parity bar, on every well-conditioned pixel.
A pixel is ill-conditioned when the oracle's own intensity or step count
moves under a 1e-12 change of the ray's initial wavevector (a ray grazing
the photon ring, where the closed-form and the autodiff Christoffel
symbols round differently and the orbit amplifies it); those are counted
and must stay a small fraction.
"""

import numpy as np
import pytest

from conftest import golden, rel_err

pytestmark = pytest.mark.gpu

PIX_TOL = 1e-8


def _model(arrs, fluid_gamma=13. / 9):
    from mahakala_gb300.grmhd.athenak import AthenakFluidModel
    return AthenakFluidModel(arrs, arrs.bhspin, fluid_gamma=fluid_gamma)


def test_make_image_matches_reference_golden(cuda, tiny_arrays):
    from mahakala_gb300.images import make_image
    d = golden("image")
    model = _model(tiny_arrays, float(d["fluid_gamma"]))
    for n in range(2):
        inc, dist, ms, M, rh, nu, fov, res, N = d[f"case{n}_kw"]
        img = make_image(model, camera_inclination=inc, camera_distance=dist, mass_scale=ms, M_bh=M, r_high=rh,
                         observing_frequency=nu, fov=fov, resolution=int(res), max_nsteps=int(N))
        ref = d[f"case{n}_image"]
        assert img.shape == ref.shape
        assert np.max(rel_err(img, ref, floor=1e-4 * ref.max())) < PIX_TOL, n


def _medium():
    from mahakala_gb300.grmhd.synthetic import make_synthetic_snapshot
    return make_synthetic_snapshot(nblocks=4, cells_per_block=16, extent=50.0, bhspin=0.94, seed=11)


@pytest.fixture(scope="module")
def medium():
    return _medium()


@pytest.mark.parametrize("inc,rh,nu", [(17.0, 40.0, 230e9), (60.0, 10.0, 86e9), (85.0, 1.0, 345e9)])
def test_render_matches_oracle(cuda, orc, medium, inc, rh, nu):
    from mahakala_gb300.images import RenderRequest, render_requests
    model = _model(medium)
    kw = dict(camera_inclination=inc, camera_distance=1000, mass_scale=3e26, M_bh=6.5e9 * 1.989e33, r_high=rh,
              observing_frequency=nu, fov=50.0, resolution=32, max_nsteps=3000)
    req = RenderRequest(model, **kw)
    img = render_requests([req], with_steps=True)[0][0].cpu().numpy()
    steps = req.out["nsteps"].cpu().numpy()
    osnap = orc.OracleSnapshot(medium)
    oimg, osteps = orc.make_image(osnap, return_steps=True, **kw)
    assert oimg.max() > 0
    s0 = orc.initialize_geodesics_at_camera(medium.bhspin, inc, 1000, -25.0, 25.0, 32)
    rkw = dict(mass_scale=kw["mass_scale"], M_bh=kw["M_bh"], r_high=rh, observing_frequency=nu, max_nsteps=3000)
    pimg, psteps = orc.render_rays(osnap, orc.perturbed(s0), **rkw)
    pimg, psteps = pimg.reshape(32, 32), psteps.reshape(32, 32)
    floor = 1e-4 * oimg.max()
    ill = (psteps != osteps) | (rel_err(pimg, oimg, floor=floor) > 1e-10)
    assert ill.mean() < 0.05, f"{ill.sum()} ill-conditioned pixels"
    ok = ~ill
    assert np.array_equal(steps[ok], osteps[ok])
    err = rel_err(img, oimg, floor=floor)
    assert np.max(err[ok]) < PIX_TOL
    assert abs(img[ok].sum() - oimg[ok].sum()) / oimg[ok].sum() < 1e-8


def test_multifrequency_pass_equals_single(cuda, medium):
    """One ray pass at three frequencies equals three single renders."""
    from mahakala_gb300.images import make_image
    model = _model(medium)
    kw = dict(camera_inclination=60, mass_scale=3e26, fov=50.0, resolution=24, max_nsteps=3000)
    multi = make_image(model, observing_frequency=[86e9, 230e9, 345e9], **kw)
    for c, nu in enumerate((86e9, 230e9, 345e9)):
        single = make_image(model, observing_frequency=nu, **kw)
        assert np.array_equal(multi[c], single)


def test_batched_requests_equal_isolated(cuda, medium, tiny_arrays):
    """Requests of different sizes, spins and snapshots packed into one
    launch give exactly the images each gives alone."""
    from mahakala_gb300.images import RenderRequest, render_requests
    m1 = _model(medium)
    m2 = _model(tiny_arrays)
    reqs = [RenderRequest(m1, camera_inclination=30, resolution=16, fov=50.0, max_nsteps=2000),
            RenderRequest(m2, camera_inclination=70, resolution=7, fov=30.0, r_high=5, max_nsteps=1500,
                          mass_scale=1e27),
            RenderRequest(m1, camera_inclination=80, resolution=20, fov=40.0, bhspin=0.5,
                          observing_frequency=[86e9, 345e9], max_nsteps=2000)]
    together = [t.cpu().numpy() for t in render_requests(reqs)]
    for r, t in zip(reqs, together):
        alone = render_requests([RenderRequest(**{k: getattr(r, k) for k in (
            "model", "camera_inclination", "camera_distance", "mass_scale", "M_bh", "r_high",
            "observing_frequency", "fov", "resolution", "max_nsteps", "r_low", "bhspin")})])[0].cpu().numpy()
        assert np.array_equal(t, alone)


def test_render_rejects_missing_fluid_gamma(cuda, tiny_arrays):
    from mahakala_gb300.images import make_image
    model = _model(tiny_arrays, fluid_gamma=None)
    with pytest.raises(TypeError):
        make_image(model, resolution=4)


@pytest.mark.parametrize("res", [1, 2, 3])
def test_tiny_images_every_form(cuda, orc, tiny_arrays, res):
    """1x1, 2x2 and 3x3 images -- a single ray and warps with 1, 4 or 9 live
    lanes of 32: the FP64 form within the parity bar of the oracle, the
    mixed forms within their bars of the FP64 image."""
    from mahakala_gb300 import metrics
    from mahakala_gb300.grmhd.athenak import AthenakFluidModel
    from mahakala_gb300.images import make_image
    model = AthenakFluidModel(tiny_arrays, tiny_arrays.bhspin, fluid_gamma=13. / 9)
    kw = dict(camera_inclination=60, mass_scale=1e27, r_high=3, fov=30, resolution=res, max_nsteps=2000)
    img = make_image(model, **kw)
    o = orc.make_image(orc.OracleSnapshot(tiny_arrays), **kw)
    assert img.shape == o.shape == (res, res)
    assert np.max(rel_err(img, o, floor=1e-4 * max(np.abs(o).max(), 1e-300))) < 1e-8
    for form in ("mixed", "mixed_strict", "mixed_df"):
        mixed = make_image(model, precision=form, **kw)
        assert np.all(np.isfinite(mixed))
        assert metrics.max_pixel_rel_err(mixed, img) <= 1e-2, form
        assert metrics.flux_rel_err(mixed, img) <= 1e-3, form


def test_render_of_zero_rays_is_a_no_op(cuda, tiny_arrays):
    """total_rays = 0: mk_render returns MK_OK and writes no image."""
    import torch

    from mahakala_gb300 import _lib
    from mahakala_gb300._device import ptr, stream_ptr
    from mahakala_gb300.grmhd.athenak import AthenakFluidModel
    from mahakala_gb300.images import PreparedRender, RenderRequest
    model = AthenakFluidModel(tiny_arrays, tiny_arrays.bhspin, fluid_gamma=13. / 9)
    for form in ("fp64", "mixed"):
        prep = PreparedRender([RenderRequest(model, resolution=4, fov=30)], precision=form)
        prep.images[0].fill_(-7.0)
        _lib.call("mk_render", ptr(prep.reqs_dev), 1, 0, ptr(prep.snaps_dev), prep.nsnap, prep.precision,
                  ptr(prep.ws), prep.ws.numel() * 8, stream_ptr(None))
        torch.cuda.synchronize()
        assert bool((prep.images[0] == -7.0).all()), form


def test_render_from_athdf_path_equals_arrays(cuda, tiny_arrays, tmp_path):
    """AthenakFluidModel(path) -- the reference's call, the file read by the
    package's own HDF5 reader -- renders the image the same arrays give,
    bit for bit, in FP64 and in the mixed form."""
    from mahakala_gb300.grmhd.athenak import AthenakFluidModel
    from mahakala_gb300.grmhd.hdf5 import write_athdf
    from mahakala_gb300.images import make_image
    path = str(tmp_path / "tiny.athdf")
    write_athdf(path, tiny_arrays, chunk_blocks=True, deflate=True)
    from_file = AthenakFluidModel(path, tiny_arrays.bhspin, fluid_gamma=13. / 9)
    from_arrays = AthenakFluidModel(tiny_arrays, tiny_arrays.bhspin, fluid_gamma=13. / 9)
    kw = dict(camera_inclination=60, mass_scale=1e27, r_high=3, fov=30, resolution=16, max_nsteps=1500)
    for form in ("fp64", "mixed"):
        a = make_image(from_file, precision=form, **kw)
        b = make_image(from_arrays, precision=form, **kw)
        assert b.max() > 0 and np.array_equal(a, b), form
