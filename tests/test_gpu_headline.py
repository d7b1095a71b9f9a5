"""The benchmark's headline image against the oracle: the 256x256 render of
the seeded 256^3-cell snapshot (16^3 meshblocks of 16^3 cells over
[-50, 50]^3 M; a=0.94, 17 deg, +-25 M, 230 GHz, R_high 40, <= 8192 steps),
make_image (images.py:30-144).

The whole image is rendered on the GPU in FP64 and in the mixed form; the
oracle renders every 4th pixel in x and y (4,096 rays) of the same camera
over the full snapshot.  FP64 bar (oracle.image_parity): on well-
conditioned rays -- those a 1e-12 change of the initial wavevector moves
by less than 1e-10 -- equal step counts, every pixel within 1e-8 relative
(floor 1e-4 of the maximum) and the summed flux within 1e-8; fewer than 5 %
of the rays ill-conditioned.  Mixed bar, against the oracle directly:
flux within 1e-3 and every pixel within 1e-2.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STRIDE = 4


@pytest.fixture(scope="module")
def headline(cuda, orc):
    from mahakala_gb300 import configs
    from mahakala_gb300.grmhd.athenak import AthenakFluidModel
    spec = configs.RENDER_256
    arrays = spec.snapshot.build()
    model = AthenakFluidModel(arrays, spec.snapshot.bhspin, fluid_gamma=spec.snapshot.fluid_gamma)
    res = spec.resolution
    ix, iy = np.meshgrid(np.arange(0, res, STRIDE), np.arange(0, res, STRIDE), indexing="ij")
    pix = (ix * res + iy).reshape(-1)
    s0 = orc.initialize_geodesics_at_camera(spec.bhspin, spec.inclination, spec.camera_distance, -spec.half_fov,
                                            spec.half_fov, res)[pix]
    snap = orc.OracleSnapshot(arrays)
    args = (spec.mass_scale, spec.M_bh, spec.r_high, list(spec.freqs), spec.max_nsteps, spec.r_low)
    oimg, osteps = orc.render_rays(snap, s0, *args)
    pimg, psteps = orc.render_rays(snap, orc.perturbed(s0), *args)
    return dict(spec=spec, model=model, pix=pix, oimg=oimg, osteps=osteps, pimg=pimg, psteps=psteps)


def _render(h, precision):
    from mahakala_gb300.images import PreparedRender
    req = h["spec"].request(h["model"])
    prep = PreparedRender([req], precision=precision, with_steps=True)
    prep.launch()
    img = prep.images[0].reshape(1, -1)[:, h["pix"]].cpu().numpy()
    steps = req.out["nsteps"].reshape(-1)[h["pix"]].cpu().numpy()
    return img, steps


def test_headline_fp64_image_matches_oracle(headline, orc):
    h = headline
    img, steps = _render(h, "fp64")
    assert h["oimg"].max() > 0
    rep = orc.image_parity(img, steps, h["oimg"], h["osteps"], h["pimg"], h["psteps"])
    print("headline fp64 vs oracle:", rep)
    assert rep["ill_conditioned"] < 0.05 * rep["rays"], rep
    assert rep["steps_equal"], rep
    assert rep["max_pixel_rel_err"] <= 1e-8, rep
    assert rep["flux_rel_err"] <= 1e-8, rep
    assert rep["ok"]


def test_headline_mixed_image_within_bars_of_oracle(headline):
    from mahakala_gb300 import metrics
    h = headline
    img, _ = _render(h, "mixed")
    assert np.all(np.isfinite(img))
    pix_err = metrics.max_pixel_rel_err(img[0], h["oimg"][0])
    flux_err = metrics.flux_rel_err(img[0], h["oimg"][0])
    print(f"headline mixed vs oracle: pixel {pix_err:.3e}, flux {flux_err:.3e}")
    assert pix_err <= 1e-2
    assert flux_err <= 1e-3
