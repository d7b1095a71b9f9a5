"""Multi-level (refined) meshes on the device against the reference's own
outputs (tests/golden/amr.npz, produced by executing the reference's loader
and sampler) and against the oracle.

Bars: ghost-filled blocks bit-exact (float32 storage = the reference's
float64 values rounded once; the binary64 copies of blocks with
fine-to-coarse ghosts bit-exact); sampled primitives bit-exact and block
ids identical on every golden point (inside blocks, on faces of every
level, outside); fluid scalars 1e-13 (pitch angle 1e-12 absolute); the FP64
render within 1e-8 of the oracle and of the reference image; the mixed
form within its 1e-2 / 1e-3 bars.
"""

import numpy as np
import pytest

from conftest import amr_arrays, golden, rel_err

pytestmark = pytest.mark.gpu


def _model(case):
    from mahakala_gb300.grmhd.athenak import AthenakFluidModel
    return AthenakFluidModel(amr_arrays(case), 0.94, fluid_gamma=13. / 9)


@pytest.mark.parametrize("case", [0, 1])
def test_multilevel_ghost_fill_matches_reference(cuda, case):
    d = golden("amr")
    ref = d[f"case{case}_all_meshblocks"].transpose(0, 2, 3, 4, 1)   # -> (mb, k, j, i, prim)
    snap = _model(case).snapshot
    got = snap.blocks().cpu().numpy()
    assert np.array_equal(got, ref.astype(np.float32))
    assert snap.n64 > 0
    b64 = snap.blocks64.cpu().numpy()
    rows = snap.block64.cpu().numpy()
    for mb in range(snap.nmb):
        if rows[mb] >= 0:
            assert np.array_equal(b64[rows[mb]], ref[mb]), mb
        else:  # every value of a block without a binary64 copy is a float32 value
            assert np.array_equal(ref[mb].astype(np.float32).astype(np.float64), ref[mb]), mb


@pytest.mark.parametrize("case", [0, 1])
def test_multilevel_sampling_matches_reference(cuda, case):
    d = golden("amr")
    p = f"case{case}_"
    model = _model(case)
    pr = model.get_prims_from_geodesics(d[p + "S"])
    sc = model.get_fluid_scalars_from_geodesics(d[p + "S"])
    for k in ("dens", "u", "U1", "U2", "U3", "B1", "B2", "B3"):
        assert np.array_equal(pr[k].cpu().numpy(), d[p + "pr_" + k]), k
    for k in ("dens", "u", "kdotu", "b"):
        g = sc[k].cpu().numpy()
        assert np.array_equal(np.isnan(g), np.isnan(d[p + "sc_" + k])), k
        assert np.nanmax(rel_err(g, d[p + "sc_" + k])) < 1e-13, k
    assert np.nanmax(np.abs(sc["pitch_angle"].cpu().numpy() - d[p + "sc_pitch_angle"])) < 1e-12


def test_multilevel_block_lookup_equals_scan(cuda, orc):
    """Block ids of the device lookup equal the literal last-match scan on
    points exactly on the faces of every level."""
    import torch
    from mahakala_gb300 import _lib
    arrs = amr_arrays(0)
    model = _model(0)
    rng = np.random.Generator(np.random.PCG64(3))
    faces = np.unique(np.concatenate([arrs.x1f.ravel(), arrs.x2f.ravel()]))
    S = np.zeros((4000, 8))
    S[:, 1:4] = rng.uniform(-9, 9, (4000, 3))
    S[:2000, 1] = rng.choice(faces, 2000)
    S[1000:3000, 2] = rng.choice(faces, 2000)
    S[:, 4] = 1.0
    Sd = torch.as_tensor(S, device="cuda")
    out = torch.empty((4000, 8), dtype=torch.float64, device="cuda")
    blk = torch.empty(4000, dtype=torch.int32, device="cuda")
    _lib.call("mk_fluid_prims", _lib.ctypes.byref(model.snapshot.view), Sd.data_ptr(), 4000, out.data_ptr(),
              blk.data_ptr(), None)
    ref = orc.OracleSnapshot(arrs).get_prims_from_geodesics(S)["block"]
    assert np.array_equal(blk.cpu().numpy(), ref)
    assert (ref >= 0).sum() > 2000 and (ref == -1).sum() > 100


def test_multilevel_render_matches_oracle_and_reference(cuda, orc):
    from mahakala_gb300 import metrics
    from mahakala_gb300.images import make_image
    d = golden("amr")
    inc, dist, ms, M, rh, nu, fov, res, N = d["case0_image_kw"]
    kw = dict(camera_inclination=inc, camera_distance=dist, mass_scale=ms, M_bh=M, r_high=rh,
              observing_frequency=nu, fov=fov, max_nsteps=int(N))
    model = _model(0)
    img = make_image(model, resolution=int(res), **kw)
    ref = d["case0_image"]
    assert np.max(np.abs(img - ref)) / np.max(np.abs(ref)) < 1e-8
    # a larger image against the oracle, FP64 and mixed
    big = make_image(model, resolution=24, **kw)
    o = orc.make_image(orc.OracleSnapshot(amr_arrays(0)), resolution=24, **kw)
    assert o.max() > 0
    assert np.max(rel_err(big, o, floor=1e-4 * o.max())) < 1e-8
    mixed = make_image(model, resolution=24, precision="mixed", **kw)
    assert metrics.flux_rel_err(mixed, o) <= 1e-3
    assert metrics.max_pixel_rel_err(mixed, o) <= 1e-2
