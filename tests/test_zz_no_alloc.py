"""mk_render_noalloc: the render entry point for callers that cannot hand
this library device memory (its scratch is a static device array).

Called through the C ABI; its images must equal those of mk_render with a
caller workspace (same kernels; the parity tolerance of the render tests,
1e-8 relative, is the bar, and equality is expected), on two calls in a
row -- the static array keeps the previous call's contents, so the second
call checks that everything that must start at zero is cleared.  Collected
last (file name), so a stop at the first failure has run every other test.
"""

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _model(arrs):
    from mahakala_gb300.grmhd.athenak import AthenakFluidModel
    return AthenakFluidModel(arrs, arrs.bhspin, fluid_gamma=13. / 9)


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_strict", "mixed_df"])
def test_noalloc_matches_workspace_render(cuda, tiny_arrays, precision):
    import torch

    from mahakala_gb300 import _lib
    from mahakala_gb300.images import PRECISIONS, PreparedRender, RenderRequest

    model = _model(tiny_arrays)
    kws = [dict(camera_inclination=60, mass_scale=1e27, r_high=3, fov=30, resolution=12, max_nsteps=1500),
           dict(camera_inclination=25, mass_scale=3e26, r_high=10, fov=36, resolution=9, max_nsteps=1500,
                observing_frequency=[86e9, 345e9])]
    ref = PreparedRender([RenderRequest(model, **k) for k in kws], precision=precision)
    ref.launch()
    expected = [img.cpu().numpy() for img in ref.images]

    out = PreparedRender([RenderRequest(model, **k) for k in kws], precision=precision)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        for img in out.images:
            img.fill_(np.nan)
        _lib.call("mk_render_noalloc", out.reqs_dev.data_ptr(), len(out.requests), out.total_rays,
                  out.snaps_dev.data_ptr(), out.nsnap, PRECISIONS[precision], stream)
        torch.cuda.synchronize()
        for got, exp in zip(out.images, expected):
            g = got.cpu().numpy()
            assert np.all(np.isfinite(g)), f"call {call}: unwritten pixels"
            assert np.max(rel_err(g, exp, floor=1e-4 * np.abs(exp).max())) <= 1e-8, f"call {call}"


def test_noalloc_rejects_jobs_beyond_its_static_workspace(cuda, tiny_arrays):
    """A mixed-form job of one 229x229 request, 52,441 rays (above the
    52,428-ray limit of the static array), is refused before any launch; the
    request's pixels really add up to the ray total, so even a regressed
    check would render in bounds."""
    from mahakala_gb300 import _lib
    from mahakala_gb300.images import PreparedRender, RenderRequest

    prep = PreparedRender([RenderRequest(_model(tiny_arrays), resolution=229, fov=30, max_nsteps=100)],
                          precision="fp64")
    assert prep.total_rays == 229 * 229 > _lib.NOALLOC_MAX_MIXED_RAYS
    with pytest.raises(_lib.MKError) as e:
        _lib.call("mk_render_noalloc", prep.reqs_dev.data_ptr(), 1, prep.total_rays, prep.snaps_dev.data_ptr(), 1,
                  _lib.MK_MIXED, None)
    assert e.value.code == _lib.MK_ERR_LIMIT
    assert "static workspace" in str(e.value)


def test_noalloc_takes_the_documented_maximum(cuda, tiny_arrays):
    """Exactly MK_NOALLOC_MAX_MIXED_RAYS rays in the mixed form (three
    requests of 226^2 + 34^2 + 14^2 = 52,428 pixels) are accepted and render
    the images mk_render gives with a caller workspace."""
    import torch

    from mahakala_gb300 import _lib
    from mahakala_gb300.images import PRECISIONS, PreparedRender, RenderRequest

    model = _model(tiny_arrays)
    kws = [dict(resolution=226, fov=30, max_nsteps=400, camera_inclination=60, mass_scale=1e27, r_high=3),
           dict(resolution=34, fov=24, max_nsteps=400, camera_inclination=30, mass_scale=1e27, r_high=3),
           dict(resolution=14, fov=36, max_nsteps=400, camera_inclination=80, mass_scale=1e27, r_high=3)]
    ref = PreparedRender([RenderRequest(model, **k) for k in kws], precision="mixed")
    assert ref.total_rays == _lib.NOALLOC_MAX_MIXED_RAYS
    ref.launch()
    expected = [img.cpu().numpy() for img in ref.images]
    out = PreparedRender([RenderRequest(model, **k) for k in kws], precision="mixed")
    for img in out.images:
        img.fill_(np.nan)
    _lib.call("mk_render_noalloc", out.reqs_dev.data_ptr(), len(out.requests), out.total_rays,
              out.snaps_dev.data_ptr(), out.nsnap, PRECISIONS["mixed"], torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    for got, exp in zip(out.images, expected):
        g = got.cpu().numpy()
        assert np.all(np.isfinite(g))
        assert np.max(rel_err(g, exp, floor=1e-4 * np.abs(exp).max())) <= 1e-8
