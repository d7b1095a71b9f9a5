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


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_strict"])
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
    from mahakala_gb300 import _lib
    from mahakala_gb300.images import PreparedRender, RenderRequest

    prep = PreparedRender([RenderRequest(_model(tiny_arrays), resolution=4, fov=30, max_nsteps=100)],
                          precision="mixed")
    too_many = _lib.NOALLOC_MAX_MIXED_RAYS + 1
    with pytest.raises(_lib.MKError) as e:
        _lib.call("mk_render_noalloc", prep.reqs_dev.data_ptr(), 1, too_many, prep.snaps_dev.data_ptr(), 1,
                  _lib.MK_MIXED, None)
    assert e.value.code == _lib.MK_ERR_LIMIT
    assert "static workspace" in str(e.value)
