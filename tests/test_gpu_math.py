"""The FP64 path's own reciprocal square root, reciprocal and square root
(mk_probe_math: a float-unit seed refined by one third-order correction in
binary64) against the library's correctly rounded forms on the GPU.

Bar: within 2 ulp over 1e6 log-uniform arguments spanning 2^-125..2^125 --
the seeded range 2^-120..2^119 and the library fallback on either side --
and bit-identical (NaN for NaN) on zero, subnormals, negative values,
infinities and NaN.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(fn, x):
    import torch

    from mahakala_gb300 import _lib
    xd = torch.as_tensor(x, dtype=torch.float64, device="cuda")
    out = torch.empty_like(xd)
    _lib.call("mk_probe_math", fn, xd.data_ptr(), xd.numel(), out.data_ptr(),
              torch.cuda.current_stream().cuda_stream)
    return out.cpu().numpy()


def _ulp_err(a, b):
    # distance in units of the reference's last place
    with np.errstate(all="ignore"):
        return np.abs(a - b) / np.spacing(np.abs(b))


@pytest.mark.parametrize("fn,lib_fn,sign", [("RSQRT", "LIB_RSQRT", 1.0), ("RCP", "LIB_RCP", 1.0),
                                            ("RCP", "LIB_RCP", -1.0), ("SQRT", "LIB_SQRT", 1.0)])
def test_fp64_math_within_two_ulp(cuda, fn, lib_fn, sign):
    from mahakala_gb300 import _lib
    rng = np.random.Generator(np.random.PCG64(7))
    x = sign * np.exp2(rng.uniform(-125.0, 125.0, 1_000_000))
    got = _run(getattr(_lib, "MK_MATH_" + fn), x)
    ref = _run(getattr(_lib, "MK_MATH_" + lib_fn), x)
    err = _ulp_err(got, ref)
    assert np.all(np.isfinite(got))
    assert err.max() <= 2.0, (fn, float(err.max()), x[np.argmax(err)])


@pytest.mark.parametrize("fn,lib_fn", [("RSQRT", "LIB_RSQRT"), ("RCP", "LIB_RCP"), ("SQRT", "LIB_SQRT")])
def test_fp64_math_special_values_match_library(cuda, fn, lib_fn):
    from mahakala_gb300 import _lib
    x = np.array([0.0, -0.0, 5e-324, 1e-310, -1.0, -2.5e-300, np.inf, -np.inf, np.nan, 2.0 ** -121, 2.0 ** 120,
                  2.0 ** -120, 2.0 ** 119 * 1.999])
    got = _run(getattr(_lib, "MK_MATH_" + fn), x)
    ref = _run(getattr(_lib, "MK_MATH_" + lib_fn), x)
    same = (got == ref) | (np.isnan(got) & np.isnan(ref))
    edge = np.abs(_ulp_err(got, ref)) <= 2.0  # the two seeded end points
    assert np.all(same | edge), list(zip(x, got, ref))
    assert np.all(same[:9]), list(zip(x[:9], got[:9], ref[:9]))
