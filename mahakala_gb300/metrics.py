"""Image comparison metrics for the mixed-precision form against FP64.

* max per-pixel relative error, with the floor max(|I_ref|, floor_frac *
  max I_ref) so that near-empty pixels do not dominate (floor_frac 1e-4);
* total-flux relative error (sum over pixels, the flux up to a constant);
* shadow diameter 2 sqrt(A / pi) from the area A of the captured-ray mask
  (ray status MK_RAY_CAPTURED), in the camera's length units.
"""

import numpy as np

from . import _lib

PIXEL_FLOOR = 1e-4


def _np(x):
    try:
        import torch
        if isinstance(x, torch.Tensor):
            return x.detach().cpu().numpy()
    except ImportError:  # pragma: no cover
        pass
    return np.asarray(x)


def max_pixel_rel_err(img, ref, floor_frac=PIXEL_FLOOR):
    img, ref = _np(img).astype(np.float64), _np(ref).astype(np.float64)
    den = np.maximum(np.abs(ref), floor_frac * np.max(np.abs(ref)))
    with np.errstate(all="ignore"):
        e = np.abs(img - ref) / np.where(den > 0, den, 1.0)
    return float(np.max(np.where(img == ref, 0.0, e)))


def flux_rel_err(img, ref):
    img, ref = _np(img).astype(np.float64), _np(ref).astype(np.float64)
    s = ref.sum()
    return float(abs(img.sum() - s) / abs(s)) if s != 0 else float(abs(img.sum()))


def shadow_diameter(status, fov):
    """2 sqrt(A/pi) of the captured-ray region of a (res, res) status map."""
    st = _np(status)
    res = st.shape[-1]
    area = np.count_nonzero(st == _lib.MK_RAY_CAPTURED) * (fov / res) ** 2
    return float(2.0 * np.sqrt(area / np.pi))


def compare(img, ref, status=None, ref_status=None, fov=None):
    out = dict(max_pixel_rel_err=max_pixel_rel_err(img, ref), flux_rel_err=flux_rel_err(img, ref))
    if status is not None and ref_status is not None and fov is not None:
        d, d0 = shadow_diameter(status, fov), shadow_diameter(ref_status, fov)
        out.update(shadow_diameter=d, shadow_diameter_fp64=d0,
                   shadow_diameter_rel_err=abs(d - d0) / d0 if d0 else float(d != d0))
    return out
