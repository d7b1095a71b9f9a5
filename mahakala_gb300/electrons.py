"""Electron temperature model (mahakala/electrons.py), same call surface."""

import torch

from . import _lib
from ._device import device, f64, ptr, stream_ptr
from .constants import CL, ME, MP  # noqa: F401  (kept beside the model as in the reference)

__all__ = ["rlow_rhigh_model"]


def rlow_rhigh_model(dens, u, beta, r_low=1, r_high=40, electron_gamma=4. / 3, ion_gamma=5. / 3):
    """electrons.py:32-50 -> dimensionless electron temperature Theta_e."""
    dev = device()
    ts = [t.contiguous() for t in torch.broadcast_tensors(f64(dens, dev), f64(u, dev), f64(beta, dev))]
    out = torch.empty_like(ts[0])
    _lib.call("mk_rlow_rhigh", ptr(ts[0]), ptr(ts[1]), ptr(ts[2]), ts[0].numel(), float(r_low), float(r_high),
              float(electron_gamma - 1.), float(ion_gamma - 1.), ptr(out), stream_ptr())
    return out
