"""Synchrotron coefficients and the transfer solve (mahakala/transfer.py),
same call surface; float64 CUDA tensors in and out."""

import torch

from . import _lib
from ._device import device, f64, ptr, stream_ptr

__all__ = ["synchrotron_coefficients", "solve_specific_intensity", "solve_attenuated_emissivity"]


def synchrotron_coefficients(Ne, Theta_e, B, pitch_angle, nu, invariant=True, rescale_nu=1.):
    """transfer.py:30-86 -> (emissivity, absorptivity)."""
    dev = device()
    ts = torch.broadcast_tensors(*[f64(v, dev) for v in (Ne, Theta_e, B, pitch_angle, nu)])
    ts = [t.contiguous() for t in ts]
    em = torch.empty_like(ts[0])
    ab = torch.empty_like(ts[0])
    _lib.call("mk_synchrotron", *[ptr(t) for t in ts], ts[0].numel(), int(bool(invariant)), float(rescale_nu),
              ptr(em), ptr(ab), stream_ptr())
    return em, ab


def solve_specific_intensity(emissivity, absorptivity, dt, L_unit, dIs=False):
    """transfer.py:89-119 on (nsteps, npx) arrays."""
    dev = device()
    em, ab, d = f64(emissivity, dev), f64(absorptivity, dev), f64(dt, dev)
    nsteps, npx = em.shape
    I = torch.empty(npx, dtype=torch.float64, device=dev)
    dI = torch.empty((max(nsteps - 1, 0), npx), dtype=torch.float64, device=dev) if dIs else None
    _lib.call("mk_solve_intensity", ptr(em), ptr(ab), ptr(d), nsteps, npx, float(L_unit), ptr(I), ptr(dI),
              stream_ptr())
    return (I, dI) if dIs else I


def solve_attenuated_emissivity(emissivity, absorptivity, dt, L_unit):
    """transfer.py:122-144 -> (nsteps-1, npx)."""
    dev = device()
    em, ab, d = f64(emissivity, dev), f64(absorptivity, dev), f64(dt, dev)
    nsteps, npx = em.shape
    out = torch.zeros((max(nsteps - 1, 0), npx), dtype=torch.float64, device=dev)
    _lib.call("mk_attenuated_emissivity", ptr(em), ptr(ab), ptr(d), nsteps, npx, float(L_unit), ptr(out),
              stream_ptr())
    return out
