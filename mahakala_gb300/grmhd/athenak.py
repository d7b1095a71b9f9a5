"""AthenaK fluid model with a device-resident snapshot.

Mirrors ``mahakala/grmhd/athenak.py``: ``AthenakFluidModel(grmhd_filename,
bhspin, fluid_gamma=None)`` with ``get_fluid_scalars_from_geodesics`` and
``get_prims_from_geodesics``.  The snapshot is uploaded once and kept on the
GPU as ghost-filled AoS float32 meshblocks (built by ``mk_snapshot_build``);
every sampling call runs in the sm_103a kernels.

``grmhd_filename`` may be a path to an ``.athdf`` file (needs h5py) or a
``SnapshotArrays`` (the synthetic generator's output, or arrays the caller
read itself).  Single-level meshes only: the multi-level ghost fill of
athenak.py:235-502 is not built.
"""

import ctypes
import os
import time

import numpy as np
import torch

from .. import _lib
from .._device import device, f64, ptr, stream_ptr
from .grmhd import GRMHDFluidModel
from .synthetic import SnapshotArrays, VARIABLE_NAMES


def load_athdf(path):
    """Read the datasets load_athenak_meshblocks reads (athenak.py:77-97)."""
    try:
        import h5py
    except ImportError as e:  # pragma: no cover - h5py is optional
        raise RuntimeError("reading .athdf files needs h5py; pass a SnapshotArrays instead") from e
    with h5py.File(path, "r") as f:
        names = [n.decode("utf-8") for n in f.attrs["VariableNames"]]
        d = {k: np.array(f[k]) for k in ("x1v", "x2v", "x3v", "x1f", "x2f", "x3f", "uov", "B",
                                         "LogicalLocations", "Levels")}
    return SnapshotArrays(uov=d["uov"].astype(np.float32), B=d["B"].astype(np.float32), x1v=d["x1v"],
                          x2v=d["x2v"], x3v=d["x3v"], x1f=d["x1f"], x2f=d["x2f"], x3f=d["x3f"],
                          LogicalLocations=d["LogicalLocations"], Levels=d["Levels"],
                          VariableNames=tuple(names))


class DeviceSnapshot:
    """Resident meshblocks on one GPU plus the geometry tables of the lookup."""

    def __init__(self, arrs, dev=None):
        dev = dev or device()
        names = [v.lower().strip() for v in arrs.VariableNames]
        expect = [v for v in VARIABLE_NAMES]
        if names != expect:
            # athenak.py:707-710 requires contiguous velx..velz and bcc1..3
            raise ValueError(f"unexpected primitive order {names}, expected {expect}")
        uov, B = arrs.uov, arrs.B
        nprim, nmb, nk, nj, ni = uov.shape
        if nprim != 5 or B.shape[0] != 3 or not (nk == nj == ni):
            raise ValueError("expected uov (5, nmb, n, n, n) and B (3, nmb, n, n, n) with cubic blocks")
        levels = np.asarray(arrs.Levels)
        if np.any(levels != levels[0]):
            raise NotImplementedError("multi-level (AMR) snapshots are not supported yet")
        n = int(ni)
        locs = np.ascontiguousarray(np.asarray(arrs.LogicalLocations, dtype=np.int32))
        nb = [int(locs[:, c].max()) + 1 for c in range(3)]
        if np.any(locs < 0):
            raise ValueError("negative logical locations")
        table = -np.ones((nb[2], nb[1], nb[0]), np.int32)
        table[locs[:, 2], locs[:, 1], locs[:, 0]] = np.arange(nmb, dtype=np.int32)
        if len(np.unique(locs, axis=0)) != nmb:
            raise ValueError("duplicate logical locations")
        faces = []
        for c, f in enumerate((arrs.x1f, arrs.x2f, arrs.x3f)):
            fa = np.full(nb[c] + 1, np.nan)
            fa[locs[:, c]] = f[:, 0]
            fa[locs[:, c] + 1] = f[:, -1]
            if np.any(np.isnan(fa)) or np.any(np.diff(fa) <= 0):
                raise ValueError("block faces do not form a single-level grid")
            faces.append(fa)
        geom = np.stack([arrs.x1v[:, 0], arrs.x2v[:, 0], arrs.x3v[:, 0], arrs.x1v[:, 1] - arrs.x1v[:, 0],
                         arrs.x2v[:, 1] - arrs.x2v[:, 0], arrs.x3v[:, 1] - arrs.x3v[:, 0]], axis=1)
        self.n, self.nmb, self.nb = n, nmb, nb
        self.device = dev
        self.geom = f64(geom, dev)
        self.faces = f64(np.concatenate(faces), dev)
        self.table = torch.as_tensor(table, device=dev)
        self.locs = torch.as_tensor(locs, device=dev)
        nbytes = _lib.load().mk_snapshot_bytes(nmb, n)
        self.storage = torch.empty(nbytes // 4, dtype=torch.float32, device=dev)
        uov_d = torch.as_tensor(np.ascontiguousarray(uov, dtype=np.float32), device=dev)
        B_d = torch.as_tensor(np.ascontiguousarray(B, dtype=np.float32), device=dev)
        lo = [float(fa[0]) for fa in faces]
        width = [float((fa[-1] - fa[0]) / (len(fa) - 1)) for fa in faces]
        view = _lib.SnapshotView()
        _lib.call("mk_snapshot_build", ptr(uov_d), ptr(B_d), ptr(self.locs), ptr(self.geom), ptr(self.faces),
                  ptr(self.table), nmb, n, (ctypes.c_int32 * 3)(*nb), (ctypes.c_double * 3)(*lo),
                  (ctypes.c_double * 3)(*width), ptr(self.storage), nbytes, ctypes.byref(view), stream_ptr())
        torch.cuda.current_stream().synchronize()
        del uov_d, B_d
        self.view = view
        self.view_dev = torch.frombuffer(bytearray(bytes(view)), dtype=torch.uint8).to(dev)

    @property
    def nbytes(self):
        return (self.storage.numel() * 4 + self.geom.numel() * 8 + self.faces.numel() * 8
                + self.table.numel() * 4 + self.locs.numel() * 4)

    def blocks(self):
        """(nmb, n+2, n+2, n+2, 8) float32 view of the resident meshblocks."""
        n2 = self.n + 2
        return self.storage[: self.nmb * n2 ** 3 * 8].view(self.nmb, n2, n2, n2, 8)


class AthenakFluidModel(GRMHDFluidModel):

    def __init__(self, grmhd_filename, bhspin, fluid_gamma=None):
        arrs = grmhd_filename if isinstance(grmhd_filename, SnapshotArrays) else load_athdf(grmhd_filename)
        self.bhspin = bhspin
        self.fluid_gamma = fluid_gamma
        self.variable_names = np.array(arrs.VariableNames)
        self.x1v, self.x2v, self.x3v = arrs.x1v, arrs.x2v, arrs.x3v
        self.x1f, self.x2f, self.x3f = arrs.x1f, arrs.x2f, arrs.x3f
        self.Levels, self.LogicalLocations = arrs.Levels, arrs.LogicalLocations
        self.nprim_all = 8
        self.snapshot = DeviceSnapshot(arrs)

    def get_index_for_primitive_by_name(self, prim):
        """athenak.py:53-63."""
        prim = prim.lower().strip()
        names = [v.lower().strip() for v in self.variable_names]
        return names.index(prim) if prim in names else -1

    def _points(self, S):
        S = f64(S)
        if S.shape[-1] != 8:
            raise ValueError("S must have a last axis of 8 (x^mu, k^mu)")
        return S.reshape(-1, 8).contiguous(), S.shape[:-1]

    def get_fluid_scalars_from_geodesics(self, S, fallback_pitch_angle=np.pi / 3., profile=False):
        """athenak.py:639-812 -> dict(dens, u, pitch_angle, kdotu, b)."""
        t0 = time.time()
        pts, shape = self._points(S)
        out = torch.empty((pts.shape[0], 5), dtype=torch.float64, device=pts.device)
        _lib.call("mk_fluid_scalars", ctypes.byref(self.snapshot.view), float(self.bhspin), ptr(pts),
                  pts.shape[0], float(np.cos(fallback_pitch_angle)), ptr(out), stream_ptr())
        if profile:
            torch.cuda.current_stream().synchronize()
            print(f"Time to compute scalar data: {time.time() - t0}")
        out = out.reshape(tuple(shape) + (5,))
        return dict(dens=out[..., 0], u=out[..., 1], pitch_angle=out[..., 2], kdotu=out[..., 3], b=out[..., 4])

    def get_prims_from_geodesics(self, S, profile=False):
        """athenak.py:527-637 -> dict(dens, u, U1..U3, B1..B3)."""
        pts, shape = self._points(S)
        out = torch.empty((pts.shape[0], 8), dtype=torch.float64, device=pts.device)
        _lib.call("mk_fluid_prims", ctypes.byref(self.snapshot.view), ptr(pts), pts.shape[0], ptr(out), None,
                  stream_ptr())
        out = out.reshape(tuple(shape) + (8,))
        return dict(dens=out[..., 0], u=out[..., 4], U1=out[..., 1], U2=out[..., 2], U3=out[..., 3],
                    B1=out[..., 5], B2=out[..., 6], B3=out[..., 7])
