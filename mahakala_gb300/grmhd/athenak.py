"""AthenaK fluid model with a device-resident snapshot.

Mirrors ``mahakala/grmhd/athenak.py``: ``AthenakFluidModel(grmhd_filename,
bhspin, fluid_gamma=None)`` with ``get_fluid_scalars_from_geodesics`` and
``get_prims_from_geodesics``.  The snapshot is uploaded once and kept on the
GPU as ghost-filled AoS float32 meshblocks (built by ``mk_snapshot_build``);
every sampling call runs in the sm_103a kernels.

``grmhd_filename`` may be a path to an ``.athdf`` file (read by this
package's own HDF5 reader, ``grmhd/hdf5.py``; h5py is used only for files
that reader refuses, when h5py is installed) or a ``SnapshotArrays`` (the
synthetic generators' output, or arrays the caller read itself).  Single- and multi-level meshes: the ghost fill of
athenak.py:67-525 runs on the device (``mk_snapshot_build``).
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


_ATHDF_DATASETS = ("x1v", "x2v", "x3v", "x1f", "x2f", "x3f", "uov", "B", "LogicalLocations", "Levels")


def load_athdf(path):
    """Read the datasets load_athenak_meshblocks reads (athenak.py:77-97):
    x1v..x3f, uov, B, LogicalLocations, Levels and the root attribute
    VariableNames, with this package's HDF5 reader (no h5py); a file using
    a part of HDF5 that reader does not implement is read with h5py when
    it is installed, else the reader's error is raised."""
    from .hdf5 import File, HDF5Error
    try:
        f = File(path)
        names = [bytes(n).split(b"\0")[0].decode("utf-8") for n in np.atleast_1d(f.attrs["VariableNames"])]
        d = {k: f[k] for k in _ATHDF_DATASETS}
    except HDF5Error:
        try:
            import h5py
        except ImportError:
            raise
        with h5py.File(path, "r") as hf:
            names = [n.decode("utf-8") for n in hf.attrs["VariableNames"]]
            d = {k: np.array(hf[k]) for k in _ATHDF_DATASETS}
    return SnapshotArrays(uov=d["uov"].astype(np.float32), B=d["B"].astype(np.float32), x1v=d["x1v"],
                          x2v=d["x2v"], x3v=d["x3v"], x1f=d["x1f"], x2f=d["x2f"], x3f=d["x3f"],
                          LogicalLocations=d["LogicalLocations"], Levels=d["Levels"],
                          VariableNames=tuple(names))


def mesh_tables(arrs, max_table_cells=1 << 28):
    """The block-grid metadata of a (single- or multi-level) mesh, from its
    logical locations, levels and faces (no field data): the finest-level
    block table, per-block faces, the sorted level/location keys, and which
    blocks have a ghost region filled from finer neighbours (those get a
    binary64 copy on the device)."""
    locs = np.ascontiguousarray(np.asarray(arrs.LogicalLocations, dtype=np.int32))
    levels = np.ascontiguousarray(np.asarray(arrs.Levels, dtype=np.int32))
    nmb = len(levels)
    if np.any(locs < 0) or np.any(levels < 0) or np.any(locs >= 1 << 18) or np.any(levels >= 512):
        raise ValueError("logical locations must lie in [0, 2^18) and levels in [0, 512)")
    keys = _lib.mesh_key(levels, locs[:, 0], locs[:, 1], locs[:, 2])
    if len(np.unique(keys)) != nmb:
        raise ValueError("duplicate (level, logical location) blocks")
    order = np.argsort(keys, kind="stable")
    faces = np.stack([arrs.x1f[:, 0], arrs.x1f[:, -1], arrs.x2f[:, 0], arrs.x2f[:, -1],
                      arrs.x3f[:, 0], arrs.x3f[:, -1]], axis=1).astype(np.float64)
    left, right = faces[:, 0::2], faces[:, 1::2]
    widths = right - left
    if np.any(widths <= 0):
        raise ValueError("block faces must increase")
    wf = widths.min(axis=0)
    lo, hi = left.min(axis=0), right.max(axis=0)
    nb = [int(round((hi[a] - lo[a]) / wf[a])) for a in range(3)]
    if int(np.prod(nb, dtype=np.int64)) > max_table_cells:
        raise ValueError(f"finest-level block table {nb} exceeds {max_table_cells} cells")
    table = -np.ones((nb[2], nb[1], nb[0]), np.int32)
    start = np.rint((left - lo) / wf).astype(np.int64)
    span = np.rint(widths / wf).astype(np.int64)
    for m in range(nmb):
        sl = tuple(slice(start[m, a], start[m, a] + span[m, a]) for a in (2, 1, 0))
        if np.any(table[sl] >= 0):
            raise ValueError("overlapping blocks")
        table[sl] = m
    keyset = set(keys.tolist())
    fine_ghosts = np.zeros(nmb, bool)
    if np.any(levels != levels[0]):
        for m in range(nmb):
            lv, t = int(levels[m]), [int(v) for v in locs[m]]
            for d in ((di, dj, dk) for di in (-1, 0, 1) for dj in (-1, 0, 1) for dk in (-1, 0, 1)):
                if d == (0, 0, 0):
                    continue
                u = [t[a] + d[a] for a in range(3)]
                if min(u) >= 0 and int(_lib.mesh_key(lv, *u)) in keyset:
                    continue
                if lv > 0 and int(_lib.mesh_key(lv - 1, *[v // 2 for v in u])) in keyset:
                    continue
                if min(u) >= 0 and int(_lib.mesh_key(lv + 1, *[2 * v for v in u])) in keyset:
                    fine_ghosts[m] = True
                    break
    block64 = np.where(fine_ghosts, np.cumsum(fine_ghosts) - 1, -1).astype(np.int32)
    return dict(locs=locs, levels=levels, keys=np.ascontiguousarray(keys[order]),
                key_block=np.ascontiguousarray(order.astype(np.int32)), faces=faces, table=table, nb=nb,
                lo=lo, width=wf, block64=block64, n64=int(fine_ghosts.sum()))


class DeviceSnapshot:
    """Resident meshblocks on one GPU plus the geometry tables of the lookup
    (single- or multi-level meshes)."""

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
        n = int(ni)
        t = mesh_tables(arrs)
        geom = np.stack([arrs.x1v[:, 0], arrs.x2v[:, 0], arrs.x3v[:, 0], arrs.x1v[:, 1] - arrs.x1v[:, 0],
                         arrs.x2v[:, 1] - arrs.x2v[:, 0], arrs.x3v[:, 1] - arrs.x3v[:, 0]], axis=1)
        self.n, self.nmb, self.nb = n, nmb, t["nb"]
        self.levels_host = t["levels"]
        self.device = dev
        self.geom = f64(geom, dev)
        self.faces = f64(t["faces"], dev)
        self.table = torch.as_tensor(t["table"], device=dev)
        self.locs = torch.as_tensor(t["locs"], device=dev)
        self.levels = torch.as_tensor(t["levels"], device=dev)
        keys = torch.as_tensor(t["keys"], device=dev)
        key_block = torch.as_tensor(t["key_block"], device=dev)
        self.n64 = t["n64"]
        n2 = n + 2
        self.blocks64 = (torch.empty((self.n64, n2, n2, n2, 8), dtype=torch.float64, device=dev)
                         if self.n64 else None)
        self.block64 = torch.as_tensor(t["block64"], device=dev) if self.n64 else None
        nbytes = _lib.load().mk_snapshot_bytes(nmb, n)
        self.storage = torch.empty(nbytes // 4, dtype=torch.float32, device=dev)
        uov_d = torch.as_tensor(np.ascontiguousarray(uov, dtype=np.float32), device=dev)
        B_d = torch.as_tensor(np.ascontiguousarray(B, dtype=np.float32), device=dev)
        mesh = _lib.MeshDesc()
        mesh.uov, mesh.B, mesh.locs, mesh.levels = ptr(uov_d), ptr(B_d), ptr(self.locs), ptr(self.levels)
        mesh.keys, mesh.key_block = ptr(keys), ptr(key_block)
        mesh.geom, mesh.faces, mesh.table = ptr(self.geom), ptr(self.faces), ptr(self.table)
        mesh.blocks64, mesh.block64 = ptr(self.blocks64), ptr(self.block64)
        mesh.nmb, mesh.n, mesh.n64 = nmb, n, self.n64
        for a in range(3):
            mesh.nb[a], mesh.lo[a], mesh.width[a] = t["nb"][a], float(t["lo"][a]), float(t["width"][a])
        view = _lib.SnapshotView()
        _lib.call("mk_snapshot_build", ctypes.byref(mesh), ptr(self.storage), nbytes, ctypes.byref(view),
                  stream_ptr())
        torch.cuda.current_stream().synchronize()
        del uov_d, B_d, keys, key_block
        self.view = view
        self.view_dev = torch.frombuffer(bytearray(bytes(view)), dtype=torch.uint8).to(dev)

    @property
    def nbytes(self):
        extra = self.blocks64.numel() * 8 + self.block64.numel() * 4 if self.n64 else 0
        return (self.storage.numel() * 4 + self.geom.numel() * 8 + self.faces.numel() * 8
                + self.table.numel() * 4 + self.locs.numel() * 4 + self.levels.numel() * 4 + extra)

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
