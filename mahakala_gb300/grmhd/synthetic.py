"""Seeded synthetic GRMHD-like snapshot in AthenaK's in-memory layout.

No GRMHD snapshot file is available, so renders run on a deterministic
synthetic torus built here with NumPy ``Generator(PCG64(seed))``.  The arrays
are returned exactly as ``AthenakFluidModel.load_athenak_meshblocks`` reads
them from an ``.athdf`` file (``mahakala/grmhd/athenak.py:67-97``):

* ``uov``  float32 ``(5, nmb, nk, nj, ni)`` in the order dens, velx, vely,
  velz, eint;
* ``B``    float32 ``(3, nmb, nk, nj, ni)`` (bcc1..3);
* ``x1v/x2v/x3v`` ``(nmb, n)`` cell centres, ``x1f/x2f/x3f`` ``(nmb, n+1)``
  cell faces (float64);
* ``LogicalLocations`` int32 ``(nmb, 3)`` = (i, j, k) block coordinates and
  ``Levels`` int32 ``(nmb,)`` (a single refinement level);
* ``VariableNames`` the eight primitive names.

Field model (per cell centre; r is the Kerr-Schild radius of the metric, R
the cylindrical radius):

* rho = (r/6)^-1.5 * exp(-z^2 / (2 (0.4 R)^2)) * exp(0.3 * N(0,1))
* u   = 0.1 * rho / r
* velocity (normal-frame 4-velocity components velx..velz): Keplerian
  v_K = r^-1/2 along phi-hat plus a radial inflow of -0.05 v_K along r-hat
* magnetic field: |B| = sqrt(2 (gamma-1) u / beta) with plasma beta = 10,
  split 0.8 toroidal (phi-hat) + 0.6 vertical (z-hat)
* every primitive is zero in cells whose centre lies inside the horizon.

Block ``mb = bi + nb*(bj + nb*bk)`` covers cells ``[bi*n, (bi+1)*n)`` etc.
The cell size is ``2*extent/(nb*n)``; the standard sizes (16 or 32 blocks of
16 cells over +-50 or +-100) give dx = 25/64, exactly representable, so the
grid coordinates carry no rounding.
"""

from dataclasses import dataclass, field

import numpy as np

VARIABLE_NAMES = ("dens", "velx", "vely", "velz", "eint", "bcc1", "bcc2", "bcc3")


@dataclass
class SnapshotArrays:
    uov: np.ndarray
    B: np.ndarray
    x1v: np.ndarray
    x2v: np.ndarray
    x3v: np.ndarray
    x1f: np.ndarray
    x2f: np.ndarray
    x3f: np.ndarray
    LogicalLocations: np.ndarray
    Levels: np.ndarray
    VariableNames: tuple = VARIABLE_NAMES
    bhspin: float = 0.0
    fluid_gamma: float = 13.0 / 9.0
    params: dict = field(default_factory=dict)

    @property
    def nmb(self):
        return self.uov.shape[1]

    @property
    def cells_per_block(self):
        return self.uov.shape[-1]


def _ks_radius(x, y, z, a):
    aa = a * a
    kk = 0.5 * (x * x + y * y + z * z - aa)
    return np.sqrt(np.sqrt(kk * kk + aa * z * z) + kk)


def make_synthetic_snapshot(nblocks=16, cells_per_block=16, extent=50.0,
                            bhspin=0.94, seed=0, fluid_gamma=13.0 / 9.0,
                            plasma_beta=10.0, noise_sigma=0.3):
    """Build the seeded synthetic snapshot (see module docstring)."""
    nb = int(nblocks)
    n = int(cells_per_block)
    ntot = nb * n
    dx = 2.0 * extent / ntot
    x0 = -float(extent)
    a = float(bhspin)
    r_h = 1.0 + np.sqrt(1.0 - a * a)
    rng = np.random.Generator(np.random.PCG64(seed))

    centres = x0 + (np.arange(ntot, dtype=np.float64) + 0.5) * dx
    prim = np.zeros((8, ntot, ntot, ntot), dtype=np.float32)  # [p, k, j, i]
    yy, xx = np.meshgrid(centres, centres, indexing="ij")  # [j, i]
    for k in range(ntot):
        z = centres[k]
        noise = rng.standard_normal((ntot, ntot), dtype=np.float32)
        r = _ks_radius(xx, yy, z, a)
        R = np.sqrt(xx * xx + yy * yy)
        H = 0.4 * R
        rho = (r / 6.0) ** -1.5 * np.exp(-z * z / (2.0 * H * H)) \
            * np.exp(noise_sigma * noise.astype(np.float64))
        u = 0.1 * rho / r
        vk = 1.0 / np.sqrt(r)
        phx, phy = -yy / R, xx / R
        vr = -0.05 * vk
        vx = vk * phx + vr * xx / r
        vy = vk * phy + vr * yy / r
        vz = vr * z / r
        bmag = np.sqrt(2.0 * (fluid_gamma - 1.0) * u / plasma_beta)
        bx = 0.8 * bmag * phx
        by = 0.8 * bmag * phy
        bz = 0.6 * bmag * np.ones_like(bmag)
        inside = r < r_h
        for p, arr in enumerate((rho, vx, vy, vz, u, bx, by, bz)):
            arr = np.where(inside, 0.0, arr)
            prim[p, k] = arr.astype(np.float32)

    # global [p, k, j, i] -> blocks [p, mb, k, j, i] with mb = bi + nb*(bj + nb*bk)
    blocks = prim.reshape(8, nb, n, nb, n, nb, n).transpose(0, 1, 3, 5, 2, 4, 6)
    blocks = np.ascontiguousarray(blocks.reshape(8, nb ** 3, n, n, n))
    del prim

    bi, bj, bk = np.meshgrid(np.arange(nb), np.arange(nb), np.arange(nb), indexing="ij")
    # order blocks with bi fastest
    bi = bi.transpose(2, 1, 0).reshape(-1)
    bj = bj.transpose(2, 1, 0).reshape(-1)
    bk = bk.transpose(2, 1, 0).reshape(-1)
    locs = np.stack([bi, bj, bk], axis=1).astype(np.int32)
    cell = np.arange(n, dtype=np.float64)
    face = np.arange(n + 1, dtype=np.float64)

    def axis_coords(bidx):
        v = x0 + (bidx[:, None] * n + cell[None, :] + 0.5) * dx
        f = x0 + (bidx[:, None] * n + face[None, :]) * dx
        return v, f

    x1v, x1f = axis_coords(bi)
    x2v, x2f = axis_coords(bj)
    x3v, x3f = axis_coords(bk)
    return SnapshotArrays(
        uov=blocks[:5], B=blocks[5:], x1v=x1v, x2v=x2v, x3v=x3v,
        x1f=x1f, x2f=x2f, x3f=x3f, LogicalLocations=locs,
        Levels=np.zeros(nb ** 3, dtype=np.int32), bhspin=a,
        fluid_gamma=float(fluid_gamma),
        params=dict(nblocks=nb, cells_per_block=n, extent=float(extent),
                    seed=int(seed), plasma_beta=float(plasma_beta),
                    noise_sigma=float(noise_sigma)))


def _torus_fields(x, y, z, a, rng, fluid_gamma, plasma_beta, noise_sigma):
    """The field model of the module docstring at cell centres (x, y, z)
    (broadcast arrays); returns 8 float32 arrays dens, velx..velz, eint,
    bcc1..3."""
    r_h = 1.0 + np.sqrt(1.0 - a * a)
    r = _ks_radius(x, y, z, a)
    R = np.maximum(np.sqrt(x * x + y * y), 1e-12)
    H = 0.4 * R
    noise = rng.standard_normal(np.shape(r))
    rho = (r / 6.0) ** -1.5 * np.exp(-z * z / (2.0 * H * H)) * np.exp(noise_sigma * noise)
    u = 0.1 * rho / r
    vk = 1.0 / np.sqrt(r)
    phx, phy = -y / R, x / R
    vr = -0.05 * vk
    bmag = np.sqrt(2.0 * (fluid_gamma - 1.0) * u / plasma_beta)
    out = (rho, vk * phx + vr * x / r, vk * phy + vr * y / r, vr * z / r, u,
           0.8 * bmag * phx, 0.8 * bmag * phy, 0.6 * bmag)
    inside = r < r_h
    return [np.where(inside, 0.0, np.broadcast_to(v, np.shape(r))).astype(np.float32) for v in out]


def make_multilevel_snapshot(nblocks=2, cells_per_block=8, extent=8.0, refine=((0, 0, 0, 0),),
                             bhspin=0.94, seed=0, fluid_gamma=13.0 / 9.0, plasma_beta=10.0,
                             noise_sigma=0.3):
    """A mesh refined like AthenaK's static/adaptive refinement: nblocks^3
    root blocks (level 0) of cells_per_block^3 cells over [-extent, extent]^3;
    each entry (level, i, j, k) of ``refine``, applied in order, replaces that
    block by its 8 children at level + 1 (logical locations 2i + {0,1}, ...).
    Blocks are listed by level, then k, j, i.  Same field model as
    make_synthetic_snapshot, evaluated at each block's own cell centres."""
    nb, n = int(nblocks), int(cells_per_block)
    blocks = {(0, i, j, k) for i in range(nb) for j in range(nb) for k in range(nb)}
    for key in refine:
        key = tuple(int(v) for v in key)
        if key not in blocks:
            raise ValueError(f"no block {key} to refine")
        blocks.remove(key)
        lv, i, j, k = key
        for c in range(8):
            blocks.add((lv + 1, 2 * i + (c & 1), 2 * j + ((c >> 1) & 1), 2 * k + (c >> 2)))
    order = sorted(blocks, key=lambda b: (b[0], b[3], b[2], b[1]))
    rng = np.random.Generator(np.random.PCG64(seed))
    a = float(bhspin)
    nmb = len(order)
    data = np.zeros((8, nmb, n, n, n), np.float32)
    coords = {c: (np.zeros((nmb, n)), np.zeros((nmb, n + 1))) for c in range(3)}
    for m, (lv, i, j, k) in enumerate(order):
        w = 2.0 * extent / (nb * 2 ** lv)  # block width at this level
        dx = w / n
        cen, fac = [], []
        for c, loc in enumerate((i, j, k)):
            left = -extent + loc * w
            v = left + (np.arange(n) + 0.5) * dx
            f = left + np.arange(n + 1) * dx
            coords[c][0][m], coords[c][1][m] = v, f
            cen.append(v)
        zz, yy, xx = np.meshgrid(cen[2], cen[1], cen[0], indexing="ij")
        for p, arr in enumerate(_torus_fields(xx, yy, zz, a, rng, fluid_gamma, plasma_beta, noise_sigma)):
            data[p, m] = arr
    locs = np.array([[i, j, k] for _, i, j, k in order], np.int32)
    levels = np.array([lv for lv, _, _, _ in order], np.int32)
    return SnapshotArrays(uov=data[:5], B=data[5:], x1v=coords[0][0], x2v=coords[1][0], x3v=coords[2][0],
                          x1f=coords[0][1], x2f=coords[1][1], x3f=coords[2][1], LogicalLocations=locs,
                          Levels=levels, bhspin=a, fluid_gamma=float(fluid_gamma),
                          params=dict(nblocks=nb, cells_per_block=n, extent=float(extent),
                                      refine=[tuple(r) for r in refine], seed=int(seed)))
