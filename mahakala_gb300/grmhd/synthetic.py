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
