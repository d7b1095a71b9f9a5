"""Named synthetic workloads (all inputs seeded; no external data).

* ``VACUUM_SHADOW``   Kerr a=0.94, camera r=1000 M at 60 deg, 128x128 over
  +-10 M, at most 4096 steps, no plasma.
* ``RENDER_256``      FP64 full render: 16^3 meshblocks of 16^3 cells over
  [-50,50]^3 M, a=0.94, 17 deg, 256x256 over +-25 M, 230 GHz, R_low 1 /
  R_high 40, M = 6.5e9 Msun at 16.8 Mpc, at most 8192 steps.
* ``MIXED_SWEEP_512`` the RENDER_256 snapshot at 512x512, swept over spin
  {0, 0.5, 0.94} x inclination {17, 60, 85} x R_high {1, 10, 40}.
* ``SERVING``         Poisson request stream (20/s) over two resident
  snapshots (seeds 0, 1), resolutions {64..512}^2, spins {0, 0.5, 0.94},
  inclination U[10, 85], frequency {86, 230, 345} GHz, R_high U[1, 80].
* ``STRESS_1024``     32^3 meshblocks of 16^3 cells over [-100,100]^3 M,
  a=0.94, 60 deg, 1024x1024 over +-40 M, 86/230/345 GHz in one pass, at
  most 16384 steps.

``mass_scale`` is frozen per workload at the largest density scale whose
FP64 render keeps the reference's explicit Euler transfer stable (see
MASS_SCALE_256).
"""

from dataclasses import dataclass

from .constants import PARSEC, Msun


@dataclass(frozen=True)
class SnapshotSpec:
    nblocks: int = 16
    cells_per_block: int = 16
    extent: float = 50.0
    bhspin: float = 0.94
    seed: int = 0
    fluid_gamma: float = 13.0 / 9.0

    def build(self):
        from .grmhd.synthetic import make_synthetic_snapshot
        return make_synthetic_snapshot(nblocks=self.nblocks, cells_per_block=self.cells_per_block,
                                       extent=self.extent, bhspin=self.bhspin, seed=self.seed,
                                       fluid_gamma=self.fluid_gamma)


@dataclass(frozen=True)
class RenderSpec:
    snapshot: SnapshotSpec
    bhspin: float
    inclination: float
    resolution: int
    half_fov: float
    freqs: tuple
    max_nsteps: int
    r_low: float = 1.0
    r_high: float = 40.0
    M_bh: float = 6.5e9 * Msun
    distance_pc: float = 16.8e6
    mass_scale: float = 1.0e26
    camera_distance: float = 1000.0

    @property
    def fov(self):
        return 2.0 * self.half_fov

    @property
    def distance_cm(self):
        return self.distance_pc * PARSEC

    def request(self, model, **over):
        from .images import RenderRequest
        kw = dict(camera_inclination=self.inclination, camera_distance=self.camera_distance,
                  mass_scale=self.mass_scale, M_bh=self.M_bh, r_high=self.r_high,
                  observing_frequency=list(self.freqs) if len(self.freqs) > 1 else self.freqs[0],
                  fov=self.fov, resolution=self.resolution, max_nsteps=self.max_nsteps, r_low=self.r_low,
                  bhspin=self.bhspin)
        kw.update(over)
        return RenderRequest(model, **kw)


SNAP_256 = SnapshotSpec(nblocks=16, cells_per_block=16, extent=50.0, bhspin=0.94, seed=0)
SNAP_256_SEED1 = SnapshotSpec(nblocks=16, cells_per_block=16, extent=50.0, bhspin=0.94, seed=1)
SNAP_512 = SnapshotSpec(nblocks=32, cells_per_block=16, extent=100.0, bhspin=0.94, seed=0)

# mass_scale: the largest density scale whose FP64 render keeps every
# transfer step stable (per-step optical depth w*alpha below ~1).  The
# electron model (u = 0.1 rho/r, plasma beta 10) gives Theta_e ~ 3/r at
# R_high = 40, so a ~0.5 Jy image is out of reach before the explicit Euler
# solve of the reference turns unstable; these values give a few mJy.
MASS_SCALE_256 = 8.0e28
MASS_SCALE_512 = 8.0e28
# the 1024x1024 three-frequency stress render at 60 deg: the 86 GHz channel
# sets the bound (largest per-step optical depth 0.72 at 3e27, 4.7 at 5e27)
MASS_SCALE_STRESS = 3.0e27


_MS_ANCHORS = ((1.0, 3e26), (10.0, 3e27), (40.0, 8e28))


def mass_scale_for(r_high):
    """Stable mass_scale for an R_high: log-log interpolation through the
    anchors (1, 3e26), (10, 3e27), (40, 8e28), extended linearly in log-log
    beyond R_high = 40 (hotter electrons need less density)."""
    import numpy as np
    lx = np.log10([a for a, _ in _MS_ANCHORS])
    ly = np.log10([b for _, b in _MS_ANCHORS])
    x = np.log10(min(max(float(r_high), 1.0), 1e3))
    if x <= lx[-1]:
        return float(10 ** np.interp(x, lx, ly))
    slope = (ly[-1] - ly[-2]) / (lx[-1] - lx[-2])
    return float(10 ** (ly[-1] + slope * (x - lx[-1])))


def stable_mass_scale(r_high, inclination=17.0, nu=230e9):
    """Density scale that keeps the transfer's per-step optical depth below
    ~1 for any view of the synthetic torus: mass_scale_for(r_high) (set at
    17 deg, 230 GHz), times 0.1 + 0.9 cos^2(inclination) (edge-on rays
    cross the dense midplane; the optical depth grows roughly as the fifth
    power of the density scale, so a few-fold reduction suffices), times
    min(1, nu / 230 GHz)^2 (absorption grows toward low frequency: on the
    512^3-cell snapshot at 60 deg the 86 GHz channel's largest per-step
    optical depth is 47 at the linear factor and 0.7 at 3e27)."""
    import numpy as np
    c = np.cos(np.radians(float(inclination)))
    return mass_scale_for(r_high) * (0.1 + 0.9 * c * c) * min(1.0, float(nu) / 230e9) ** 2


RENDER_256 = RenderSpec(snapshot=SNAP_256, bhspin=0.94, inclination=17.0, resolution=256, half_fov=25.0,
                        freqs=(230e9,), max_nsteps=8192, r_high=40.0, mass_scale=MASS_SCALE_256)

STRESS_1024 = RenderSpec(snapshot=SNAP_512, bhspin=0.94, inclination=60.0, resolution=1024, half_fov=40.0,
                         freqs=(86e9, 230e9, 345e9), max_nsteps=16384, r_high=40.0,
                         mass_scale=MASS_SCALE_STRESS)

VACUUM_SHADOW = dict(bhspin=0.94, inclination=60.0, distance=1000.0, half_fov=10.0, resolution=128,
                     max_nsteps=4096, hfrac=0.05, hmin=0.01, hmax=10.0, capture=1.01, r_escape=1000.0)

MIXED_SWEEP = dict(spins=(0.0, 0.5, 0.94), inclinations=(17.0, 60.0, 85.0), r_highs=(1.0, 10.0, 40.0),
                   resolution=512)

SERVING = dict(rate_hz=20.0, resolutions=(64, 128, 256, 512), spins=(0.0, 0.5, 0.94), inc_range=(10.0, 85.0),
               freqs=(86e9, 230e9, 345e9), r_high_range=(1.0, 80.0), snapshots=(SNAP_256, SNAP_256_SEED1),
               seed=2024)
