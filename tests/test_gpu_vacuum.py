"""Vacuum shadow test: Kerr a=0.94, camera at r=1000, inclination 60 deg,
128x128 pixels over +-10 M, at most 4096 steps, no plasma.  Both step
policies against the oracle: the reference rule (div 40, tol 1e-4) and the
fixed-fraction rule (h = 0.05 r clamped to [0.01, 10] M, captured at
r < 1.01 r_h, escaped at r > 1000 M once r grows).

Bar: captured/escaped masks bit-exact; step counts equal and final x^mu,
k^mu within 1e-9 relative (floor 1e-3 for components that pass through
zero) for every well-conditioned ray.  A ray is ill-conditioned when the
oracle's own end state moves by more than 100x a 1e-12 change of the
initial wavevector (photon-ring grazers: no FP64 evaluation order
reproduces them to 1e-9); those are counted, and must stay a few percent.
"""

import numpy as np
import pytest

from conftest import golden, rel_err

pytestmark = pytest.mark.gpu

A, INC, RES, NMAX = 0.94, 60.0, 128, 4096


@pytest.fixture(scope="module")
def s0(orc):
    return orc.initialize_geodesics_at_camera(A, INC, 1000.0, -10.0, 10.0, RES)


def test_vacuum_reference_policy(cuda, orc, s0):
    from mahakala_gb300.geodesics import step_policy, trace
    o = orc.integrate(s0, NMAX, 40.0, 1e-4, A)
    op = orc.integrate(orc.perturbed(s0), NMAX, 40.0, 1e-4, A)
    g = trace(s0, A, step_policy(NMAX, 40.0, 1e-4))
    why, K, st = (g[k].cpu().numpy() for k in ("why", "K", "state"))
    assert np.array_equal(why, o["why"])
    cap = why == 1
    assert 0.05 < cap.mean() < 0.6          # a shadow is there
    ill = orc.ill_conditioned(o["state"], op["state"]) | (o["K"] != op["K"])
    print(f"vacuum reference policy: {ill.sum()} of {len(K)} rays ill-conditioned")
    assert ill.mean() < 0.05
    ok = ~ill
    assert np.array_equal(K[ok], o["K"][ok])
    assert np.nanmax(rel_err(st[ok], o["state"][ok], floor=1e-3)) < 1e-9


def test_vacuum_fixed_policy(cuda, orc, s0):
    from mahakala_gb300.geodesics import step_policy, trace
    o = orc.trace_fixed(s0, NMAX, A)
    op = orc.trace_fixed(orc.perturbed(s0), NMAX, A)
    g = trace(s0, A, step_policy(NMAX, kind="fixed"))
    why, K, st = (g[k].cpu().numpy() for k in ("why", "K", "state"))
    assert np.array_equal(why, o["why"])
    assert set(np.unique(why)) <= {1, 2}     # every ray captured or escaped within 4096 steps
    ill = orc.ill_conditioned(o["state"], op["state"]) | (o["nsteps"] != op["nsteps"])
    print(f"vacuum fixed policy: {ill.sum()} of {len(K)} rays ill-conditioned")
    assert ill.mean() < 0.05
    ok = ~ill
    assert np.array_equal(K[ok], o["nsteps"][ok])
    assert np.nanmax(rel_err(st[ok], o["state"][ok], floor=1e-3)) < 1e-9


@pytest.mark.parametrize("key", ["test1", "test2", "test3", "test4"])
def test_shadow_bisection_reference_fixture(cuda, key):
    """The reference's only automated test (tests/test_shadows.py:28-45) on
    its own data, through the GPU path."""
    import mahakala_gb300 as mk
    d = golden("shadow")
    r = mk.find_shadow_bisection_angles(float(d[f"{key}_bhspin"]), float(d[f"{key}_inclination"]),
                                        d[f"{key}_angles"])
    assert np.allclose(r, d[f"{key}_radii"], rtol=1e-2)


def test_shadow_bisection_matches_oracle(cuda, orc):
    import mahakala_gb300 as mk
    d = golden("shadow")
    ang = d["test3_angles"][::4]
    r = mk.find_shadow_bisection_angles(0.44, 52.0, ang)
    o = orc.find_shadow_bisection_angles(0.44, 52.0, ang)
    # one flipped decision moves the answer by at most the bracket it split
    assert np.max(np.abs(r - o)) <= 9.5 / 2 ** 13
    assert np.mean(r == o) >= 0.9
    a, inc, max_steps, err, max_it = d["short_params"]
    short = mk.find_shadow_bisection_angles(a, inc, d["short_angles"], max_steps=int(max_steps),
                                            error_allowed=err, max_it=int(max_it))
    assert np.array_equal(short, d["short_radii"])
