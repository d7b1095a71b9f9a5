"""Serving on the GPU: a mixed stream of requests (sizes, spins,
inclinations, frequencies, electron models, two snapshots) through the
continuous-batching scheduler and captured CUDA graphs.  Every result
must equal the same request rendered alone (the kernels are deterministic
per ray, so the bar is exact), requests must share launches, and both
slots must be used."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def models():
    from mahakala_gb300.grmhd.athenak import AthenakFluidModel
    from mahakala_gb300.grmhd.synthetic import make_synthetic_snapshot
    out = []
    for seed in (0, 1):
        arrs = make_synthetic_snapshot(nblocks=4, cells_per_block=16, extent=50.0, bhspin=0.94, seed=seed)
        out.append(AthenakFluidModel(arrs, 0.94, fluid_gamma=13. / 9))
    return out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_stream_results_equal_isolated(cuda, models, precision):
    from mahakala_gb300.serving import DeviceExecutor, Scheduler, isolated_times, latency_report, poisson_stream
    arrivals, reqs = poisson_stream(models, 12, rate_hz=200.0, seed=7, resolutions=(16, 24, 32, 48))
    ex = DeviceExecutor(models, precision=precision, nslots=2, buckets=(1024, 4096, 8192), max_requests=16)
    sched = Scheduler(ex, hbm_budget=ex.resident_bytes + (256 << 20), max_requests=16)
    tickets = [sched.submit(r) for r in reqs[:6]]          # six arrive together
    sched.step()
    tickets += [sched.submit(r) for r in reqs[6:]]         # six more while the first batch runs
    sched.run_until_idle()
    assert all(t.status == "done" for t in tickets)
    assert any(b["requests"] > 1 for b in sched.batches)   # packed into shared launches
    assert len({b["slot"] for b in sched.batches}) == 2     # both slots used
    _, alone = isolated_times(reqs, precision)
    for t, ref in zip(tickets, alone):
        assert t.image.shape == ref.shape
        assert np.all(np.isfinite(ref)), f"request {t.id}: non-finite pixels (unstable transfer)"
        assert np.array_equal(t.image, ref, equal_nan=True), f"request {t.id} differs in the mix"
    rep = latency_report(tickets, wall=max(t.finished for t in tickets) - min(t.arrival for t in tickets))
    assert rep["served"] == 12 and rep["p99_ms"] > 0


def test_oversize_and_bad_requests_rejected(cuda, models):
    from mahakala_gb300.images import RenderRequest
    from mahakala_gb300.serving import DeviceExecutor, RequestError, Scheduler
    ex = DeviceExecutor(models[:1], precision="mixed", nslots=1, buckets=(1024,), capture=False)
    sched = Scheduler(ex, hbm_budget=ex.resident_bytes + (64 << 20))
    with pytest.raises(RequestError):
        sched.submit(RenderRequest(models[0], resolution=64))      # 4096 rays > bucket
    with pytest.raises(RequestError):
        sched.submit(RenderRequest(models[0], resolution=16, observing_frequency=[]))
    t = sched.submit(RenderRequest(models[0], resolution=16, fov=50.0, max_nsteps=2000))
    sched.run_until_idle()
    assert t.status == "done" and np.all(np.isfinite(t.image))
