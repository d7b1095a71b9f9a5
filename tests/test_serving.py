"""Serving scheduler logic on the CPU with a fake executor: continuous
batching across slots, bucket choice, HBM-budget admission, rejection of
malformed and oversize requests, cancellation, and failure propagation.
Failures are injected on the host (an executor that reports an error or
raises at launch); nothing here touches a GPU."""

import numpy as np
import pytest

from mahakala_gb300.serving import RequestError, Scheduler, latency_report, output_bytes


class FakeModel:
    bhspin = 0.9
    fluid_gamma = 13. / 9

    class snapshot:
        pass


class Clock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t


class FakeExecutor:
    """Each batch takes `cost * rays` seconds of fake time."""

    def __init__(self, clock, nslots=2, buckets=(100, 400, 1600), resident=1000, cost=1e-3, fail_batches=(),
                 raise_batches=()):
        self.clock, self.nslots, self.buckets, self.resident_bytes = clock, nslots, buckets, resident
        self.cost, self.fail, self.raise_ = cost, set(fail_batches), set(raise_batches)
        self.launches = []

    def launch(self, slot, bucket, tickets):
        n = len(self.launches)
        self.launches.append((slot, bucket, [t.id for t in tickets]))
        if n in self.raise_:
            raise RuntimeError("injected launch error")
        rays = sum(t.rays for t in tickets)
        return dict(n=n, done_at=self.clock() + self.cost * rays, tickets=tickets)

    def poll(self, h):
        if "error" in h:
            return dict(ok=False, error=h["error"], images=None)
        if self.clock() < h["done_at"]:
            return None
        if h["n"] in self.fail:
            return dict(ok=False, error="injected kernel error status", images=None)
        return dict(ok=True, error=None, images=[np.full((1, 2, 2), t.id, float) for t in h["tickets"]])


def req(res, nu=230e9, **kw):
    from mahakala_gb300.images import RenderRequest
    return RenderRequest(FakeModel, resolution=res, observing_frequency=nu, **kw)


def drive(sched, clock, until=100.0, dt=1e-3):
    while not sched.idle() and clock.t < until:
        sched.step()
        clock.t += dt


def test_concurrent_arrivals_share_one_launch_and_bucket():
    clock = Clock()
    ex = FakeExecutor(clock)
    s = Scheduler(ex, hbm_budget=10 ** 9, clock=clock)
    ts = [s.submit(req(r)) for r in (8, 10, 12)]            # 64 + 100 + 144 = 308 rays
    s.step()
    assert len(ex.launches) == 1 and ex.launches[0][1] == 400
    assert ex.launches[0][2] == [t.id for t in ts]
    drive(s, clock)
    assert all(t.status == "done" for t in ts)
    assert [int(t.image[0, 0, 0]) for t in ts] == [t.id for t in ts]


def test_continuous_batching_overlaps_slots():
    clock = Clock()
    ex = FakeExecutor(clock, cost=1e-2)
    s = Scheduler(ex, hbm_budget=10 ** 9, clock=clock)
    a = s.submit(req(20))                                     # 400 rays -> slot 0, busy 4 s
    s.step()
    clock.t = 1.0
    b = s.submit(req(10))                                     # arrives while slot 0 runs
    s.step()
    assert [x[0] for x in ex.launches] == [0, 1]              # went to the free slot at once
    assert b.launched == 1.0 and a.status == "running"
    drive(s, clock)
    assert a.finished > b.finished                            # the small one did not wait for the big one


def test_budget_admission_waits_for_memory():
    clock = Clock()
    ex = FakeExecutor(clock, resident=0, cost=1e-2)
    one = output_bytes(req(10))
    s = Scheduler(ex, hbm_budget=one + one // 2, clock=clock)  # room for one request's outputs
    a, b = s.submit(req(10)), s.submit(req(10))
    s.step()
    assert len(ex.launches) == 1 and b.status == "waiting"   # slot free, memory not
    drive(s, clock)
    assert len(ex.launches) == 2 and b.launched >= a.finished
    assert s.in_flight_bytes == 0


def test_rejections():
    clock = Clock()
    s = Scheduler(FakeExecutor(clock), hbm_budget=10 ** 9, clock=clock)
    with pytest.raises(RequestError):
        s.submit(req(41))                                     # 1681 rays > largest bucket (1600)
    with pytest.raises(RequestError):
        s.submit(req(0))
    with pytest.raises(RequestError):
        s.submit(req(8, nu=[1e9, 2e9, 3e9, 4e9, 5e9]))
    with pytest.raises(RequestError):
        s.submit(req(8, bhspin=1.2))
    with pytest.raises(RequestError):
        s.submit(req(8, mass_scale=-1.0))
    small = Scheduler(FakeExecutor(clock, resident=0), hbm_budget=100, clock=clock)
    with pytest.raises(RequestError):
        small.submit(req(8))                                  # outputs alone exceed the budget
    with pytest.raises(RequestError):
        Scheduler(FakeExecutor(clock, resident=10 ** 6), hbm_budget=10, clock=clock)


def test_cancel_before_launch():
    clock = Clock()
    ex = FakeExecutor(clock, nslots=1, cost=1e-2)
    s = Scheduler(ex, hbm_budget=10 ** 9, clock=clock)
    a = s.submit(req(20))
    s.step()
    b, c = s.submit(req(10)), s.submit(req(10))
    assert s.cancel(b) and b.status == "cancelled"
    assert not s.cancel(a)                                    # already running
    drive(s, clock)
    assert a.status == c.status == "done" and b.image is None
    assert all(b.id not in ids for _, _, ids in ex.launches)


def test_failed_batches_fail_their_requests_only():
    clock = Clock()
    ex = FakeExecutor(clock, nslots=1, fail_batches={0}, raise_batches={1})
    s = Scheduler(ex, hbm_budget=10 ** 9, clock=clock)
    a = s.submit(req(20))
    s.step()
    b = s.submit(req(20))
    drive(s, clock, until=0.5)
    c = s.submit(req(20))
    drive(s, clock)
    assert a.status == "failed" and "kernel error" in a.error
    assert b.status == "failed" and "launch failed" in b.error
    assert c.status == "done"
    rep = latency_report([a, b, c], wall=clock.t)
    assert rep["served"] == 1 and rep["failed"] == 2


def test_request_cap_per_batch():
    clock = Clock()
    ex = FakeExecutor(clock, buckets=(10 ** 6,))
    s = Scheduler(ex, hbm_budget=10 ** 12, max_requests=4, clock=clock)
    for _ in range(10):
        s.submit(req(4))
    drive(s, clock)
    assert [len(ids) for _, _, ids in ex.launches] == [4, 4, 2]


def _overload(clock, latency_bound):
    """An arrival every 0.05 s of requests that each take 0.1 s alone on a
    one-slot executor (offered load 2), served with or without a latency
    bound."""
    ex = FakeExecutor(clock, nslots=1, buckets=(100, 400, 1600), cost=1e-3)
    kw = {} if latency_bound is None else dict(latency_bound=latency_bound,
                                               predict=lambda r: 1e-3 * int(r.resolution) ** 2)
    s = Scheduler(ex, hbm_budget=10 ** 9, clock=clock, **kw)
    tickets = []
    for k in range(40):
        while clock.t < 0.05 * k:
            s.step()
            clock.t += 1e-3
        tickets.append(s.submit(req(10), arrival=clock.t))
    drive(s, clock, until=1000.0)
    return tickets


def test_latency_bound_sheds_under_overload_and_bounds_served_latency():
    """Offered load 2: without a bound every request is served and the
    queue (and latency) grows; with k = 2, some requests are shed and every
    served one finishes within 2x its isolated time (plus the 1 ms poll
    step of the fake clock)."""
    free = _overload(Clock(), None)
    assert all(t.status == "done" for t in free)
    assert max(t.latency for t in free) > 10 * 0.1
    bounded = _overload(Clock(), 2.0)
    served = [t for t in bounded if t.status == "done"]
    shed = [t for t in bounded if t.status == "shed"]
    assert served and shed and len(served) + len(shed) == len(bounded)
    assert all(t.latency <= 2.0 * 0.1 + 2e-3 for t in served), max(t.latency for t in served)
    assert all(t.error.startswith("shed") for t in shed)
    rep = latency_report(bounded, 3.0)
    assert rep["shed"] == len(shed) and rep["served"] == len(served)


def test_latency_bound_admits_everything_under_light_load():
    clock = Clock()
    ex = FakeExecutor(clock, cost=1e-3)
    s = Scheduler(ex, hbm_budget=10 ** 9, clock=clock, latency_bound=2.0,
                  predict=lambda r: 1e-3 * int(r.resolution) ** 2)
    tickets = []
    for k in range(10):
        while clock.t < 0.5 * k:
            s.step()
            clock.t += 1e-3
        tickets.append(s.submit(req(10), arrival=clock.t))
    drive(s, clock)
    assert all(t.status == "done" for t in tickets)


def test_latency_bound_keeps_batches_within_every_members_bound():
    """A small request is not packed behind a large one when the batch's
    predicted time would break the small one's bound."""
    clock = Clock()
    ex = FakeExecutor(clock, nslots=1, buckets=(100, 400, 1600), cost=1e-3)
    s = Scheduler(ex, hbm_budget=10 ** 9, clock=clock, latency_bound=2.0,
                  predict=lambda r: 1e-3 * int(r.resolution) ** 2)
    big = s.submit(req(30))      # 0.9 s
    small = s.submit(req(4))     # 0.016 s: would wait for the big one's 0.9 s
    s.step()
    assert ex.launches[0][2] == [big.id]
    drive(s, clock)
    assert big.status == "done" and small.status == "shed"


def test_latency_bound_needs_a_predictor():
    clock = Clock()
    with pytest.raises(ValueError):
        Scheduler(FakeExecutor(clock), hbm_budget=10 ** 9, clock=clock, latency_bound=2.0)
    with pytest.raises(ValueError):
        Scheduler(FakeExecutor(clock), hbm_budget=10 ** 9, clock=clock, latency_bound=1.0, predict=lambda r: 1.0)


def test_latency_bound_counts_work_already_on_the_gpu():
    """A persistent render holds the SMs until it ends, so a request is not
    sent to a free slot beside a long batch when that batch's remaining work
    would break the request's bound: with two free slots, a 900 ms request
    and a 16 ms one submitted together, the long one launches and the short
    one is shed instead of launching beside it."""
    clock = Clock()
    ex = FakeExecutor(clock, nslots=2, buckets=(100, 400, 1600), cost=1e-3)
    s = Scheduler(ex, hbm_budget=10 ** 9, clock=clock, latency_bound=2.0,
                  predict=lambda r: 1e-3 * int(r.resolution) ** 2)
    big = s.submit(req(30))
    small = s.submit(req(4))
    s.step()
    assert [x[2] for x in ex.launches] == [[big.id]]
    assert small.status == "shed" and "work ahead" in small.error
    drive(s, clock)
    assert big.status == "done"


def test_latency_bound_uses_low_for_own_bound_and_high_for_work_ahead():
    """With (low, high) predictions a request alone is admitted on its low
    figure, while the work it puts ahead of a later request counts at its
    high figure."""
    clock = Clock()
    ex = FakeExecutor(clock, nslots=2, buckets=(100, 400, 1600), cost=1e-3)
    s = Scheduler(ex, hbm_budget=10 ** 9, clock=clock, latency_bound=2.0,
                  predict=lambda r: (1e-3 * int(r.resolution) ** 2, 3e-3 * int(r.resolution) ** 2))
    first = s.submit(req(10))          # low 0.1 s, high 0.3 s: alone, within 2 x 0.1
    s.step()
    assert first.status == "running"
    clock.t = 0.15                     # by the low figure it is done; by the high one 0.15 s remain
    later = s.submit(req(8), arrival=clock.t)   # low 0.064 s: 0.15 + 0.064 > 0.128
    assert later.status == "shed"
    drive(s, clock)
    assert first.status == "done"


def test_latency_bound_holds_back_a_batch_that_would_delay_a_running_request():
    """A long request is not launched beside a running short one when the
    shared GPU would push the short one past its bound; it launches once
    the short one is done."""
    clock = Clock()
    ex = FakeExecutor(clock, nslots=2, buckets=(100, 400, 1600), cost=1e-3)
    s = Scheduler(ex, hbm_budget=10 ** 9, clock=clock, latency_bound=2.0,
                  predict=lambda r: 1e-3 * int(r.resolution) ** 2)
    short = s.submit(req(10))          # 0.1 s
    s.step()
    clock.t = 0.01
    long_ = s.submit(req(20))          # 0.4 s: 0.01 + 0.09 + 0.4 > 0.2 for the short one
    s.step()
    assert [x[2] for x in ex.launches] == [[short.id]] and long_.status == "waiting"
    drive(s, clock)
    assert short.status == "done" and long_.status == "done"
    assert [x[2] for x in ex.launches] == [[short.id], [long_.id]]
