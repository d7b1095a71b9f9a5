"""The near-hole pipeline's synchronisation protocol, modelled on the host.

render_zone_kernel (mahakala_gb300/csrc/mk_render.cu) runs one integrating
warp and three sampling warps per block.  Message j goes through slot
j % ZONE_SLOTS of a ring in shared memory; each slot has a `full` and an
`empty` mbarrier (32 arrivals complete a phase; a wait on parity P
succeeds once the phase of parity P has completed, so a fresh barrier's
parity-1 wait succeeds at once); sampler j % 3 takes message j and folds
it once the shared fold counter reads j.  After its last message the
integrator sends one ZM_DONE message to each other sampler.  Every wait is
bounded: one that runs out sets the block's abort flag, which ends the
other warps' waits.

This model runs the same sequence of waits, arrivals and stores for each
warp as the kernel, under many random interleavings of the four warps, and
checks what the kernel relies on: every message is read once, by its
sampler, after it was written and before its slot is reused; folds happen
in message order; every warp ends.  With the first message withheld (the
kernel's zone_wait_test switch) every warp ends through the wait limit
instead of hanging.  No GPU is involved.
"""

import random

import pytest

ZONE_SLOTS = 6
SAMPLERS = 3
WAIT_LIMIT = 400  # polls of a wait before it runs out (the kernel bounds by time)


class MBarrier:
    """mbarrier with an expected count of one arrival per warp (the kernel's
    32 per-lane arrivals of one warp complete a phase together)."""

    def __init__(self):
        self.completed = 0  # phases completed

    def arrive(self):
        self.completed += 1

    def test(self, parity):
        # the phase of parity `parity` has completed once the current
        # (incomplete) phase has the other parity
        return (self.completed & 1) != parity


class Block:
    def __init__(self, n_messages, withhold=False):
        self.full = [MBarrier() for _ in range(ZONE_SLOTS)]
        self.empty = [MBarrier() for _ in range(ZONE_SLOTS)]
        self.slot = [None] * ZONE_SLOTS
        self.folded = 0
        self.abort = False
        self.errors = 0
        self.n_messages = n_messages
        self.withhold = withhold
        self.read_log = []      # (sampler, message) in the order read
        self.fold_log = []      # messages in the order folded
        self.done = [False] * (1 + SAMPLERS)


def wait(block, cond):
    """A bounded wait (zone_wait / zone_wait_fold): yields while polling;
    returns False when the limit runs out or the block aborted."""
    for _ in range(WAIT_LIMIT):
        if cond():
            return True
        if block.abort:
            return False
        yield
    return False


def fail(block):
    block.abort = True
    block.errors += 1


def integrator(block):
    last = block.n_messages - 1
    for it in range(block.n_messages):
        sl = it % ZONE_SLOTS
        if it >= ZONE_SLOTS:
            ok = yield from wait(block, lambda: block.empty[sl].test(((it // ZONE_SLOTS) - 1) & 1))
            if not ok:
                fail(block)
                block.done[0] = True
                return
        assert block.slot[sl] is None, f"slot {sl} overwritten before message {it - ZONE_SLOTS} was read"
        block.slot[sl] = ("msg", it, it == last)
        yield
        if not (block.withhold and it == 0):
            block.full[sl].arrive()
        yield
    # one ZM_DONE message for each of the other samplers
    for e in range(1, SAMPLERS):
        jt = last + e
        se = jt % ZONE_SLOTS
        if jt >= ZONE_SLOTS:
            ok = yield from wait(block, lambda: block.empty[se].test(((jt // ZONE_SLOTS) - 1) & 1))
            if not ok:
                fail(block)
                block.done[0] = True
                return
        assert block.slot[se] is None
        block.slot[se] = ("msg", jt, True)
        yield
        block.full[se].arrive()
        yield
    block.done[0] = True


def sampler(block, k):
    j = k
    while True:
        sl = j % ZONE_SLOTS
        ok = yield from wait(block, lambda: block.full[sl].test((j // ZONE_SLOTS) & 1))
        if not ok:
            fail(block)
            block.done[1 + k] = True
            return
        kind, m, is_done = block.slot[sl]
        assert m == j, f"sampler {k} read message {m} in slot {sl}, expected {j}"
        block.read_log.append((k, j))
        block.slot[sl] = None       # read into registers
        yield
        block.empty[sl].arrive()    # the slot is free for message j + ZONE_SLOTS
        yield
        ok = yield from wait(block, lambda: block.folded == j)
        if not ok:
            fail(block)
            block.done[1 + k] = True
            return
        block.fold_log.append(j)
        yield
        block.folded = j + 1
        if is_done:
            block.done[1 + k] = True
            return
        j += SAMPLERS


def run(block, seed, max_ticks=200000):
    rng = random.Random(seed)
    warps = [integrator(block)] + [sampler(block, k) for k in range(SAMPLERS)]
    live = list(range(len(warps)))
    for _ in range(max_ticks):
        if not live:
            return True
        w = rng.choice(live)
        try:
            next(warps[w])
        except StopIteration:
            live.remove(w)
    return False


@pytest.mark.parametrize("n_messages", [1, 2, 3, 5, 6, 7, 12, 13, 40])
def test_every_message_read_once_folded_in_order(n_messages):
    for seed in range(60):
        b = Block(n_messages)
        assert run(b, seed), f"a warp did not end (n={n_messages}, seed={seed})"
        assert b.errors == 0 and not b.abort
        assert all(b.done)
        total = n_messages + SAMPLERS - 1  # the real messages and the extra ZM_DONE ones
        assert sorted(m for _, m in b.read_log) == list(range(total))
        assert all(m % SAMPLERS == k for k, m in b.read_log)
        assert b.fold_log == list(range(total))


def test_fresh_barrier_parity_rule():
    bar = MBarrier()
    assert bar.test(1) and not bar.test(0)  # the preceding (parity-1) phase counts as complete
    bar.arrive()
    assert bar.test(0) and not bar.test(1)
    bar.arrive()
    assert bar.test(1) and not bar.test(0)


@pytest.mark.parametrize("n_messages", [1, 7, 40])
def test_withheld_first_message_ends_through_the_wait_limit(n_messages):
    """The zone_wait_test switch: message 0's full barrier never completes.
    Sampler 0 waits on it until its limit runs out and aborts the block; the
    other warps' waits then end too, so every warp returns and the block
    reports its waits that ran out."""
    for seed in range(30):
        b = Block(n_messages, withhold=True)
        assert run(b, seed), f"a warp hung (n={n_messages}, seed={seed})"
        assert all(b.done)
        assert b.abort and b.errors >= 1
        assert 0 not in b.fold_log and all(m != 0 for _, m in b.read_log)
