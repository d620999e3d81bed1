"""The mbarrier protocol of the tensor-core kernel (q1tsim_gb300/csrc/
fused_tc.cu, k_fused_tc), replayed on the CPU under random schedules.

The kernel's agents -- one loader warp, two storer warps taking alternate
tiles, NG consumer groups taking every NG-th tile -- share a ring of nst
stages through three mbarriers per stage (full, out, empty) and wait on
them by phase parity.  A parity wait cannot tell phase u from phase u-2: it
is only correct if the phase before the awaited one has completed when the
wait starts.  This model runs the agents' loops step by step, with mbarrier
phases, arrival counts and parity waits as the hardware defines them, and
checks at every successful wait that the awaited phase, and no other, is
the last completed one; that every tile is loaded, processed and stored
exactly once; and that the schedule never deadlocks.

Copies land asynchronously and in any order.  The storers and the groups
wait for the stage's previous store (its empty phase u-1) before they wait
for its out or full phase u.  Without the storers' wait, a storer that
runs ahead with an odd number of stages passes its out wait on phase u-2
(the stage's previous use belongs to the other storer); without the
groups' wait, a copy that lands before an earlier copy to the same stage
lets a group pass its full wait on phase u-2.  The model finds both
schedules, which is checked below too.
"""
import random

import pytest


class Barrier:
    def __init__(self, count):
        self.count = count
        self.pending = count
        self.phase = 0          # phases completed so far

    def arrive(self):
        assert self.pending > 0, "arrival on a completed phase"
        self.pending -= 1
        if self.pending == 0:
            self.phase += 1
            self.pending = self.count

    def test_wait(self, parity):
        # true when the phase of this parity before the current one completed
        return (self.phase & 1) != parity


class Aliased(Exception):
    pass


def simulate(ng, nst, ntiles, seed, storer_waits_empty=True, consumer_waits_empty=True):
    rng = random.Random(seed)
    full = [Barrier(1) for _ in range(nst)]
    empty = [Barrier(1) for _ in range(nst)]
    out = [Barrier(1) for _ in range(nst)]       # one arrival per group (128 threads in the kernel)
    stage_tile = [None] * nst                    # which tile a stage holds
    stored = []
    in_flight = []                               # copies issued, not landed: (stage, tile)

    def wait(bar, use):
        # a wait for phase `use` by parity; correct only if phase use-1 is done
        while not bar.test_wait(use & 1):
            yield
        if bar.phase != use + 1:
            raise Aliased(f"wait for phase {use} passed at {bar.phase} completed phases")

    def loader():
        s, u = 0, 0
        for i in range(ntiles):
            if u > 0:
                yield from wait(empty[s], u - 1)
            in_flight.append((s, i))             # arrive.expect_tx, then the copy
            yield
            s += 1
            if s == nst:
                s, u = 0, u + 1

    def storer(w):
        s, u = w, 0
        for i in range(w, ntiles, 2):
            if storer_waits_empty and u > 0:
                yield from wait(empty[s], u - 1)
            yield from wait(out[s], u)
            assert stage_tile[s] == i, (stage_tile[s], i)
            stored.append(i)
            yield                                # the store reads the stage
            empty[s].arrive()
            s += 2
            if s >= nst:
                s, u = s - nst, u + 1

    def copies():
        # copies land one at a time, in any order
        while True:
            if in_flight:
                s, i = in_flight.pop(rng.randrange(len(in_flight)))
                stage_tile[s] = i
                full[s].arrive()                 # the transaction count reaches zero
            yield

    def group(g):
        s, u = g, 0
        for i in range(g, ntiles, ng):
            if consumer_waits_empty and u > 0:
                yield from wait(empty[s], u - 1)
            yield from wait(full[s], u)
            assert stage_tile[s] == i, (stage_tile[s], i)
            for _ in range(rng.randint(1, 6)):   # work on the tile
                yield
            out[s].arrive()
            s += ng
            if s >= nst:
                s, u = s - nst, u + 1

    agents = [loader(), storer(0), storer(1)] + [group(g) for g in range(ng)]
    live = list(agents)
    landing = copies()
    steps = 0
    while live:
        a = rng.choice(live + [landing])
        steps += 1
        assert steps < 10 ** 6, "deadlock"
        try:
            next(a)
        except StopIteration:
            live.remove(a)
    assert sorted(stored) == list(range(ntiles))


@pytest.mark.parametrize("ng", [2, 4])
@pytest.mark.parametrize("nst", [3, 4, 5, 6, 7, 8])
def test_stage_ring_protocol_is_exact(ng, nst):
    if nst < ng + (1 if ng == 4 else 0):
        pytest.skip("the kernel launches this shape with more stages")
    for seed in range(300):
        simulate(ng, nst, ntiles=4 * nst + 7, seed=seed)


@pytest.mark.parametrize("storer,consumer,ng,nst", [(False, True, 4, 5), (False, True, 2, 5), (True, False, 4, 6)])
def test_without_the_empty_waits_a_parity_wait_aliases(storer, consumer, ng, nst):
    """Each empty wait is needed: without the storers' one, a storer that
    runs ahead passes its out wait on the wrong phase when the ring is odd;
    without the consumers' one, a copy that lands before an earlier copy
    to the same stage lets a group pass its full wait on the wrong phase."""
    found = False
    for seed in range(3000):
        try:
            simulate(ng, nst, ntiles=4 * nst + 7, seed=seed, storer_waits_empty=storer,
                     consumer_waits_empty=consumer)
        except (Aliased, AssertionError):
            found = True
            break
    assert found
