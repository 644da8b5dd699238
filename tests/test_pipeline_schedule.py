"""Model check of the ring pipeline's schedule (tile_pipeline in
<pkg>/csrc/step_ring.cuh) on the CPU.

The kernel's block takes its tiles j = 0, 1, ... (tile blockIdx.x + j * gridDim.x); tile j goes
to stage j % kStages (use j / kStages of that stage) and is issued by producer warp j % kProd,
which first waits on the stage's `empty` barrier for the release of tile j - kStages (parity
(j / kStages - 1) & 1); the kW consumer warps take the tiles in order, wait on the stage's
`full` barrier (parity (j / kStages) & 1) and arrive on `empty` when done. An mbarrier parity
wait only tells the two most recent phases apart, so the schedule is correct only if no
barrier ever runs more than one phase ahead of a waiter. This test replays the schedule under
random interleavings of producers, consumers and copy completions, with barriers modelled as
phase counters, and checks: every tile issued once and consumed by every consumer warp in
order, every wait satisfied by exactly the phase it targets (never a later one), no deadlock,
and the single-producer loop's incremental stage / phase equal to the general formulas, for
kProd <= kStages (the kernel's requirement; with more producers than stages the model finds
interleavings where a parity wait would pass early). It also checks the producers' error-path
drain (the last kStages tiles a producer may still have in flight).
"""

import random

import pytest


def simulate(n_prod, n_stages, n_cons, n_tiles, seed):
    rng = random.Random(seed)
    full_done = [0] * n_stages   # completed phases of full[s]
    empty_done = [0] * n_stages  # completed phases of empty[s]
    empty_arr = [0] * n_stages   # arrivals in the current phase of empty[s]
    in_flight = []               # (stage, tile) copies issued, not landed
    issued = []
    prod_next = list(range(n_prod))
    cons_next = [0] * n_cons
    consumed = [[] for _ in range(n_cons)]

    def parity_ok(done, parity, expect_done):
        # try_wait.parity(P) succeeds once the phase of parity P completed; the model also
        # asserts that the barrier is exactly at the targeted phase, not beyond it.
        if (done & 1) == parity:  # current (incomplete) phase has parity P: wait
            return False
        assert done == expect_done, f"barrier ran ahead: {done} phases done, waiter expects {expect_done}"
        return True

    steps = 0
    while True:
        steps += 1
        assert steps < 10_000_000
        actions = []
        for p in range(n_prod):
            j = prod_next[p]
            if j >= n_tiles:
                continue
            s = j % n_stages
            if j >= n_stages:
                par = (j // n_stages - 1) & 1
                if (empty_done[s] & 1) == par:
                    continue
            actions.append(("prod", p))
        for w in range(n_cons):
            k = cons_next[w]
            if k >= n_tiles:
                continue
            s = k % n_stages
            if (full_done[s] & 1) == ((k // n_stages) & 1):
                continue
            actions.append(("cons", w))
        if in_flight:
            actions.append(("land", None))
        if not actions:
            break
        kind, who = rng.choice(actions)
        if kind == "prod":
            j = prod_next[who]
            s = j % n_stages
            if j >= n_stages:
                assert parity_ok(empty_done[s], (j // n_stages - 1) & 1, j // n_stages)
            assert full_done[s] == j // n_stages, "stage armed before its previous use completed"
            issued.append(j)
            in_flight.append((s, j))
            prod_next[who] += n_prod
        elif kind == "land":
            s, j = in_flight.pop(rng.randrange(len(in_flight)))
            assert full_done[s] == j // n_stages
            full_done[s] += 1
        else:
            k = cons_next[who]
            s = k % n_stages
            assert parity_ok(full_done[s], (k // n_stages) & 1, k // n_stages + 1)
            consumed[who].append(k)
            cons_next[who] += 1
            empty_arr[s] += 1
            if empty_arr[s] == n_cons:
                empty_arr[s] = 0
                empty_done[s] += 1
    assert sorted(issued) == list(range(n_tiles)), "every tile issued once"
    assert all(c == list(range(n_tiles)) for c in consumed), "no deadlock, tiles consumed in order"


@pytest.mark.parametrize("n_prod,n_stages", [(1, 1), (1, 2), (1, 3), (1, 4), (2, 2), (2, 3), (2, 4),
                                             (3, 3), (3, 4), (4, 4)])
def test_schedule_random_interleavings(n_prod, n_stages):
    for seed in range(12):
        for n_tiles in (0, 1, n_stages, n_stages + 1, 17, 40):
            simulate(n_prod, n_stages, n_cons=4, n_tiles=n_tiles, seed=seed * 101 + n_tiles)


@pytest.mark.parametrize("n_prod,n_stages", [(2, 1), (3, 2), (4, 3)])
def test_more_producers_than_stages_is_unsafe(n_prod, n_stages):
    # Why tile_pipeline requires kProd <= kStages: with more producers, some interleaving lets a
    # producer reach use n of a stage while its `empty` barrier is two phases behind, and the
    # parity wait would pass early.
    failures = 0
    for seed in range(40):
        try:
            simulate(n_prod, n_stages, n_cons=4, n_tiles=40, seed=seed)
        except AssertionError as e:
            assert "ran ahead" in str(e)
            failures += 1
    assert failures > 0


@pytest.mark.parametrize("n_stages", [1, 2, 3, 4])
def test_single_producer_incremental_form(n_stages):
    # The single-producer loop advances s and phase incrementally and waits from the
    # (kStages + 1)-th tile on; it must match stage j % kStages and parity (j / kStages - 1) & 1.
    s, issued, phase = 0, 0, 0
    for j in range(50):
        if issued >= n_stages:
            assert phase ^ 1 == (j // n_stages - 1) & 1
        assert s == j % n_stages
        s += 1
        issued += 1
        if s == n_stages:
            s, phase = 0, phase ^ 1


@pytest.mark.parametrize("n_prod,n_stages", [(1, 2), (1, 3), (2, 2), (2, 3), (2, 4), (3, 4)])
def test_error_drain_covers_in_flight_tiles(n_prod, n_stages):
    # After a failed wait, producer p drains j = last, last - kProd, ... while j > last - kStages:
    # exactly its tiles among the last kStages tiles of the block, the only ones whose stages it
    # may not have seen released.
    for p in range(n_prod):
        mine = list(range(p, 60, n_prod))
        for last in mine:
            drained = [j for j in range(last, -1, -n_prod) if j > last - n_stages]
            expect = [j for j in mine if last - n_stages < j <= last]
            assert sorted(drained) == expect
