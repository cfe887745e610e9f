"""The scheduling argument of the batch's line sweep queue (k_lines_queue), restated on the CPU.

The queue holds the line sweeps of every case of a batch: phases (one sweep colour, or one
wake-cut injection, of one case) in iteration order, each phase of every case before the next,
within a phase the largest cases first; a phase depends on the previous phase of its case.
Resident CTAs take items in queue order from a counter and wait until the item's dependency is
complete.  Because a dependency always comes earlier in the queue, the lowest item not done has
nothing left to wait for, so the queue empties for any number of resident CTAs.  This model
builds the phase table the way the C++ host does (smac_api.cu, batch_queue_tables) and runs the
protocol as a discrete-event simulation with random item times; it is a restatement of the
argument, not the kernel (the kernel is compared bit for bit with the packed layout by the GPU
tests).
"""
import heapq

import numpy as np
import pytest

SWEEP, BCIMP = 0, 1


def phase_table(cases, njsp=2, nksp=2, nbcimp=1):
    """cases: list of (jmax, kmax).  Returns phases as dicts: case, kind, dir, color, first,
    n (items), dep (phase index or -1)."""
    order = sorted(range(len(cases)), key=lambda i: -cases[i][0] * cases[i][1])  # stable: largest first
    phases, nitems, last = [], 0, [-1] * len(cases)

    def add(kind, i, d, col, n):
        nonlocal nitems
        phases.append(dict(case=i, kind=kind, dir=d, color=col, first=nitems, n=n, dep=last[i]))
        nitems += n
        last[i] = len(phases) - 1

    for d, nsp in ((0, njsp), (1, nksp)):
        for sw in range(1, nsp + 1):
            col = 0 if sw & 1 else 1
            for cc in (col, 1 - col):
                for i in order:
                    nl = cases[i][1] if d == 0 else cases[i][0]
                    add(SWEEP, i, d, cc, (nl - cc + 1) // 2)
            if (sw // nbcimp) * nbcimp == sw:
                for i in order:
                    add(BCIMP, i, d, 0, 1)
    return phases, nitems


def simulate(phases, nitems, nctas, rng):
    """CTAs take the next item when free; an item whose dependency is not complete waits (its CTA
    is held).  Returns the start and end time of every item and the completion time of every
    phase; raises if the simulation stalls."""
    first = np.array([p["first"] for p in phases])
    phase_of = np.searchsorted(first, np.arange(nitems), side="right") - 1
    left = [p["n"] for p in phases]
    done_at = [None] * len(phases)
    start, end = np.full(nitems, np.nan), np.full(nitems, np.nan)
    head, t = 0, 0.0
    free = list(range(nctas))
    waiting = []   # (cta, item): taken, dependency not complete
    running = []   # heap of (end time, cta, item)
    while head < nitems or waiting or running:
        while free and head < nitems:  # free CTAs take items in queue order
            waiting.append((free.pop(), head))
            head += 1
        still = []
        for cta, item in waiting:      # start the items whose dependency is complete
            dep = phases[phase_of[item]]["dep"]
            if dep < 0 or done_at[dep] is not None:
                start[item] = t
                heapq.heappush(running, (t + rng.uniform(0.1, 3.0), cta, item))
            else:
                still.append((cta, item))
        waiting = still
        if not running:
            raise AssertionError(f"stalled with {len(waiting)} waiting items at item {head} of {nitems}")
        t, cta, item = heapq.heappop(running)
        end[item] = t
        ph = phase_of[item]
        left[ph] -= 1
        if left[ph] == 0:
            done_at[ph] = t
        free.append(cta)
    return start, end, done_at, phase_of


def test_every_dependency_precedes_its_phase():
    cases = [(79, 21), (119, 31), (241, 61), (119, 31), (481, 121), (961, 241)]
    phases, nitems = phase_table(cases)
    assert sum(p["n"] for p in phases) == nitems
    for k, p in enumerate(phases):
        assert p["dep"] < k
        if p["dep"] >= 0:
            assert phases[p["dep"]]["case"] == p["case"]
            assert phases[p["dep"]]["first"] + phases[p["dep"]]["n"] <= p["first"]
    # within a phase of the iteration the cases come largest first
    firsts = [p for p in phases if p["kind"] == SWEEP and p["dir"] == 0 and p["color"] == 0][:len(cases)]
    sizes = [cases[p["case"]][0] * cases[p["case"]][1] for p in firsts]
    assert sizes == sorted(sizes, reverse=True)


@pytest.mark.parametrize("nctas", [1, 2, 7, 64, 1000])
def test_queue_empties_for_any_number_of_resident_ctas(nctas):
    rng = np.random.default_rng(nctas)
    cases = [(79, 21), (119, 31), (241, 61), (119, 31), (481, 121)]
    phases, nitems = phase_table(cases)
    start, end, done_at, phase_of = simulate(phases, nitems, nctas, rng)
    assert not np.isnan(end).any() and all(d is not None for d in done_at)
    # no item starts before its dependency phase is complete
    for item in range(nitems):
        dep = phases[phase_of[item]]["dep"]
        if dep >= 0:
            assert start[item] >= done_at[dep]
