"""The ordering rules of the persistent batch step kernel (k_batch_step in
natrix_gb300/csrc/batch.cu), checked on a model of its schedule.

The host lays a step out as a list of items, phase-major over all
simulations (build_step_items): for each phase, every simulation's items of
that phase (bands of rows, or sweep tiles).  Persistent CTAs claim items in
list order; an item waits until its simulation's previous phase has counted
all of its items; a CTA claims its next item while the current one runs and
holds its completion counts, up to four, sending them under one fence when
it holds four, before it waits on a counter that is not yet reached, and
when it leaves.

Random interleavings (random simulations, phase sequences, item counts and
durations, CTA counts) must:
  * start an item only after every item of its simulation's previous phase
    has finished;
  * finish (no two CTAs wait on each other's held counts).
Without the flush before a wait the same model deadlocks, which is why the
kernel flushes there."""
from __future__ import annotations

import random

import pytest

HOLD = 4  # completion counts a CTA holds before it flushes them


def make_step(rng):
    """Items (sim, phase) in list order and the item count per (sim, phase)."""
    n = rng.randint(1, 5)
    phases = 9
    seq = []
    for _ in range(n):
        q = [0, 1]
        q += [p for p in (2, 3, 4) if rng.random() < 0.5]  # vorticity / viscosity phases
        q += [5] + list(range(6, 6 + rng.randint(0, 2))) + [8]
        seq.append(sorted(set(q)))
    count = {(i, ph): rng.randint(1, 4) for i in range(n) for ph in seq[i]}
    order = list(range(n))
    rng.shuffle(order)
    items = []
    for ph in range(phases):
        for i in order:
            if ph in seq[i]:
                pos = seq[i].index(ph)
                prev = seq[i][pos - 1] if pos > 0 else None
                items += [(i, ph, prev)] * count[(i, ph)]
    return items, count


def simulate(items, count, ctas, rng, flush_before_wait=True):
    """One random schedule: None, or the first violation found."""
    total = len(items)
    counter = {k: 0 for k in count}   # counts sent
    finished = {k: 0 for k in count}  # items actually finished
    claim = 0
    # CTA: [item index or None, phase, work left, next claim, held counts]
    cta = []
    for _ in range(ctas):
        cta.append([claim if claim < total else None, "wait" if claim < total else "leave",
                    0, None, []])
        claim += 1

    def flush(c):
        for k in c[4]:
            counter[k] += 1
        c[4] = []

    def satisfied(j):
        i, ph, prev = items[j]
        return prev is None or counter[(i, prev)] >= count[(i, prev)]

    steps = 0
    while any(c[1] != "gone" for c in cta):
        steps += 1
        if steps > 200000:
            return "no progress"
        moves = []
        for n_, c in enumerate(cta):
            if c[1] in ("run", "leave"):
                moves.append(n_)
            elif c[1] == "wait":
                if satisfied(c[0]) or (flush_before_wait and c[4]):
                    moves.append(n_)
        if not moves:
            return "deadlock"
        n_ = rng.choice(moves)
        c = cta[n_]
        if c[1] == "leave":
            flush(c)
            c[1] = "gone"
            continue
        if c[1] == "wait":
            if not satisfied(c[0]):
                flush(c)  # a held count is sent before the CTA waits
                continue
            i, ph, prev = items[c[0]]
            if prev is not None and finished[(i, prev)] != count[(i, prev)]:
                return f"item {c[0]} of simulation {i} phase {ph} started early"
            c[1], c[2] = "run", rng.randint(1, 4)
            c[3] = claim if claim < total else None
            claim += 1
            continue
        c[2] -= 1
        if c[2] > 0:
            continue
        i, ph, _ = items[c[0]]
        finished[(i, ph)] += 1
        c[4].append((i, ph))
        if len(c[4]) == HOLD:
            flush(c)
        if c[3] is not None:
            c[0], c[1] = c[3], "wait"
        else:
            c[0], c[1] = None, "leave"
    if any(counter[k] != count[k] for k in count):
        return "counts lost"
    return None


@pytest.mark.parametrize("seed", range(30))
def test_batch_rules_hold_on_random_schedules(seed):
    rng = random.Random(seed)
    for _ in range(20):
        items, count = make_step(rng)
        ctas = rng.randint(1, len(items) + 2)
        err = simulate(items, count, ctas, rng)
        assert err is None, err


def test_without_flush_before_wait_it_deadlocks():
    rng = random.Random(2)
    found = None
    for _ in range(3000):
        items, count = make_step(rng)
        err = simulate(items, count, rng.randint(2, 6), rng, flush_before_wait=False)
        if err is not None:
            found = err
            break
    assert found == "deadlock"
