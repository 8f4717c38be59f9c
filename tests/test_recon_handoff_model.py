"""Model check of the reconstruction epilogue's hand-off protocol (k_crt_recon in
bachelor-thesis_gb300/csrc/crt.cu), on the CPU.

Two epilogue warps share a TMEM lane quadrant: half 0 takes the low 128 columns of
each N tile, half 1 the high 128.  They pass values through per-entry shared-memory
slots guarded by single-arrival mbarriers:

- qready: half 0's fixed-point quotient and sign of an entry tile (slot q);
- to1: half 0's carry of an N tile (slot carry1; top0 after an entry's last N tile);
- to0: half 1's carry to half 0's next N tile (slot carry0).

The model replays both halves' operation sequences for one CTA under random
interleavings.  Barrier waits follow mbarrier parity semantics: a waiter that has
consumed `ph` phases tests parity ph & 1, so a barrier two phases ahead looks
incomplete (aliasing).  A read must see the value written for its own tile and N
tile.  The protocol the kernel uses is checked to be free of overwrites, aliasing
and deadlock; the order it replaced is shown to break for one N tile per entry tile.
The grouped form (entry tiles of several products, so N-tile counts that vary
from tile to tile) is checked on random tile sequences.
"""
import random

import pytest


def half0_ops(nts, mode):
    """nts: the N-tile count of each entry tile of the CTA.  mode: "old" (the
    order the kernel replaced), "fixed" (the kernel's single-product form: the
    early take when an entry tile has one N tile) or "uni" (the grouped form: the
    early take at every entry tile but the first)."""
    ops, first = [], True
    for t, NT in enumerate(nts):
        uni = mode == "uni" or (mode == "fixed" and NT == 1)
        for j in range(NT):
            took0 = False
            if j == 0:
                if not first and uni:
                    ops.append(("wait", "to0"))
                    took0 = True
                ops.append(("write", "q", t))
                ops.append(("arrive", "qready"))
            if not first and not took0:
                ops.append(("wait", "to0"))
                if j > 0:
                    ops.append(("read", "carry0", (t, j - 1)))
            first = False
            ops.append(("write", "carry1", (t, j)))
            if j == NT - 1:
                ops.append(("write", "top0", t))
            ops.append(("arrive", "to1"))
    return ops


def half1_ops(nts, mode):
    ops = []
    for t, NT in enumerate(nts):
        uni = mode == "uni" or (mode == "fixed" and NT == 1)
        last_t = t == len(nts) - 1
        for j in range(NT):
            if j == 0:
                ops.append(("wait", "qready"))
                ops.append(("read", "q", t))
            ops.append(("wait", "to1"))
            ops.append(("read", "carry1", (t, j)))
            if j < NT - 1:
                ops.append(("write", "carry0", (t, j)))
            if mode != "old":
                if j < NT - 1 or (not uni and not last_t):
                    ops.append(("arrive", "to0"))
            elif not (last_t and j == NT - 1):
                ops.append(("arrive", "to0"))
        ops.append(("read", "top0", t))  # the finalize
        if mode != "old" and uni and not last_t:
            ops.append(("arrive", "to0"))
    return ops


def run(nts, mode, rng):
    """One random interleaving; returns None, or the first violation."""
    progs = [half0_ops(nts, mode), half1_ops(nts, mode)]
    pc = [0, 0]
    done = {"qready": 0, "to1": 0, "to0": 0}   # completed phases
    used = [dict(done), dict(done)]            # phases each half has waited for
    slots = {}
    bias = rng.random()                        # how much more often half 0 runs
    while pc[0] < len(progs[0]) or pc[1] < len(progs[1]):
        runnable = []
        for a in (0, 1):
            if pc[a] == len(progs[a]):
                continue
            op = progs[a][pc[a]]
            if op[0] == "wait":
                ahead = done[op[1]] - used[a][op[1]]
                if ahead >= 2:
                    return f"parity aliasing on {op[1]} (half {a})"
                if ahead == 0:
                    continue
            runnable.append(a)
        if not runnable:
            return "deadlock"
        a = runnable[0] if len(runnable) == 1 else (0 if rng.random() < bias else 1)
        op = progs[a][pc[a]]
        pc[a] += 1
        if op[0] == "wait":
            used[a][op[1]] += 1
        elif op[0] == "arrive":
            done[op[1]] += 1
        elif op[0] == "write":
            slots[op[1]] = op[2]
        elif slots.get(op[1]) != op[2]:
            return f"half {a} read {op[1]} = {slots.get(op[1])}, expected {op[2]}"
    # every arrival is consumed by the half that waits on that barrier
    waits = {"qready": used[1]["qready"], "to1": used[1]["to1"], "to0": used[0]["to0"]}
    if waits != done:
        return f"unconsumed arrivals: completed {done}, waited {waits}"
    return None


@pytest.mark.parametrize("NT", [1, 2, 3])
@pytest.mark.parametrize("T", [1, 2, 3, 5])
def test_protocol_is_safe(T, NT):
    rng = random.Random(1000 * T + NT)
    for _ in range(3000):
        err = run([NT] * T, "fixed", rng)
        assert err is None, (T, NT, err)


def test_replaced_order_breaks_for_one_table_tile():
    rng = random.Random(7)
    errors = {run([1] * 3, "old", rng) for _ in range(3000)} - {None}
    assert errors, "the model should expose the old order's race"
    # with more than one N tile the old order was already safe
    for NT in (2, 3):
        assert all(run([NT] * 3, "old", rng) is None for _ in range(3000))


def test_grouped_protocol_is_safe_for_any_tile_sequence():
    """A grouped launch hands one CTA entry tiles of different products, so the
    N-tile count changes from tile to tile; the grouped form stays safe."""
    rng = random.Random(11)
    for _ in range(400):
        nts = [rng.choice([1, 1, 2, 3, 5]) for _ in range(rng.randint(1, 6))]
        for _ in range(40):
            err = run(nts, "uni", rng)
            assert err is None, (nts, err)


def test_single_product_form_breaks_when_tile_counts_vary():
    """The single-product form relies on one N-tile count for every entry tile:
    a tile of several N tiles followed by one of a single N tile lets half 0
    overwrite the quotient slot before half 1 has read it."""
    rng = random.Random(5)
    errors = {run([2, 1, 1], "fixed", rng) for _ in range(3000)} - {None}
    assert errors
