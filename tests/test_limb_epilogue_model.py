"""CPU restatement of the per-entry product kernel's warp-parallel carry
resolution (resolve_store_warp in csrc/limb.cu), run on exact integers with
64-bit two's-complement wrap made explicit.  It checks the algorithm itself:
lane segments formed from carry-in 0, the 31-step chain that corrects each
lane's carry-out by floor((r + c) / 2^(32 len)), the sign, the ballot-driven
negation and the normalized size, against the exact value of the column sums
(plus the old C for C += A*B), including carries that ripple across whole
lanes, values that cancel to zero or to -1, one-limb last segments and sums
that do not fit (which must be flagged)."""
import random

import pytest

M64 = (1 << 64) - 1


def s64(x):
    x &= M64
    return x - (1 << 64) if x >> 63 else x


def resolve_model(col, Lc, LB, old=0, nlimbs=None):
    """col: list of (s0, s1, s2) for t < Lc.  Returns (status, value) with status
    'ok' or 'capacity'; value is the stored signed integer."""
    nlimbs = LB if nlimbs is None else nlimbs
    cn = (abs(old).bit_length() + 31) // 32
    if cn > LB or cn > nlimbs:
        return "capacity", None
    old_limbs = [(abs(old) >> (32 * t)) & 0xFFFFFFFF for t in range(cn)]
    S = max(2, (LB + 31) // 32)
    buf = [0] * LB
    lanes = []
    for lane in range(32):
        t0 = min(lane * S, LB)
        t1 = min(t0 + S, LB)
        q = 0
        for t in range(t0, t1):
            w0, w1, w2 = col[t] if t < Lc else (0, 0, 0)
            extra = 0
            if t < cn:
                extra = -old_limbs[t] if old < 0 else old_limbs[t]
            lo = s64((w0 & 0xFFFFFFFF) + (q & 0xFFFFFFFF) + extra)
            buf[t] = lo & 0xFFFFFFFF
            q = s64((lo >> 32) + (q >> 32) + (w0 >> 32) + w1 + s64(w2 << 32))
        lanes.append((t0, t1, q))

    def carry_out(lane, c):
        t0, t1, q = lanes[lane]
        if t0 >= t1:
            return c
        if t1 - t0 == 1:
            return s64(q + ((buf[t0] + c) >> 32))
        low64 = buf[t0] | (buf[t0 + 1] << 32)
        hi = buf[t0 + 2:t1]
        if c >= 0:
            return q + (1 if (low64 + c > M64 and all(x == 0xFFFFFFFF for x in hi)) else 0)
        return q - (1 if (low64 < -c and all(x == 0 for x in hi)) else 0)

    cin = [0] * 32
    for l in range(31):
        cin[l + 1] = carry_out(l, cin[l])
    for l in range(32):
        assert abs(cin[l]) < 1 << 53
    fin = carry_out(31, cin[31])
    if fin not in (0, -1):
        return "capacity", None
    for l in range(32):
        t0, t1, _ = lanes[l]
        c = cin[l]
        for t in range(t0, t1):
            lo = buf[t] + (c & 0xFFFFFFFF)
            buf[t] = lo & 0xFFFFFFFF
            c = (lo >> 32) + (c >> 32)
    neg = fin < 0
    if neg:
        zmask = [all(buf[t] == 0 for t in range(lanes[l][0], lanes[l][1])) for l in range(32)]
        for l in range(32):
            c1 = 1 if all(zmask[:l]) else 0
            for t in range(lanes[l][0], lanes[l][1]):
                v = (~buf[t] + c1) & 0xFFFFFFFF
                c1 = 1 if (c1 and v == 0) else 0
                buf[t] = v
    top = max([t + 1 for t in range(LB) if buf[t]], default=0)
    if top > nlimbs:
        return "capacity", None
    mag = sum(buf[t] << (32 * t) for t in range(top))
    return "ok", -mag if neg else mag


def exact(col, old=0):
    return old + sum((s0 + (s1 << 32) + (s2 << 64)) << (32 * t) for t, (s0, s1, s2) in enumerate(col))


def check(col, Lc, LB, old=0, nlimbs=None):
    st, v = resolve_model(col, Lc, LB, old, nlimbs)
    e = exact(col, old)
    fits = abs(e) < 1 << (32 * min(LB, LB if nlimbs is None else nlimbs))
    if st == "ok":
        assert v == e
    else:
        assert not fits or abs(e) >= 1 << (32 * LB - 1), (e, LB)


@pytest.mark.parametrize("Lc", [2, 4, 20, 40, 63, 64, 130, 256, 272])
def test_random_column_sums(Lc):
    rng = random.Random(Lc)
    LB = Lc + 2
    for _ in range(60):
        nterms = rng.choice([1, 17, 300, 4000])
        col = []
        for t in range(Lc):
            s0 = rng.randrange(nterms << 32)
            s1 = rng.randrange(nterms << 32)
            s2 = rng.randrange(-nterms, nterms + 1)
            col.append((s0, s1, s2))
        check(col, Lc, LB)
        old = rng.randrange(-(1 << (32 * Lc)), 1 << (32 * Lc))
        check(col, Lc, LB, old=old)


def _cols_for(value, Lc, rng, spread=True):
    """Column sums whose total is `value`: each column holds (s0, s1, s2) with an
    arbitrary split, so carries between columns are large and of either sign."""
    col = []
    rest = value
    for t in range(Lc):
        if t == Lc - 1:
            v = rest >> (32 * t)
            s2, r = divmod(v, 1 << 64)
            s1, s0 = divmod(r, 1 << 32)
            col.append((s0, s1, s2))
            rest -= v << (32 * t)
            break
        lim = 1 << 70 if spread else 1 << 32
        v = (rest >> (32 * t)) & 0xFFFFFFFF
        k = rng.randrange(-(lim >> 40), (lim >> 40) + 1)
        v += k << 32          # borrow from / lend to the next column
        s2, r = divmod(v, 1 << 64)
        s1, s0 = divmod(r, 1 << 32)
        col.append((s0, s1, s2))
        rest -= v << (32 * t)
    assert rest == 0 and exact(col) == value
    return col


@pytest.mark.parametrize("Lc", [4, 30, 62, 130, 258])
def test_adversarial_values(Lc):
    """Totals that make carries ripple through whole lane segments: zero, -1,
    2^k - 1, -2^k, values with long runs of all-ones or all-zero limbs."""
    rng = random.Random(100 + Lc)
    LB = Lc + 2
    bits = 32 * (Lc + 1)
    vals = [0, -1, 1, (1 << bits) - 1, -(1 << bits) + 1, -(1 << (bits - 7)), 1 << 32, -(1 << 64)]
    for k in range(0, bits, 37):
        vals += [(1 << k) - 1, -(1 << k), (1 << k), -((1 << k) - 1)]
        ones = ((1 << bits) - 1) ^ ((1 << k) - 1)
        vals += [ones, -ones, ones | 5, -(ones | 5)]
    for v in vals:
        for spread in (False, True):
            col = _cols_for(v, Lc, rng, spread)
            st, got = resolve_model(col, Lc, LB)
            assert st == "ok" and got == v, (v, spread)


def test_capacity_flags():
    """A result with more limbs than C holds is flagged (column sums with bounded
    high words always fit the LB = Lc + 2 limbs the kernel resolves)."""
    rng = random.Random(5)
    Lc, LB = 10, 12
    col = _cols_for(1 << (32 * 5), Lc, rng)
    assert resolve_model(col, Lc, LB, nlimbs=5)[0] == "capacity"
    assert resolve_model(col, Lc, LB, nlimbs=6) == ("ok", 1 << 160)
