"""CPU checks of the arithmetic claims the CRT kernels rely on (bachelor-thesis_gb300/csrc/crt.cu).

The kernels do modular reductions in FP32 and exact integer sums in FP32
accumulators; these tests restate each step with exact rationals and an explicit
round-to-nearest-even FP32 rounding, and check the bounds the kernels assume:

- red(x) = x - rint(x * fl(1/p)) * p (two roundings: the FMA with 1.5 * 2^23 and
  the final FMA) is congruent to x and lies in [-p/2 - 2, p/2 + 2] for |x| <= 2^24;
- bal_split(r) gives byte digits of magnitude <= 128 for |r| <= 32772;
- the epilogue combinations stay below 2^24 in magnitude;
- the reconstruction's per-limb 64-bit accumulation equals sum x_u 128^u;
- the 96-bit fixed-point sum decides q and the sign of C whenever
  |C| > Mod * 2^-76, for moduli chosen with an 18-bit margin.
"""
import math
import random
from fractions import Fraction as F

import numpy as np
import pytest

MAGIC = F(12582912)  # 1.5 * 2^23
FIXB = 96


def rnd32(x):
    """Round a rational to the nearest FP32 value (ties to even), no overflow."""
    x = F(x)
    if x == 0:
        return F(0)
    s = -1 if x < 0 else 1
    a = abs(x)
    e = a.numerator.bit_length() - a.denominator.bit_length()
    while F(2) ** e > a:
        e -= 1
    while F(2) ** (e + 1) <= a:
        e += 1
    ulp = F(2) ** (e - 23)
    q = a / ulp
    n = math.floor(q)
    r = q - n
    if r > F(1, 2) or (r == F(1, 2) and n % 2 == 1):
        n += 1
    return s * n * ulp


def red(x, p):
    inv = rnd32(F(1, p))
    q = rnd32(rnd32(x * inv + MAGIC) - MAGIC)
    return rnd32(x - q * p)


def bal_split(r):
    hi = rnd32(rnd32(r * F(1, 256) + MAGIC) - MAGIC)
    lo = rnd32(r - 256 * hi)
    return hi, lo


def primes_desc(n):
    out, x = [], 65535
    while len(out) < n:
        if all(x % d for d in range(2, int(x ** 0.5) + 1)):
            out.append(x)
        x -= 1
    return out


PRIMES = primes_desc(1023)


def test_red_bounds_and_congruence():
    rng = random.Random(11)
    ps = PRIMES[:4] + PRIMES[-4:]
    for t in range(4000):
        p = rng.choice(ps)
        if t % 3 == 0:  # quotients near a half-integer, where rint may pick either side
            k = rng.randint(-255, 255)
            x = k * p + p // 2 + rng.randint(-2, 3)
        else:
            x = rng.randint(-(1 << 24), 1 << 24)
        x = max(-(1 << 24), min(1 << 24, x))
        r = red(F(x), p)
        assert r.denominator == 1 and (x - r) % p == 0
        assert abs(r) <= F(p, 2) + 2


def test_bal_split_digits():
    for r in list(range(-32772, -32600)) + list(range(-300, 300)) + list(range(32600, 32773)):
        hi, lo = bal_split(F(r))
        assert hi * 256 + lo == r and abs(hi) <= 128 and abs(lo) <= 128
        # the kernels take a digit's bf16 bits as the top half of its FP32 bits
        for d in (hi, lo):
            assert int(np.array([float(d)], dtype=np.float32).view(np.uint32)[0]) & 0xFFFF == 0


def _limb_digits_bal(w, cin, last):
    """Restatement of limb_digits_bal (csrc/crt.cu) step by step: x = w ^ 0x80808080,
    the carry bits c = ((w & 0x80808080) >> 7 << 8) | cin, the FP32 bits
    0x4B000000 + (x_i) + c_i, one FP32 subtraction of 2^23 + 128, and for the row's
    last digit +256 when its byte's top bit is set."""
    x = w ^ 0x80808080
    c = ((((w & 0x80808080) >> 7) << 8) | cin) & 0xFFFFFFFF
    out = []
    for i in range(4):
        bits = 0x4B000000 + ((x >> (8 * i)) & 255) + ((c >> (8 * i)) & 255)
        v = np.array([bits], dtype=np.uint32).view(np.float32)[0]
        d = np.float32(v) - np.float32(8388736.0)
        if last and i == 3 and (w >> 31):
            d = d + np.float32(256.0)
        d = float(d)
        assert d == int(d) and int(np.array([d], dtype=np.float32).view(np.uint32)[0]) & 0xFFFF == 0
        out.append(int(d))
    return out


@pytest.mark.parametrize("nlimbs,dxp", [(1, 64), (16, 64), (15, 64), (128, 512), (127, 512), (129, 576), (300, 1216)])
def test_balanced_digit_rows(nlimbs, dxp):
    """A digit row as k_crt_digits writes it: each limb's digits from its own bytes
    and the top bit of the limb below; the row's last digit unreduced.  The digits
    keep the value, lie in [-128, 128] (the last in [0, 256]), and the row's digits
    past 4 * nlimbs are zero but for one carry digit."""
    rng = random.Random(nlimbs * 7 + dxp)
    for kind in ("rand", "ones", "top"):
        limbs = [rng.getrandbits(32) for _ in range(nlimbs)]
        if kind == "ones":
            limbs = [0xFFFFFFFF] * nlimbs
        elif kind == "top":
            limbs = [0x80808080 | rng.getrandbits(32) for _ in range(nlimbs)]
        words = limbs + [0] * (dxp // 4 - nlimbs)
        digits = []
        for l, w in enumerate(words):
            cin = (words[l - 1] >> 31) if l > 0 else 0
            digits += _limb_digits_bal(w, cin, last=(4 * l + 4 == dxp))
        assert len(digits) == dxp
        x = sum(w << (32 * l) for l, w in enumerate(limbs))
        assert sum(d << (8 * i) for i, d in enumerate(digits)) == x
        assert all(-128 <= d <= 128 for d in digits[:-1]) and 0 <= digits[-1] <= 256
        assert all(d == 0 for d in digits[4 * nlimbs + 1:])


def test_epilogue_sums_stay_exact():
    # residue: 256 red(s1) + red(s0) + res; product: 256 red(D_hi) + red(D_lo)
    assert 256 * 32772 + 32772 + 32772 < 1 << 24
    # residue groups: 512 unsigned byte digits, or 960 balanced digits (|d| <= 128, the row's last digit <= 256)
    # against table digits |t| <= 128; product: 2k = 1024 terms of 128^2;
    # reconstruction: 2P = 2046 terms of 128 x 64
    assert 512 * 255 * 128 <= 1 << 24
    assert 959 * 128 * 128 + 256 * 128 < 1 << 24
    assert 960 == 15 * 64
    assert 1024 * 128 * 128 <= 1 << 24
    assert 2046 * 128 * 64 <= 1 << 24


def test_reconstruction_limb_accumulators():
    rng = random.Random(5)

    def i64(v):
        assert -(1 << 63) <= v < (1 << 63)
        return v

    for t in range(1500):
        nch = rng.randint(1, 4)
        lim = (1 << 24) - 1 if t % 2 else 300
        xs = [rng.randint(-lim, lim) for _ in range(32 * nch)]
        exact = sum(x * 128 ** u for u, x in enumerate(xs))
        carry, limbs = 0, []
        for c in range(nch):
            A = [carry] + [0] * 6
            for u in range(32):
                A[(7 * u) >> 5] = i64(A[(7 * u) >> 5] + xs[32 * c + u] * (1 << ((7 * u) & 31)))
            for li in range(7):
                if li < 6:
                    A[li + 1] = i64(A[li + 1] + (A[li] >> 32))
                limbs.append(A[li] & 0xFFFFFFFF)
            carry = A[6] >> 32
        val = sum(l << (32 * i) for i, l in enumerate(limbs)) + carry * (1 << (224 * nch))
        assert val == exact


def test_fixed_point_sign_and_quotient():
    rng = random.Random(3)
    P = 40
    pr = PRIMES[:P]
    Mod = 1
    for p in pr:
        Mod *= p
    wh = [((1 << (FIXB + 8)) + p // 2) // p for p in pr]
    wl = [((1 << FIXB) + p // 2) // p for p in pr]
    inv = [pow(Mod // p, -1, p) for p in pr]
    for t in range(600):
        mag = rng.choice([Mod >> 20, Mod >> 40, Mod >> 70, 1 << 20, 3])
        C = rng.randint(-mag, mag)
        S, X = 0, 0
        for i, p in enumerate(pr):
            y = (C * inv[i]) % p
            if y > p // 2:
                y -= p
            hi, lo = bal_split(F(y))
            S += int(hi) * wh[i] + int(lo) * wl[i]
            X += y * (Mod // p)
        q = (S + (1 << (FIXB - 1))) >> FIXB
        frac = S - (q << FIXB)
        assert X - q * Mod == C
        tol = 1 << 20
        if abs(frac) > tol:
            assert (frac < 0) == (C < 0)
        else:
            assert abs(C) <= Mod >> 75


def _balanced128(x, ndig):
    out, carry = [], 0
    for t in range(ndig):
        v = ((x >> (7 * t)) & 127) + carry
        d = v - 128 if v >= 64 else v
        carry = (v - d) // 128
        out.append(d)
    return out


def _chunk_words(md, n):
    """Mod's digits of 32-digit chunk n as the kernel's table: 7 words of the
    two's-complement value sum_u Mod_(32n+u) 128^u, plus the sign word."""
    v = sum(md[32 * n + u] * 128 ** u for u in range(32) if 32 * n + u < len(md))
    assert abs(v) < 1 << 223
    w = v & ((1 << 256) - 1)
    return [(w >> (32 * k)) & 0xFFFFFFFF for k in range(8)]


def test_reconstruction_epilogue_emulation():
    """The reconstruction epilogue restated on exact integers: column sums of
    y_i against Mod/p_i digits, q and the sign from the fixed-point columns,
    per-chunk subtraction of q Mod through the 7-word table, on-the-fly negation
    of negative results and the final carry rule."""
    rng = random.Random(8)
    P = 24
    pr = PRIMES[:P]
    Mod = 1
    for p in pr:
        Mod *= p
    modbits = 32 * ((Mod.bit_length() + 31) // 32)
    Dout = (modbits + 6) // 7 + 2
    md = _balanced128(Mod, Dout)
    nch = (Dout + 31) // 32
    vt = [_chunk_words(md, n) for n in range(nch)]
    tabs = []
    for p in pr:
        Mi = Mod // p
        tabs.append((_balanced128(256 * Mi, Dout), _balanced128(Mi, Dout),
                     ((1 << (FIXB + 8)) + p // 2) // p, ((1 << FIXB) + p // 2) // p))
    inv = [pow(Mod // p, -1, p) for p in pr]
    cases = [0, 1, -1, 5, -(1 << 40)] + [rng.randint(-(Mod >> 19), Mod >> 19) for _ in range(60)]
    cases += [rng.randint(-(Mod >> 90), Mod >> 90) for _ in range(20)]
    for C in cases:
        ys = []
        for i, p in enumerate(pr):
            y = (C * inv[i]) % p
            ys.append(y - p if y > p // 2 else y)
        dig = [bal_split(F(y)) for y in ys]
        S = sum(int(h) * tabs[i][2] + int(l) * tabs[i][3] for i, (h, l) in enumerate(dig))
        acc = [sum(int(h) * tabs[i][0][r] + int(l) * tabs[i][1][r] for i, (h, l) in enumerate(dig)) for r in range(Dout)]
        acc += [0] * (nch * 32 - Dout)
        q = (S + (1 << (FIXB - 1))) >> FIXB
        frac = S - (q << FIXB)
        sgn = -1 if frac < -(1 << 20) else 1
        carry, nc, limbs = 0, 1, []
        for n in range(nch):
            A = [carry] + [0] * 6
            for u in range(32):
                A[(7 * u) >> 5] += acc[32 * n + u] * (1 << ((7 * u) & 31))
            for k in range(7):
                A[k] -= q * vt[n][k]
            for k in range(7):
                if k < 6:
                    A[k + 1] += A[k] >> 32
                limb = A[k] & 0xFFFFFFFF
                if sgn < 0:
                    nl = (~limb + nc) & 0xFFFFFFFF
                    nc &= int(limb == 0)
                    limb = nl
                limbs.append(limb)
            carry = (A[6] >> 32) + (q if vt[n][7] else 0)
        if sgn < 0:
            carry = -carry - 1 + nc
        value = sum(l << (32 * i) for i, l in enumerate(limbs))
        if carry < 0:  # the undecided-sign path: two's complement, negated in place
            assert carry == -1 and abs(frac) <= 1 << 20
            value = value - (1 << (32 * len(limbs)))
        else:
            assert carry == 0
        assert (-value if sgn < 0 else value) == C
