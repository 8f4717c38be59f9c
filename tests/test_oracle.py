"""The CPU oracle against the golden fixtures (made by the reference's own
mat-cpu and Python integers) and against Python integers on random cases."""
import random

import numpy as np
import pytest

from conftest import golden_cases, load_golden


@pytest.mark.parametrize("name", golden_cases())
@pytest.mark.parametrize("method", [1, 3, 31, 35])
def test_oracle_matches_golden(oracle, name, method):
    text, expect = load_golden(name)
    out, _ = oracle.matmul_text(text, method=method, basesz=4 if method != 1 else 32, jobsz=16, nthreads=2)
    assert out == expect


@pytest.mark.parametrize("name", ["cfg1_like_16x16x16_1024b", "rect_7x13x5_zeros", "allones_8x8x8_256b"])
def test_oracle_gmp_backend_matches_golden(oracle, name):
    if not oracle.gmp_available():
        pytest.skip("libgmp.so.10 not present")
    text, expect = load_golden(name)
    assert oracle.set_backend(1)
    try:
        out, _ = oracle.matmul_text(text, method=35, basesz=4, nthreads=1)
    finally:
        oracle.set_backend(0)
    assert out == expect


def test_oracle_against_reference_cli(oracle):
    if not oracle.ref_cli_available():
        pytest.skip("reference mat-cpu not built here")
    rng = random.Random(5)
    K, M, N = 5, 9, 4
    A = [rng.getrandbits(333) * rng.choice((-1, 1)) for _ in range(K * M)]
    B = [rng.getrandbits(200) * rng.choice((-1, 1)) for _ in range(M * N)]
    import gbmm
    text = f"{K} {M} {N}\n" + gbmm.format_matrix(K, M, A) + gbmm.format_matrix(M, N, B)
    assert oracle.matmul_text(text, method=1)[0] == oracle.run_ref_cli(text, method=1)


def _planes(vals, nl):
    import gbmm
    return gbmm.ints_to_planes(vals, nl)


def test_oracle_planes_and_accumulate(oracle):
    import gbmm
    rng = random.Random(11)
    K, M, N = 6, 7, 5
    A = [rng.getrandbits(rng.randint(0, 250)) * rng.choice((-1, 1)) for _ in range(K * M)]
    B = [rng.getrandbits(rng.randint(0, 250)) * rng.choice((-1, 1)) for _ in range(M * N)]
    C0 = [rng.getrandbits(300) * rng.choice((-1, 1)) for _ in range(K * N)]
    Ap, Bp = _planes(A, 8), _planes(B, 8)
    Cl, Cs = oracle.matmul_planes(K, M, N, Ap, Bp, 20, method=35, basesz=2)
    got = gbmm.planes_to_ints(Cl, Cs)
    exp = [sum(A[y * M + k] * B[k * N + x] for k in range(M)) for y in range(K) for x in range(N)]
    assert got == exp
    Cl, Cs = oracle.matmul_planes(K, M, N, Ap, Bp, 20, C=_planes(C0, 20))
    assert gbmm.planes_to_ints(Cl, Cs) == [c + e for c, e in zip(C0, exp)]


def test_oracle_mpn_ops(oracle):
    rng = np.random.default_rng(3)
    n, nb = 9, 37
    u = rng.integers(0, 2**32, size=(n, nb), dtype=np.uint64).astype(np.uint32)
    v = rng.integers(0, 2**32, size=(n, nb), dtype=np.uint64).astype(np.uint32)
    u[:, 0] = 0xFFFFFFFF
    v[:, 0] = 1
    def val(p, b):
        return int.from_bytes(np.ascontiguousarray(p[:, b]).tobytes(), "little")
    r, cy = oracle.mpn_add_n(u, v)
    for b in range(nb):
        assert val(r, b) + (int(cy[b]) << (32 * n)) == val(u, b) + val(v, b)
    r, cy = oracle.mpn_add_n(u, v, sub=True)
    for b in range(nb):
        assert val(r, b) - (int(cy[b]) << (32 * n)) == val(u, b) - val(v, b)
    vl = rng.integers(0, 2**32, size=nb, dtype=np.uint64).astype(np.uint32)
    for op in (0, 1, 2):
        r0 = rng.integers(0, 2**32, size=(n, nb), dtype=np.uint64).astype(np.uint32)
        r, cy = oracle.mpn_mul1ops(op, r0, u, vl)
        for b in range(nb):
            x = val(u, b) * int(vl[b])
            if op == 0:
                assert val(r, b) + (int(cy[b]) << (32 * n)) == x
            elif op == 1:
                assert val(r, b) + (int(cy[b]) << (32 * n)) == val(r0, b) + x
            else:
                assert val(r, b) - (int(cy[b]) << (32 * n)) == val(r0, b) - x
    w = oracle.mpn_mul_basecase(u, v[:4])
    for b in range(nb):
        assert val(w, b) == val(u, b) * val(v[:4], b)


def _val(planes, b):
    return int.from_bytes(np.ascontiguousarray(planes[:, b]).tobytes(), "little")


def test_oracle_mpn_rest_against_python_ints(oracle):
    """The oracle's restatement of mpn_add / sub / add_1 / sub_1 / cmp / zero_p /
    neg / com against Python integer arithmetic (GMP semantics: results mod
    2^(32 n), carries and borrows as 0/1, cmp as -1/0/1, neg's flag 1 unless the
    operand is zero)."""
    rng = np.random.default_rng(4)
    un, vn, nb = 9, 4, 300
    u = rng.integers(0, 2**32, size=(un, nb), dtype=np.uint64).astype(np.uint32)
    v = rng.integers(0, 2**32, size=(vn, nb), dtype=np.uint64).astype(np.uint32)
    u[:, :20] = 0xFFFFFFFF
    u[:, 20:40] = 0
    u[0, 30:40] = 1
    vl = rng.integers(0, 2**32, size=nb, dtype=np.uint64).astype(np.uint32)
    vl[:10] = 0
    mod = 1 << (32 * un)
    for sub in (False, True):
        r, cy = oracle.mpn_addsub(u, v, sub=sub)
        r1, cy1 = oracle.mpn_addsub_1(u, vl, sub=sub)
        for b in range(nb):
            x, y = _val(u, b), _val(v, b)
            t = x - y if sub else x + y
            assert _val(r, b) == t % mod and cy[b] == (t < 0 if sub else t >= mod)
            t = x - int(vl[b]) if sub else x + int(vl[b])
            assert _val(r1, b) == t % mod and cy1[b] == (t < 0 if sub else t >= mod)
    w = u.copy()
    w[:, ::3] = u[:, ::3]
    w[5, 1::3] ^= 1
    res = oracle.mpn_cmp(u, w)
    zp = oracle.mpn_zero_p(u)
    ng, nz = oracle.mpn_neg_com(u)
    cm, _ = oracle.mpn_neg_com(u, com=True)
    for b in range(nb):
        x, y = _val(u, b), _val(w, b)
        assert res[b] == (x > y) - (x < y)
        assert zp[b] == (x == 0)
        assert _val(ng, b) == (-x) % mod and nz[b] == (x != 0)
        assert _val(cm, b) == mod - 1 - x


@pytest.mark.parametrize("gmp", [0, 1])
@pytest.mark.parametrize("method", [1, 31])
def test_oracle_row_samples_match_full_product(oracle, method, gmp):
    """The benchmark's bounded CPU samples (rows of C by the naive order, or one
    block row by -m 31's block products with Winograd leaves) equal those rows
    of the full product."""
    if gmp and not oracle.gmp_available():
        pytest.skip("libgmp.so.10 not available")
    rng = random.Random(method + 10 * gmp)
    K, M, N, bits, bs = 128, 128, 128, 300, 64
    nl = (bits + 31) // 32
    vals = lambda n: [rng.getrandbits(bits) * rng.choice((-1, 1)) if rng.random() > 0.05 else 0 for _ in range(n)]
    import gbmm
    A = gbmm.ints_to_planes(vals(K * M), nl)
    B = gbmm.ints_to_planes(vals(M * N), nl)
    cn = 2 * nl + 2
    full_l, full_s = oracle.matmul_planes(K, M, N, A, B, cn, method=1)
    oracle.set_backend(gmp)
    try:
        secs, (cl, cs) = oracle.sample_rows(K, M, N, A, B, 64, bs, method=method, basesz=16, jobsz=bs, nthreads=3,
                                            cn=cn)
    finally:
        oracle.set_backend(0)
    assert secs >= 0
    assert (cs == full_s[64 * N:(64 + bs) * N]).all()
    assert (cl == full_l[:, 64 * N:(64 + bs) * N]).all()
