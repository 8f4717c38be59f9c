"""Parity of the plain limb path (batched mpn / mpz kernels, matrix add/sub, the
per-entry product kernel and the Winograd / Strassen / squarify recursions)
against the CPU oracle and the golden fixtures.  Integer work: bit-exact."""
import random

import numpy as np
import pytest

from conftest import golden_cases, load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def g(built_lib):
    import gbmm
    gbmm.default_handle()
    return gbmm


def _rand_planes(rng, n, nb, special=None):
    u = rng.integers(0, 2**32, size=(n, nb), dtype=np.uint64).astype(np.uint32)
    if special == "ones":
        u[:, : nb // 2] = 0xFFFFFFFF
    return u


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()


def _host(t):
    return t.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("nb", [70, 20000])  # warp carry-lookahead; one thread per operand
@pytest.mark.parametrize("n", [1, 3, 31, 32, 128, 129, 300])
@pytest.mark.parametrize("sub", [False, True])
def test_mpn_add_sub_n_cla(g, oracle, n, sub, nb):
    import torch
    rng = np.random.default_rng(n + 7 * sub + nb)
    u = _rand_planes(rng, n, nb, "ones")
    v = _rand_planes(rng, n, nb)
    v[:, :8] = 0 if sub else 1          # long carry / borrow chains
    v[0, :8] = 1
    if sub:
        u[:, 8:16] = 0                   # borrow through all-zero limbs
    exp_r, exp_c = oracle.mpn_add_n(u, v, sub=sub)
    du, dv, dr = _dev(torch, u), _dev(torch, v), torch.zeros(n * nb, dtype=torch.int32, device="cuda")
    cy = torch.zeros(nb, dtype=torch.int32, device="cuda")
    (g.mpn_sub_n if sub else g.mpn_add_n)(dr, du, dv, n, nb, nb, cy)
    torch.cuda.synchronize()
    assert (_host(dr).reshape(n, nb) == exp_r).all()
    assert (_host(cy) == exp_c).all()


@pytest.mark.parametrize("op", [0, 1, 2])
def test_mpn_mul1ops(g, oracle, op):
    import torch
    rng = np.random.default_rng(op)
    n, nb = 17, 300
    u = _rand_planes(rng, n, nb, "ones")
    r0 = _rand_planes(rng, n, nb)
    vl = rng.integers(0, 2**32, size=nb, dtype=np.uint64).astype(np.uint32)
    vl[:5] = 0xFFFFFFFF
    exp_r, exp_c = oracle.mpn_mul1ops(op, r0, u, vl)
    dr, du, dvl = _dev(torch, r0), _dev(torch, u), _dev(torch, vl)
    cy = torch.zeros(nb, dtype=torch.int32, device="cuda")
    [g.mpn_mul_1, g.mpn_addmul_1, g.mpn_submul_1][op](dr, du, n, dvl, nb, nb, cy)
    torch.cuda.synchronize()
    assert (_host(dr).reshape(n, nb) == exp_r).all()
    assert (_host(cy) == exp_c).all()


@pytest.mark.parametrize("un,vn", [(1, 0), (1, 1), (7, 3), (33, 33), (130, 2)])
@pytest.mark.parametrize("sub", [False, True])
def test_mpn_add_sub_unequal(g, oracle, un, vn, sub):
    import torch
    rng = np.random.default_rng(un * 13 + vn + sub)
    nb = 700
    u = _rand_planes(rng, un, nb, "ones")
    v = _rand_planes(rng, max(vn, 1), nb)[:vn]
    if sub:
        u[:, nb // 2: nb // 2 + 20] = 0       # borrow through zero limbs
    exp_r, exp_c = oracle.mpn_addsub(u, v, sub=sub)
    dr, cy = torch.zeros(un * nb, dtype=torch.int32, device="cuda"), torch.zeros(nb, dtype=torch.int32, device="cuda")
    dv = _dev(torch, v) if vn else torch.zeros(1, dtype=torch.int32, device="cuda")
    (g.mpn_sub if sub else g.mpn_add)(dr, _dev(torch, u), un, dv, vn, nb, nb, cy)
    torch.cuda.synchronize()
    assert (_host(dr).reshape(un, nb) == exp_r).all()
    assert (_host(cy) == exp_c).all()


@pytest.mark.parametrize("n", [1, 5, 64])
@pytest.mark.parametrize("sub", [False, True])
def test_mpn_add_sub_1(g, oracle, n, sub):
    import torch
    rng = np.random.default_rng(n + 100 * sub)
    nb = 500
    u = _rand_planes(rng, n, nb, "ones")
    u[:, 300:350] = 0
    vl = rng.integers(0, 2**32, size=nb, dtype=np.uint64).astype(np.uint32)
    vl[:7] = 0
    vl[250:260] = 0xFFFFFFFF
    exp_r, exp_c = oracle.mpn_addsub_1(u, vl, sub=sub)
    du = _dev(torch, u)
    cy = torch.zeros(nb, dtype=torch.int32, device="cuda")
    (g.mpn_sub_1 if sub else g.mpn_add_1)(du, du, n, _dev(torch, vl), nb, nb, cy)   # in place, as GMP allows
    torch.cuda.synchronize()
    assert (_host(du).reshape(n, nb) == exp_r).all()
    assert (_host(cy) == exp_c).all()


@pytest.mark.parametrize("n", [1, 3, 129])
def test_mpn_cmp_zero_p_neg_com(g, oracle, n):
    import torch
    rng = np.random.default_rng(n)
    nb = 600
    u = _rand_planes(rng, n, nb, "ones")
    u[:, 400:450] = 0
    u[0, 420:430] = 5
    w = u.copy()
    w[n - 1, 1::4] ^= 8
    w[0, 2::4] += 1
    exp_cmp = oracle.mpn_cmp(u, w)
    exp_z = oracle.mpn_zero_p(u)
    exp_neg, exp_nz = oracle.mpn_neg_com(u)
    exp_com, _ = oracle.mpn_neg_com(u, com=True)
    du, dw = _dev(torch, u), _dev(torch, w)
    res = torch.zeros(nb, dtype=torch.int32, device="cuda")
    g.mpn_cmp(du, dw, n, nb, nb, res)
    torch.cuda.synchronize()
    assert (res.cpu().numpy() == exp_cmp).all()
    g.mpn_zero_p(du, n, nb, nb, res)
    torch.cuda.synchronize()
    assert (res.cpu().numpy() == exp_z).all()
    dr, cy = torch.zeros(n * nb, dtype=torch.int32, device="cuda"), torch.zeros(nb, dtype=torch.int32, device="cuda")
    g.mpn_neg(dr, du, n, nb, nb, cy)
    torch.cuda.synchronize()
    assert (_host(dr).reshape(n, nb) == exp_neg).all() and (_host(cy) == exp_nz).all()
    g.mpn_com(dr, du, n, nb, nb)
    torch.cuda.synchronize()
    assert (_host(dr).reshape(n, nb) == exp_com).all()


@pytest.mark.parametrize("un,vn", [(1, 1), (5, 3), (32, 32), (64, 17), (100, 100)])
def test_mpn_mul_basecase(g, oracle, un, vn):
    import torch
    rng = np.random.default_rng(un * 1000 + vn)
    nb = 64
    u = _rand_planes(rng, un, nb, "ones")
    v = _rand_planes(rng, vn, nb, "ones")
    exp = oracle.mpn_mul_basecase(u, v)
    dr = torch.zeros((un + vn) * nb, dtype=torch.int32, device="cuda")
    g.mpn_mul_basecase(dr, _dev(torch, u), un, _dev(torch, v), vn, nb, nb)
    torch.cuda.synchronize()
    assert (_host(dr).reshape(un + vn, nb) == exp).all()


@pytest.mark.parametrize("an,bn", [(2, 2), (3, 2), (3, 3), (8, 5), (40, 40), (41, 40), (128, 128), (127, 100), (9, 6)])
def test_mpn_toom22_and_mul(g, oracle, an, bn):
    import torch
    rng = np.random.default_rng(an * 7 + bn)
    nb = 40
    a = _rand_planes(rng, an, nb, "ones")
    b = _rand_planes(rng, bn, nb, "ones")
    a[:, 3] = 0
    a[an - 1, 3] = 1
    exp = oracle.mpn_mul_basecase(a, b)
    dp = torch.zeros((an + bn) * nb, dtype=torch.int32, device="cuda")
    s, n = an >> 1, an - (an >> 1)
    if 0 < bn - n <= s:  # GMP's toom22 preconditions (toom22_mul.cu:134-135)
        scratch = torch.zeros(g.mpn_toom22_mul_itch(an, bn) * nb, dtype=torch.int32, device="cuda")
        g.mpn_toom22_mul(dp, _dev(torch, a), an, _dev(torch, b), bn, scratch, nb, nb)
        torch.cuda.synchronize()
        assert (_host(dp).reshape(an + bn, nb) == exp).all()
    else:
        with pytest.raises(g.GbmmError):
            g.mpn_toom22_mul(dp, _dev(torch, a), an, _dev(torch, b), bn, dp, nb, nb)
    dp.zero_()
    g.mpn_mul(dp, _dev(torch, a), an, _dev(torch, b), bn, nb, nb)
    torch.cuda.synchronize()
    assert (_host(dp).reshape(an + bn, nb) == exp).all()


@pytest.mark.parametrize("kind,an,bn", [("basecase", 33, 7), ("basecase", 130, 129), ("toom22", 41, 40),
                                          ("toom22", 64, 33), ("toom22", 170, 150)])
@pytest.mark.parametrize("nb,ld", [(37, 37), (37, 41), (130, 132)])
def test_mpn_products_on_chip_strides(g, oracle, kind, an, bn, nb, ld):
    """The shared-memory products with plane strides that rule out 16-byte loads
    (ld odd: four-operand groups staged limb by limb), a last group of operands
    cut by nb, planes wider than the batch (columns past nb stay as they were),
    and operands long enough for 64- and 32-thread CTAs."""
    import torch
    rng = np.random.default_rng(an * 31 + bn + nb + ld)
    a = _rand_planes(rng, an, ld, "ones")
    b = _rand_planes(rng, bn, ld, "ones")
    exp = oracle.mpn_mul_basecase(a[:, :nb].copy(), b[:, :nb].copy())
    dp = torch.full(((an + bn) * ld,), 7, dtype=torch.int32, device="cuda")
    if kind == "basecase":
        g.mpn_mul_basecase(dp, _dev(torch, a), an, _dev(torch, b), bn, ld, nb)
    else:
        scratch = torch.zeros(g.mpn_toom22_mul_itch(an, bn) * ld, dtype=torch.int32, device="cuda")
        g.mpn_toom22_mul(dp, _dev(torch, a), an, _dev(torch, b), bn, scratch, ld, nb)
    torch.cuda.synchronize()
    got = _host(dp).reshape(an + bn, ld)
    assert (got[:, :nb] == exp).all()
    assert (got[:, nb:] == 7).all()


@pytest.mark.parametrize("un,vn", [(900, 900), (900, 760), (900, 500)])
def test_mpn_mul_operands_too_long_to_stage(g, oracle, un, vn):
    """Operands whose per-thread strings do not fit shared memory: mpn_mul takes
    Toom-2.2 through caller scratch (balanced) or the global-memory basecase."""
    import torch
    rng = np.random.default_rng(un + vn)
    nb = 48
    a = _rand_planes(rng, un, nb, "ones")
    b = _rand_planes(rng, vn, nb, "ones")
    exp = oracle.mpn_mul_basecase(a, b)
    dp = torch.zeros((un + vn) * nb, dtype=torch.int32, device="cuda")
    g.mpn_mul(dp, _dev(torch, a), un, _dev(torch, b), vn, nb, nb)
    torch.cuda.synchronize()
    assert (_host(dp).reshape(un + vn, nb) == exp).all()


def _signed(rng, n, bits, zero=0.1):
    out = []
    for i in range(n):
        b = rng.choice([0, 1, 31, 32, 33, 64, bits])
        m = 0 if rng.random() < zero else rng.getrandbits(b) if b else 0
        if rng.random() < 0.1:
            m = (1 << bits) - 1
        out.append(-m if rng.random() < 0.5 else m)
    return out


@pytest.mark.parametrize("sub", [False, True])
def test_mpz_add_sub(g, sub):
    rng = random.Random(3 + sub)
    n = 999
    U = _signed(rng, n, 200)
    V = _signed(rng, n, 200)
    V[:50] = [(-u if not sub else u) for u in U[:50]]   # exact cancellation
    V[50:100] = [(-u - 1 if not sub else u + 1) for u in U[50:100]]
    du = g.DeviceMatrix.from_ints(1, n, U, 7)
    dv = g.DeviceMatrix.from_ints(1, n, V, 7)
    dw = g.DeviceMatrix(1, n, 8)
    (g.mpz_sub if sub else g.mpz_add)(dw, du, dv)
    assert dw.to_ints() == [(u - v if sub else u + v) for u, v in zip(U, V)]


@pytest.mark.parametrize("op", ["mul", "addmul", "submul"])
def test_mpz_mulops(g, op):
    rng = random.Random(len(op))
    n = 777
    U = _signed(rng, n, 150)
    V = _signed(rng, n, 120)
    W = _signed(rng, n, 270)
    # force the |uv| > |w| / |uv| < |w| / equal cases of the signed merge
    W[:20] = [u * v * (1 if op == "submul" else -1) for u, v in zip(U[:20], V[:20])]
    du = g.DeviceMatrix.from_ints(1, n, U, 5)
    dv = g.DeviceMatrix.from_ints(1, n, V, 4)
    dw = g.DeviceMatrix.from_ints(1, n, W, 10)
    getattr(g, "mpz_" + op)(dw, du, dv)
    if op == "mul":
        exp = [u * v for u, v in zip(U, V)]
    elif op == "addmul":
        exp = [w + u * v for u, v, w in zip(U, V, W)]
    else:
        exp = [w - u * v for u, v, w in zip(U, V, W)]
    assert dw.to_ints() == exp


def _golden_device(g, name):
    text, expect = load_golden(name)
    K, M, N, A, B = g.parse_matrix_text(text)
    dA = g.DeviceMatrix.from_ints(K, M, A)
    dB = g.DeviceMatrix.from_ints(M, N, B)
    return K, M, N, dA, dB, expect


@pytest.mark.parametrize("name", golden_cases())
@pytest.mark.parametrize("method,cutoff", [(1, 0), (35, 4), (3, 4), (4, 4), (35, 32)])
def test_limb_matmul_golden(g, name, method, cutoff):
    K, M, N, dA, dB, expect = _golden_device(g, name)
    nl = g.limbs_needed(dA.nlimbs, dB.nlimbs, M, method=method, cutoff=cutoff)
    dC = g.DeviceMatrix(K, N, nl)
    g.squarify_mul(K, M, N, dC, dA, dB, method=method, cutoff=cutoff, path=g.PATH_LIMB)
    limbs, sizes = dC.download()
    assert g.format_hex(limbs, sizes, K, N) == expect


@pytest.mark.parametrize("K,M,N,bits", [(33, 17, 9, 4096), (96, 96, 96, 130), (128, 128, 128, 64),
                                        (5, 300, 3, 800), (64, 64, 64, 2048)])
def test_limb_matmul_random_vs_oracle(g, oracle, K, M, N, bits):
    rng = random.Random(K * 131 + M + N + bits)
    A = _signed(rng, K * M, bits, 0.05)
    B = _signed(rng, M * N, bits, 0.05)
    nla = nlb = (bits + 31) // 32
    dA = g.DeviceMatrix.from_ints(K, M, A, nla)
    dB = g.DeviceMatrix.from_ints(M, N, B, nlb)
    nl = g.limbs_needed(nla, nlb, M, cutoff=16)
    dC = g.DeviceMatrix(K, N, nl)
    g.squarify_mul(K, M, N, dC, dA, dB, method=g.METHOD_WINOGRAD, cutoff=16)
    Cl, Cs = oracle.matmul_planes(K, M, N, g.ints_to_planes(A, nla), g.ints_to_planes(B, nlb), nl, method=1,
                                  nthreads=4)
    limbs, sizes = dC.download()
    assert (sizes == Cs).all()
    assert (limbs == Cl).all()


def test_limb_addmul_accumulates(g):
    rng = random.Random(9)
    K = M = N = 32
    A = _signed(rng, K * M, 300)
    B = _signed(rng, M * N, 300)
    C0 = _signed(rng, K * N, 600)
    dA = g.DeviceMatrix.from_ints(K, M, A, 10)
    dB = g.DeviceMatrix.from_ints(M, N, B, 10)
    for method, cutoff in ((1, 0), (35, 8)):
        nl = g.limbs_needed(10, 10, M, method=method, cutoff=cutoff) + 1
        dC = g.DeviceMatrix.from_ints(K, N, C0, nl)
        g.mat_addmul(K, M, N, dC, dA, dB, method=method, cutoff=cutoff)
        exp = [C0[y * N + x] + sum(A[y * M + k] * B[k * N + x] for k in range(M)) for y in range(K) for x in range(N)]
        assert dC.to_ints() == exp


def test_limb_matmul_capacity_error(g):
    dA = g.DeviceMatrix.from_ints(2, 2, [2**200] * 4, 7)
    dB = g.DeviceMatrix.from_ints(2, 2, [2**200] * 4, 7)
    dC = g.DeviceMatrix(2, 2, 3)
    g.mat_mul(2, 2, 2, dC, dA, dB, method=g.METHOD_NAIVE)
    with pytest.raises(g.GbmmError) as e:
        dC.download()
    assert e.value.status == g.ERR_CAPACITY


def test_empty_shapes(g):
    dA = g.DeviceMatrix(0, 5, 2)
    dB = g.DeviceMatrix(5, 3, 2)
    dC = g.DeviceMatrix(0, 3, 5)
    g.mat_mul(0, 5, 3, dC, dA, dB)
    dA = g.DeviceMatrix.from_ints(2, 0, [], 1)
    dB = g.DeviceMatrix.from_ints(0, 2, [], 1)
    dC = g.DeviceMatrix.from_ints(2, 2, [5, 6, 7, 8], 3)
    g.mat_mul(2, 0, 2, dC, dA, dB, method=g.METHOD_NAIVE)
    assert dC.to_ints() == [0, 0, 0, 0]


@pytest.mark.parametrize("N,bits,cutoff", [(64, 4096, 16), (32, 1024, 4), (96, 300, 12), (128, 64, 8),
                                           (48, 5000, 12)])
def test_winograd_breadth_first_vs_depth_first_and_oracle(g, oracle, N, bits, cutoff):
    """The breadth-first Winograd tree (all sums of a level, all leaf products,
    all combinations of a level: one launch each) against the depth-first
    recursion and the oracle.  4096- and 5000-bit entries make one-limb-longer
    sums (129 and 158 limbs) that take the per-entry kernel's one-group-per-CTA
    form (more than 256 threads per entry)."""
    rng = random.Random(N * 7 + bits + cutoff)
    A = _signed(rng, N * N, bits, 0.05)
    B = _signed(rng, N * N, bits, 0.05)
    nl = (bits + 31) // 32
    dA = g.DeviceMatrix.from_ints(N, N, A, nl)
    dB = g.DeviceMatrix.from_ints(N, N, B, nl)
    cn = g.limbs_needed(nl, nl, N, method=g.METHOD_WINOGRAD, cutoff=cutoff)
    Cl, Cs = oracle.matmul_planes(N, N, N, g.ints_to_planes(A, nl), g.ints_to_planes(B, nl), cn, method=1,
                                  nthreads=8)
    h = g.Handle()
    for bf in (True, False):
        h.set_breadth_first(bf)
        dC = g.DeviceMatrix(N, N, cn)
        dC.limbs_t.fill_(-1)
        h.matmul(dC, dA, dB, path=g.PATH_LIMB, method=g.METHOD_WINOGRAD, cutoff=cutoff)
        limbs, sizes = dC.download()
        assert (sizes == Cs).all(), bf
        assert (limbs == Cl).all(), bf
    h.close()


def test_winograd_breadth_first_rectangular_and_small_output(g, oracle):
    """Squarify around breadth-first square cores, with C holding fewer planes
    than the recursion's headroom (the product then runs into a workspace
    matrix and is copied)."""
    rng = random.Random(21)
    K, M, N, bits = 70, 96, 66, 700
    A = _signed(rng, K * M, bits, 0.05)
    B = _signed(rng, M * N, bits, 0.05)
    nl = (bits + 31) // 32
    dA = g.DeviceMatrix.from_ints(K, M, A, nl)
    dB = g.DeviceMatrix.from_ints(M, N, B, nl)
    cn = 2 * nl + 1
    Cl, Cs = oracle.matmul_planes(K, M, N, g.ints_to_planes(A, nl), g.ints_to_planes(B, nl), cn, method=1,
                                  nthreads=8)
    dC = g.DeviceMatrix(K, N, cn)
    g.default_handle().matmul(dC, dA, dB, path=g.PATH_LIMB, method=g.METHOD_WINOGRAD, cutoff=8)
    limbs, sizes = dC.download()
    assert (sizes == Cs).all() and (limbs == Cl).all()
