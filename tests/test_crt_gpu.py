"""The CRT tensor-core path: the tcgen05 GEMM core against exact integer
products, and whole products C = A*B against the golden fixtures and the CPU
oracle (bit-exact).  Also size-independent checks at the 512^3 / 4096-bit
scale: sampled entries against Python integers and the linearity
A*(B1 + B2) = A*B1 + A*B2."""
import ctypes
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


def _bf16(torch, ints):
    return torch.tensor(ints, dtype=torch.float32).to(torch.bfloat16).cuda()


@pytest.mark.parametrize("M,N,K,a_mn", [(128, 128, 64, 0), (256, 384, 512, 0), (200, 136, 192, 0),
                                        (128, 128, 64, 1), (256, 128, 1024, 1), (192, 256, 128, 1)])
def test_tcgen05_gemm_core(g, M, N, K, a_mn):
    import torch
    rng = np.random.default_rng(M + N + K + a_mn)
    A = rng.integers(-128, 128, size=(M, K))
    B = rng.integers(-128, 128, size=(N, K))
    A[0, :] = -128
    B[0, :] = -128                       # the largest |partial sum| the CRT GEMMs rely on
    exp = A @ B.T
    dA = _bf16(torch, A.T.copy() if a_mn else A)
    dB = _bf16(torch, B)
    D = torch.zeros(M * N, dtype=torch.int32, device="cuda")
    L = g.lib()
    L.gbmmx_test_gemm.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int32] * 4 + [ctypes.c_void_p]
    g.check(L.gbmmx_test_gemm(dA.data_ptr(), dB.data_ptr(), D.data_ptr(), M, N, K, a_mn, g.stream_ptr()))
    torch.cuda.synchronize()
    got = D.cpu().numpy().reshape(M, N)
    assert (got == exp).all(), f"{(got != exp).sum()} mismatches"


@pytest.mark.parametrize("M,N,K", [(256, 256, 64), (512, 256, 512), (200, 296, 192), (768, 512, 1024)])
def test_tcgen05_gemm_pair(g, M, N, K):
    """The CTA-pair (cta_group::2, M = 256) MMA path: A and D split along M across
    two SMs, B along N, barriers shared across the pair."""
    import torch
    rng = np.random.default_rng(M * 7 + N + K)
    A = rng.integers(-128, 129, size=(M, K))
    B = rng.integers(-128, 129, size=(N, K))
    A[0, :] = -128
    B[0, :] = -128
    exp = A @ B.T
    dA, dB = _bf16(torch, A), _bf16(torch, B)
    D = torch.zeros(M * N, dtype=torch.int32, device="cuda")
    L = g.lib()
    L.gbmmx_test_gemm_pair.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int32] * 3 + [ctypes.c_void_p]
    g.check(L.gbmmx_test_gemm_pair(dA.data_ptr(), dB.data_ptr(), D.data_ptr(), M, N, K, g.stream_ptr()))
    torch.cuda.synchronize()
    got = D.cpu().numpy().reshape(M, N)
    assert (got == exp).all(), f"{(got != exp).sum()} mismatches"


def _crt(g, K, M, N, dA, dB, nl=None, nprimes=0):
    nl = nl or g.limbs_needed(dA.nlimbs, dB.nlimbs, M, path=g.PATH_CRT)
    dC = g.DeviceMatrix(K, N, nl)
    g.default_handle().matmul(dC, dA, dB, path=g.PATH_CRT, nprimes=nprimes)
    return dC


@pytest.mark.parametrize("name", golden_cases())
def test_crt_matmul_golden(g, name):
    text, expect = load_golden(name)
    K, M, N, A, B = g.parse_matrix_text(text)
    dA = g.DeviceMatrix.from_ints(K, M, A)
    dB = g.DeviceMatrix.from_ints(M, N, B)
    dC = _crt(g, K, M, N, dA, dB)
    limbs, sizes = dC.download()
    assert g.format_hex(limbs, sizes, K, N) == expect


def _signed(rng, n, bits, zero=0.05):
    out = []
    for _ in range(n):
        r = rng.random()
        if r < zero:
            m = 0
        elif r < zero + 0.05:
            m = rng.getrandbits(64)
        elif r < zero + 0.1:
            m = (1 << bits) - 1
        else:
            m = rng.getrandbits(bits)
        out.append(-m if rng.random() < 0.5 else m)
    return out


@pytest.mark.parametrize("K,M,N,bits", [(129, 65, 130, 2048), (64, 512, 64, 1024), (3, 7, 5, 16384),
                                        (256, 256, 256, 512), (1, 1, 300, 4096), (40, 200, 33, 33)])
def test_crt_matmul_vs_oracle(g, oracle, K, M, N, bits):
    rng = random.Random(K * 7 + M * 11 + N + bits)
    A = _signed(rng, K * M, bits)
    B = _signed(rng, M * N, bits)
    nl = (bits + 31) // 32
    dA = g.DeviceMatrix.from_ints(K, M, A, nl)
    dB = g.DeviceMatrix.from_ints(M, N, B, nl)
    dC = _crt(g, K, M, N, dA, dB)
    Cl, Cs = oracle.matmul_planes(K, M, N, g.ints_to_planes(A, nl), g.ints_to_planes(B, nl), dC.nlimbs, method=1,
                                  nthreads=8)
    limbs, sizes = dC.download()
    assert (sizes == Cs).all()
    assert (limbs == Cl).all()


@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("K,M,N,bits", [(70, 96, 50, 4096), (33, 37, 20, 4096), (20, 64, 24, 8192),
                                        (5, 64, 7, 16000), (10, 32, 9, 1500), (3, 45, 300, 2048)])
def test_crt_residue_forms(g, mode, K, M, N, bits):
    """The three forms of the residue GEMM (single CTAs, CTA pairs, two-CTA
    clusters sharing the table by multicast, here with odd row-block counts so a
    cluster's second block can lie past the last entry), with the epilogue's
    TMA-store output (inner dimension a multiple of 32) and its per-entry store
    output (any other), over one to four accumulation groups."""
    rng = random.Random(K + M * 3 + N * 5 + bits + mode)
    A = _signed(rng, K * M, bits)
    B = _signed(rng, M * N, bits)
    nl = (bits + 31) // 32
    dA = g.DeviceMatrix.from_ints(K, M, A, nl)
    dB = g.DeviceMatrix.from_ints(M, N, B, nl)
    f = g.lib().gbmmx_residue_mode
    f.argtypes = [ctypes.c_int32]
    f.restype = ctypes.c_int32
    old = f(mode)
    try:
        dC = _crt(g, K, M, N, dA, dB)
    finally:
        f(old)
    exp = [sum(A[y * M + k] * B[k * N + x] for k in range(M)) for y in range(K) for x in range(N)]
    assert dC.to_ints() == exp


@pytest.mark.parametrize("own_stream", [False, True])
def test_programmatic_dependent_launch_matches_plain_launches(g, own_stream):
    """The four stages' kernels are launched with programmatic stream
    serialization: a kernel's CTAs may set up while the kernel before it finishes,
    and wait for it before their first global-memory access.  Plain stream-ordered
    launches give the same product, on the legacy stream and on a created one, and
    both equal the exact product on every entry."""
    import contextlib
    import torch
    rng = random.Random(91 + int(own_stream))
    K, M, N, bits = 64, 128, 48, 3000
    A = _signed(rng, K * M, bits)
    B = _signed(rng, M * N, bits)
    nl = (bits + 31) // 32
    dA = g.DeviceMatrix.from_ints(K, M, A, nl)
    dB = g.DeviceMatrix.from_ints(M, N, B, nl)
    f = g.lib().gbmmx_launch_pdl
    f.argtypes = [ctypes.c_int32]
    f.restype = ctypes.c_int32
    got = {}
    old = f(1)
    try:
        with torch.cuda.stream(torch.cuda.Stream()) if own_stream else contextlib.nullcontext():
            for mode in (0, 1):
                f(mode)
                dC = _crt(g, K, M, N, dA, dB)
                got[mode] = dC.to_ints()
    finally:
        f(old)
    exp = [sum(A[y * M + k] * B[k * N + x] for k in range(M)) for y in range(K) for x in range(N)]
    assert got[0] == exp
    assert got[1] == exp


@pytest.mark.parametrize("K,M,N,bits,cutoff", [(64, 64, 64, 1024, 32), (128, 128, 128, 2048, 32),
                                               (96, 96, 96, 700, 24), (128, 128, 128, 4096, 64),
                                               (64, 32, 64, 512, 16)])
def test_winograd_tree_with_crt_leaves(g, K, M, N, bits, cutoff):
    """GBMM_METHOD_WINOGRAD_CRT: Winograd's breadth-first tree (limb-kernel sums
    and combinations) whose 7^L leaf products run as CRT products in the grouped
    launches, one or two levels, leaves of 24 to 64.  The result equals the plain
    CRT form's bit for bit, and sampled entries equal Python integers; a
    rectangular product takes the plain CRT form."""
    rng = random.Random(K * 3 + bits + cutoff)
    A = _signed(rng, K * M, bits)
    B = _signed(rng, M * N, bits)
    dA = g.DeviceMatrix.from_ints(K, M, A)
    dB = g.DeviceMatrix.from_ints(M, N, B)
    ref = _crt(g, K, M, N, dA, dB)
    dC = g.DeviceMatrix(K, N, ref.nlimbs)
    g.default_handle().matmul(dC, dA, dB, path=g.PATH_CRT, method=g.METHOD_WINOGRAD_CRT, cutoff=cutoff)
    got = dC.to_ints()
    assert got == ref.to_ints()
    for _ in range(8):
        y, x = rng.randrange(K), rng.randrange(N)
        assert got[y * N + x] == sum(A[y * M + k] * B[k * N + x] for k in range(M))


def test_crt_cancellation_and_tiny_results(g):
    # rows of A whose products cancel exactly (C entries 0 or tiny): the sign is
    # then decided on the two's-complement path of the reconstruction
    rng = random.Random(4)
    K, M, N, bits = 130, 64, 20, 3000
    A = _signed(rng, K * M, bits)
    B = _signed(rng, M * N, bits)
    for y in range(0, K, 2):
        for k in range(0, M, 2):
            A[y * M + k + 1] = -A[y * M + k]
    for k in range(0, M, 2):
        for x in range(N):
            B[(k + 1) * N + x] = B[k * N + x] + (1 if (k + x) % 3 == 0 else 0)
    nl = (bits + 31) // 32
    dA = g.DeviceMatrix.from_ints(K, M, A, nl)
    dB = g.DeviceMatrix.from_ints(M, N, B, nl)
    dC = _crt(g, K, M, N, dA, dB)
    exp = [sum(A[y * M + k] * B[k * N + x] for k in range(M)) for y in range(K) for x in range(N)]
    assert dC.to_ints() == exp


def test_crt_accumulate(g):
    rng = random.Random(8)
    K, M, N, bits = 70, 30, 50, 700
    A, B = _signed(rng, K * M, bits), _signed(rng, M * N, bits)
    C0 = _signed(rng, K * N, 1500)
    nl = (bits + 31) // 32
    dA = g.DeviceMatrix.from_ints(K, M, A, nl)
    dB = g.DeviceMatrix.from_ints(M, N, B, nl)
    dC = g.DeviceMatrix.from_ints(K, N, C0, 2 * nl + 3)
    g.default_handle().matmul(dC, dA, dB, path=g.PATH_CRT, accumulate=True)
    exp = [C0[y * N + x] + sum(A[y * M + k] * B[k * N + x] for k in range(M)) for y in range(K) for x in range(N)]
    assert dC.to_ints() == exp


def _entry(limbs, sizes, e):
    m = int.from_bytes(np.ascontiguousarray(limbs[:, e]).tobytes(), "little")
    return -m if sizes[e] < 0 else m


def test_crt_full_size_512_4096_sampled_and_linear(g):
    """512x512x512 at 4096 bits: 64 sampled entries exact against Python
    integers, and A*(B1+B2) == A*B1 + A*B2 over the whole matrix."""
    import bench
    rng = np.random.default_rng(99)
    K = M = N = 512
    Al, As = bench.gen_planes(rng, K * M, 4096, 0, 0, 0)
    B1l, B1s = bench.gen_planes(rng, M * N, 4095, 0, 0, 0)
    B2l, B2s = bench.gen_planes(rng, M * N, 4095, 0, 0, 0)
    dA = g.DeviceMatrix(K, M, 128)
    dA.upload(Al, As)
    dB1, dB2, dBs = g.DeviceMatrix(M, N, 128), g.DeviceMatrix(M, N, 128), g.DeviceMatrix(M, N, 128)
    dB1.upload(B1l, B1s)
    dB2.upload(B2l, B2s)
    g.mat_add(dBs, dB1, dB2)
    nl = g.limbs_needed(128, 128, M, path=g.PATH_CRT)
    C1, C2, Cs = (_crt(g, K, M, N, dA, d, nl) for d in (dB1, dB2, dBs))
    Csum = g.DeviceMatrix(K, N, nl)
    g.mat_add(Csum, C1, C2)
    l1, s1 = Cs.download()
    l2, s2 = Csum.download()
    assert (s1 == s2).all() and (l1 == l2).all()
    lc, sc = C1.download()
    srng = np.random.default_rng(5)
    for _ in range(64):
        y, x = int(srng.integers(K)), int(srng.integers(N))
        exp = sum(_entry(Al, As, y * M + k) * _entry(B1l, B1s, k * N + x) for k in range(M))
        assert _entry(lc, sc, y * N + x) == exp


@pytest.mark.parametrize("bits", [64, 600, 700])
def test_crt_reconstruction_one_table_tile_many_entry_tiles(g, bits):
    """Products whose result fits one 256-digit table tile (small entries), with
    several entry tiles per CTA: the reconstruction's two epilogue halves then hand
    over the fixed-point quotient, sign and top-limb slots once per entry tile, and
    a half running a tile ahead would overwrite them.  Repeated runs, compared bit
    for bit against the limb path and, on a sample, against Python integers."""
    rng = random.Random(bits)
    K, M, N = 420, 16, 400
    A = _signed(rng, K * M, bits)
    B = _signed(rng, M * N, bits)
    nl = (bits + 31) // 32
    dA = g.DeviceMatrix.from_ints(K, M, A, nl)
    dB = g.DeviceMatrix.from_ints(M, N, B, nl)
    cn = g.limbs_needed(nl, nl, M, path=g.PATH_CRT)
    ref = g.DeviceMatrix(K, N, cn)
    g.default_handle().matmul(ref, dA, dB, path=g.PATH_LIMB, method=g.METHOD_NAIVE)
    rl, rs = ref.download()
    srng = random.Random(1)
    for _ in range(8):
        y, x = srng.randrange(K), srng.randrange(N)
        assert _entry(rl, rs, y * N + x) == sum(A[y * M + k] * B[k * N + x] for k in range(M))
    for rep in range(12):
        dC = g.DeviceMatrix(K, N, cn)
        g.default_handle().matmul(dC, dA, dB, path=g.PATH_CRT)
        cl, cs = dC.download()
        assert (cs == rs).all() and (cl == rl).all(), rep


@pytest.mark.parametrize("mode", ["single", "batched", "host"])
def test_crt_vs_limb_random_shapes(g, mode):
    """Differential check over seeded random shapes (log-uniform dimensions, A and B
    of independent bit lengths in [16, 9000], zero and shortened entries): the CRT
    path through one entry point equals the limb path bit for bit."""
    import numpy as np
    import bench
    rng = random.Random({"single": 1, "batched": 2, "host": 3}[mode])
    nprng = np.random.default_rng(rng.randrange(1 << 30))
    lu = lambda lo, hi: int(round(float(np.exp(rng.uniform(np.log(lo), np.log(hi))))))
    jobs = []
    while len(jobs) < 12:
        K, M, N = lu(1, 400), lu(1, 600), lu(1, 400)
        ba, bb = lu(16, 9000), lu(16, 9000)
        if K * M * N * ((ba + 31) // 32) * ((bb + 31) // 32) > 1e10:
            continue
        Al, As = bench.gen_planes(nprng, K * M, ba, 0.1, 0.1, 48)
        Bl, Bs = bench.gen_planes(nprng, M * N, bb, 0.1, 0.1, 48)
        dA, dB = g.DeviceMatrix(K, M, Al.shape[0]), g.DeviceMatrix(M, N, Bl.shape[0])
        dA.upload(Al, As)
        dB.upload(Bl, Bs)
        jobs.append((K, M, N, dA, dB, Al.shape[0] + Bl.shape[0] + 2, (Al, As, Bl, Bs)))
    h = g.Handle()
    refs = []
    for K, M, N, dA, dB, cn, _ in jobs:
        r = g.DeviceMatrix(K, N, cn)
        h.matmul(r, dA, dB, path=g.PATH_LIMB, method=g.METHOD_NAIVE)
        refs.append(r.download())
    if mode == "single":
        outs = []
        for K, M, N, dA, dB, cn, _ in jobs:
            c = g.DeviceMatrix(K, N, cn)
            h.matmul(c, dA, dB, path=g.PATH_CRT)
            outs.append(c.download())
    elif mode == "batched":
        cs = [g.DeviceMatrix(j[0], j[2], j[5]) for j in jobs]
        h.matmul_batched(h.jobs([(c, j[3], j[4]) for c, j in zip(cs, jobs)], path=g.PATH_CRT), path=g.PATH_CRT)
        outs = [c.download() for c in cs]
    else:
        specs = []
        for K, M, N, dA, dB, cn, (Al, As, Bl, Bs) in jobs:
            specs.append((K, M, N, (Al, As), (Bl, Bs),
                          (np.zeros((cn, K * N), dtype=np.uint32), np.zeros(K * N, dtype=np.int32))))
        h.matmul_host(h.host_jobs(specs, path=g.PATH_CRT))
        outs = [(s[5][0], s[5][1]) for s in specs]
    for j, (rl, rs), (cl, cs_) in zip(jobs, refs, outs):
        assert (cs_ == rs).all() and (cl == rl).all(), j[:3]
    h.close()


@pytest.mark.parametrize("skip_step", [0, 3, 7])
def test_bounded_wait_expires_and_context_survives(g, skip_step):
    """The failure path of the tensor-core pipelines, made to happen: in the
    single-CTA test GEMM (K = 512: 8 K steps through 4 stages) the producer leaves
    one K step unloaded, so nothing arms that stage's barrier and the MMA issuer's
    wait for it cannot complete.  With every wait bounded to 2e7 SM clocks (about
    10 ms), each role must give up, let its in-flight copies and MMAs finish, free
    TMEM and exit: the call returns GBMM_ERR_TIMEOUT instead of hanging, and the
    same context then computes a correct product."""
    import torch
    rng = np.random.default_rng(skip_step)
    A = rng.integers(-128, 128, size=(128, 512))
    B = rng.integers(-128, 128, size=(128, 512))
    dA, dB = _bf16(torch, A), _bf16(torch, B)
    D = torch.zeros(128 * 128, dtype=torch.int32, device="cuda")
    L = g.lib()
    f = L.gbmmx_test_gemm_timeout
    f.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int32, ctypes.c_int32, ctypes.c_int64, ctypes.c_void_p]
    f.restype = ctypes.c_int
    st = f(dA.data_ptr(), dB.data_ptr(), D.data_ptr(), 512, skip_step, 20_000_000, g.stream_ptr())
    assert st == g.ERR_TIMEOUT, (st, L.gbmm_last_error_string())
    assert b"wait expired" in L.gbmm_last_error_string()
    # the device error word was read and cleared; the context still runs kernels correctly
    L.gbmmx_test_gemm.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int32] * 4 + [ctypes.c_void_p]
    g.check(L.gbmmx_test_gemm(dA.data_ptr(), dB.data_ptr(), D.data_ptr(), 128, 128, 512, 0, g.stream_ptr()))
    torch.cuda.synchronize()
    assert (D.cpu().numpy().reshape(128, 128) == A @ B.T).all()
