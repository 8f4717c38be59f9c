"""gbmm_matmul_host: products on host buffers with pipelined host <-> device
copies (two device slots, upload / compute / download streams).  Bit-exact
against Python integers, across paths, uneven shapes, empty shapes, slot growth
between calls and results that land in pinned or pageable memory."""
import random

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def g(built_lib):
    import gbmm
    gbmm.default_handle()
    return gbmm


def _rand(rng, n, bits, zero=0.1):
    return [0 if rng.random() < zero else rng.getrandbits(bits) * rng.choice((-1, 1)) for _ in range(n)]


def _exact(K, M, N, A, B):
    return [sum(A[y * M + k] * B[k * N + x] for k in range(M)) for y in range(K) for x in range(N)]


def _spec(g, rng, K, M, N, ba, bb):
    A, B = _rand(rng, K * M, ba), _rand(rng, M * N, bb)
    la, lb = max(1, (ba + 31) // 32), max(1, (bb + 31) // 32)
    Al, As = g.ints_to_planes(A, la)
    Bl, Bs = g.ints_to_planes(B, lb)
    cn = la + lb + 2
    Cl = np.zeros((cn, K * N), dtype=np.uint32)
    Cs = np.zeros(K * N, dtype=np.int32)
    return (K, M, N, (Al, As), (Bl, Bs), (Cl, Cs)), _exact(K, M, N, A, B)


SPECS = [(16, 16, 16, 64, 64), (37, 5, 19, 200, 900), (64, 64, 64, 1024, 1024), (3, 100, 7, 33, 2000),
         (50, 20, 40, 4096, 64), (1, 1, 1, 16384, 64), (20, 30, 25, 3000, 2500), (128, 64, 33, 512, 777)]


@pytest.mark.parametrize("path", ["auto", "limb", "crt"])
def test_host_jobs_exact(g, path):
    rng = random.Random(21)
    built = [_spec(g, rng, *s) for s in SPECS]
    h = g.Handle()
    p = {"auto": g.PATH_AUTO, "limb": g.PATH_LIMB, "crt": g.PATH_CRT}[path]
    arr = h.host_jobs([b[0] for b in built], path=p)
    chosen = h.matmul_host(arr)
    assert len(chosen) == len(SPECS)
    for (spec, exp), c in zip(built, chosen):
        K, M, N, _, _, (Cl, Cs) = spec
        assert g.planes_to_ints(Cl, Cs) == exp, (K, M, N, c)
    h.close()


def test_host_jobs_grow_slots_and_empty_shapes(g):
    rng = random.Random(5)
    h = g.Handle()
    small = [_spec(g, rng, 8, 8, 8, 64, 64), _spec(g, rng, 0, 4, 4, 64, 64), _spec(g, rng, 4, 0, 4, 64, 64)]
    h.matmul_host(h.host_jobs([b[0] for b in small]))
    for spec, exp in small:
        assert g.planes_to_ints(spec[5][0], spec[5][1]) == exp
    # a later call with larger jobs regrows both device slots
    big = [_spec(g, rng, 96, 80, 72, 2048, 1536) for _ in range(3)]
    h.matmul_host(h.host_jobs([b[0] for b in big], path=g.PATH_CRT))
    for spec, exp in big:
        assert g.planes_to_ints(spec[5][0], spec[5][1]) == exp
    h.close()


def test_host_jobs_pinned_buffers(g):
    torch = pytest.importorskip("torch")
    rng = random.Random(9)
    spec, exp = _spec(g, rng, 64, 48, 40, 1500, 1500)
    K, M, N, (Al, As), (Bl, Bs), (Cl, Cs) = spec
    pin = lambda a: torch.from_numpy(a).pin_memory().numpy()
    pA, pAs, pB, pBs = pin(Al), pin(As), pin(Bl), pin(Bs)
    pC, pCs = pin(np.zeros_like(Cl)), pin(np.zeros_like(Cs))
    h = g.Handle()
    jobs = h.host_jobs([(K, M, N, (pA, pAs), (pB, pBs), (pC, pCs))] * 4, path=g.PATH_CRT)
    h.matmul_host(jobs)
    assert g.planes_to_ints(pC, pCs) == exp
    h.close()


def test_host_jobs_out_of_core(g):
    """A device budget below the products' in-core footprint makes gbmm_matmul_host
    run them in blocks (C tiles, inner chunks accumulated on the device), mixed with
    in-core jobs in one call."""
    import ctypes
    rng = random.Random(31)
    big = [_spec(g, rng, 150, 130, 110, 1500, 1200), _spec(g, rng, 40, 300, 20, 64, 700)]
    small = [_spec(g, rng, 8, 8, 8, 64, 64)]
    h = g.Handle()
    h.set_device_budget(20 << 20)  # the in-core footprints are 34 MB (limb) and 82 MB (CRT) for the first job
    f = g.lib().gbmmx_host_blocks
    f.restype = ctypes.c_int64
    for path in (g.PATH_AUTO, g.PATH_CRT, g.PATH_LIMB):
        for spec, _ in big + small:
            spec[5][0][:] = 0
            spec[5][1][:] = 0
        specs = [big[0], small[0], big[1]]
        h.matmul_host(h.host_jobs([b[0] for b in specs], path=path))
        assert f() >= 2, f()  # at least one job ran as two or more block products
        for spec, exp in specs:
            assert g.planes_to_ints(spec[5][0], spec[5][1]) == exp, (spec[:3], path)
    h.close()


def test_host_jobs_staged_crt_parts(g):
    """Single-pass CRT products start on A while B uploads, and the call's last
    product returns C in entry ranges as its reconstruction finishes them.  The
    first job here (2048-bit entries, 258 moduli) reconstructs on CTA pairs in four
    ranges when it is last; followed by a limb-path job it runs whole."""
    rng = random.Random(44)
    crt = _spec(g, rng, 150, 64, 120, 2048, 2048)
    small = _spec(g, rng, 12, 9, 14, 96, 64)
    h = g.Handle()
    for order in ([crt], [crt, small], [small, crt]):
        for spec, _ in order:
            spec[5][0][:] = 0
            spec[5][1][:] = 0
        paths = [g.PATH_CRT if s is crt else g.PATH_LIMB for s in order]
        arr = h.host_jobs([s[0] for s in order], path=g.PATH_AUTO)
        for i, p in enumerate(paths):
            arr[i].path = p
        chosen = h.matmul_host(arr)
        assert list(chosen) == paths
        for spec, exp in order:
            assert g.planes_to_ints(spec[5][0], spec[5][1]) == exp, spec[:3]
    h.close()
