"""Batched uneven products (persistent work-queue kernel + CRT jobs + CUDA
graph replay), the limb-half split for entries longer than any kernel takes,
and the autotuner's dispatch table.  Bit-exact against Python integers."""
import json
import math
import os
import random

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


class _own_stream:
    """Runs the block on a torch stream of its own, so that a handle binds a real
    stream and batched calls capture and replay CUDA graphs (a handle on the
    legacy default stream runs every batch eagerly)."""

    def __enter__(self):
        import torch
        self.s = torch.cuda.Stream()
        self.s.wait_stream(torch.cuda.current_stream())
        self.ctx = torch.cuda.stream(self.s)
        self.ctx.__enter__()
        return self.s

    def __exit__(self, *exc):
        import torch
        self.ctx.__exit__(*exc)
        torch.cuda.current_stream().wait_stream(self.s)
        return False


def _make_jobs(g, rng, specs):
    out = []
    for K, M, N, ba, bb in specs:
        A, B = _rand(rng, K * M, ba), _rand(rng, M * N, bb)
        la, lb = (ba + 31) // 32, (bb + 31) // 32
        dA = g.DeviceMatrix.from_ints(K, M, A, la)
        dB = g.DeviceMatrix.from_ints(M, N, B, lb)
        dC = g.DeviceMatrix(K, N, la + lb + 2)
        out.append((K, M, N, A, B, dA, dB, dC))
    return out


SPECS = [(16, 16, 16, 64, 64), (37, 5, 19, 200, 900), (64, 64, 64, 1024, 1024), (3, 100, 7, 33, 2000),
         (50, 20, 40, 4096, 64), (1, 1, 1, 16384, 64), (20, 30, 25, 3000, 2500), (90, 17, 11, 96, 96),
         (128, 64, 33, 512, 777), (5, 5, 5, 9000, 9000), (17, 129, 33, 2048, 2048), (2, 600, 3, 700, 700)]


@pytest.mark.parametrize("path", ["auto", "limb", "crt"])
def test_batched_uneven_exact(g, path):
    rng = random.Random(7)
    jobs = _make_jobs(g, rng, SPECS)
    h = g.Handle()
    p = {"auto": g.PATH_AUTO, "limb": g.PATH_LIMB, "crt": g.PATH_CRT}[path]
    arr = h.jobs([(j[7], j[5], j[6]) for j in jobs], path=p)
    chosen = h.matmul_batched(arr, path=p)
    for (K, M, N, A, B, dA, dB, dC), c in zip(jobs, chosen):
        assert dC.to_ints() == _exact(K, M, N, A, B), (K, M, N, c)
    h.close()


def test_batched_graph_replay_sees_new_inputs(g):
    """Same buffers, new contents: the eager call, the capturing call and two
    replays must each compute the product of the current inputs."""
    rng = random.Random(3)
    specs = [(33, 40, 21, 300, 500), (64, 64, 64, 2048, 2048), (8, 9, 10, 64, 5000)]
    jobs = _make_jobs(g, rng, specs)
    with _own_stream():
        h = g.Handle()
        arr = h.jobs([(j[7], j[5], j[6]) for j in jobs])
        for rnd in range(4):
            if rnd:
                for idx, (K, M, N, A, B, dA, dB, dC) in enumerate(jobs):
                    A = _rand(rng, K * M, specs[idx][3])
                    B = _rand(rng, M * N, specs[idx][4])
                    dA.upload(*g.ints_to_planes(A, dA.nlimbs))
                    dB.upload(*g.ints_to_planes(B, dB.nlimbs))
                    jobs[idx] = (K, M, N, A, B, dA, dB, dC)
            h.matmul_batched(arr)
            for K, M, N, A, B, dA, dB, dC in jobs:
                assert dC.to_ints() == _exact(K, M, N, A, B), rnd
        h.close()


def test_grouped_crt_launches_mixed_products(g):
    """The batch's CRT products run in grouped launches: one launch per stage over
    the tiles of all of them.  Thirty products of log-uniform shapes (1 to 48) and
    bit lengths (64 to 16384, each operand its own) put, in the same launches,
    moduli counts from about 10 to over 1023 (limb-half split), unsigned and
    balanced digit rows, and reconstructions of 1 to 9 N tiles, so that one CTA
    walks entry tiles of different N-tile counts.  Eager call, capturing call and
    replay each give the exact product of the current inputs."""
    rng = random.Random(21)
    lu = lambda lo, hi: int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
    specs = [(lu(1, 48), lu(1, 48), lu(1, 48), lu(64, 16384), lu(64, 16384)) for _ in range(30)]
    specs += [(3, 7, 2, 16384, 16000), (40, 3, 1, 9000, 64)]
    jobs = _make_jobs(g, rng, specs)
    with _own_stream():
        h = g.Handle()
        arr = h.jobs([(j[7], j[5], j[6]) for j in jobs], path=g.PATH_CRT)
        for rnd in range(3):
            if rnd:
                for idx, (K, M, N, A, B, dA, dB, dC) in enumerate(jobs):
                    A = _rand(rng, K * M, specs[idx][3])
                    B = _rand(rng, M * N, specs[idx][4])
                    dA.upload(*g.ints_to_planes(A, dA.nlimbs))
                    dB.upload(*g.ints_to_planes(B, dB.nlimbs))
                    jobs[idx] = (K, M, N, A, B, dA, dB, dC)
            h.matmul_batched(arr, path=g.PATH_CRT)
            for K, M, N, A, B, dA, dB, dC in jobs:
                assert dC.to_ints() == _exact(K, M, N, A, B), (rnd, K, M, N)
        h.close()


def test_batched_graph_capture_on_own_stream(g):
    """A handle bound to a stream of its own (not the legacy default stream) runs
    the first call eagerly, captures the launch sequence into a CUDA graph on the
    second and replays it from the third: per-entry limb jobs (work queue), grouped
    CRT jobs (one of them split), and a CRT job with k > 512 (side stream).  Each
    call computes the exact product of the current inputs; a replay launches no
    more kernels than the capture recorded."""
    rng = random.Random(31)
    specs = [(40, 30, 20, 200, 96), (33, 40, 21, 3000, 2500), (6, 9, 5, 16000, 4000), (9, 700, 8, 400, 300),
             (64, 64, 64, 2048, 1024), (3, 4, 5, 64, 64)]
    jobs = _make_jobs(g, rng, specs)
    with _own_stream() as s:
        h = g.Handle()
        arr = h.jobs([(j[7], j[5], j[6]) for j in jobs])
        counts = []
        for rnd in range(5):
            if rnd:
                for idx, (K, M, N, A, B, dA, dB, dC) in enumerate(jobs):
                    A = _rand(rng, K * M, specs[idx][3])
                    B = _rand(rng, M * N, specs[idx][4])
                    dA.upload(*g.ints_to_planes(A, dA.nlimbs))
                    dB.upload(*g.ints_to_planes(B, dB.nlimbs))
                    jobs[idx] = (K, M, N, A, B, dA, dB, dC)
            n0 = g.kernel_launches()
            h.matmul_batched(arr)
            counts.append(g.kernel_launches() - n0)
            s.synchronize()
            for K, M, N, A, B, dA, dB, dC in jobs:
                assert dC.to_ints() == _exact(K, M, N, A, B), rnd
        h.close()
    # eager, capture (its kernels counted as they are recorded), then replays
    assert counts[2] == counts[3] == counts[4] == counts[1] > 0, counts


def test_batched_tables_built_mid_batch(g):
    """Products too large for the grouped launches run on side streams, and a
    product whose moduli count the handle has not met yet builds its CRT tables
    just before its launches.  The tables must have landed in device memory by
    then, whatever stream the handle is bound to: fresh handles on a stream of
    their own, eight such products of distinct moduli counts per batch, every
    product checked against Python integers on sampled entries."""
    rng = random.Random(41)
    for rnd in range(3):
        specs = [(200, 24, 180, 300 + 397 * i + 61 * rnd, 500 + 211 * i) for i in range(8)]
        jobs = _make_jobs(g, rng, specs)
        with _own_stream():
            h = g.Handle()
            h.matmul_batched(h.jobs([(j[7], j[5], j[6]) for j in jobs]))
            for K, M, N, A, B, dA, dB, dC in jobs:
                C = dC.to_ints()
                for _ in range(6):
                    y, x = rng.randrange(K), rng.randrange(N)
                    assert C[y * N + x] == sum(A[y * M + k] * B[k * N + x] for k in range(M)), (rnd, K, M, N)
            h.close()


@pytest.mark.parametrize("path", ["limb", "crt"])
def test_split_for_very_long_entries(g, path):
    rng = random.Random(11)
    K, M, N = 6, 9, 5
    A, B = _rand(rng, K * M, 12000, 0.0), _rand(rng, M * N, 30000, 0.0)
    dA = g.DeviceMatrix.from_ints(K, M, A)
    dB = g.DeviceMatrix.from_ints(M, N, B)
    dC = g.DeviceMatrix(K, N, dA.nlimbs + dB.nlimbs + 2)
    g.default_handle().matmul(dC, dA, dB, path={"limb": g.PATH_LIMB, "crt": g.PATH_CRT}[path])
    assert dC.to_ints() == _exact(K, M, N, A, B)


@pytest.mark.parametrize("path", ["limb", "crt"])
def test_split_accumulate_and_plans(g, path):
    """C += A*B through the limb-half split, with C of either sign (the combine's
    subtractions), and the stacked halves along rows (A longer) and columns (B
    longer); also the CRT_SPLIT plan on operands that would not need it."""
    rng = random.Random(13)
    for K, M, N, ba, bb in [(7, 9, 5, 30000, 12000), (6, 10, 9, 9000, 33000), (33, 17, 40, 20000, 20000)]:
        A, B = _rand(rng, K * M, ba, 0.05), _rand(rng, M * N, bb, 0.05)
        C0 = _rand(rng, K * N, ba + bb, 0.2)
        dA = g.DeviceMatrix.from_ints(K, M, A)
        dB = g.DeviceMatrix.from_ints(M, N, B)
        dC = g.DeviceMatrix.from_ints(K, N, C0, dA.nlimbs + dB.nlimbs + 3)
        g.default_handle().matmul(dC, dA, dB, path={"limb": g.PATH_LIMB, "crt": g.PATH_CRT}[path], accumulate=True)
        exp = _exact(K, M, N, A, B)
        assert dC.to_ints() == [c + e for c, e in zip(C0, exp)]
    if path == "crt":
        K, M, N = 20, 24, 18
        A, B = _rand(rng, K * M, 3000, 0.1), _rand(rng, M * N, 2500, 0.1)
        dA = g.DeviceMatrix.from_ints(K, M, A)
        dB = g.DeviceMatrix.from_ints(M, N, B)
        dC = g.DeviceMatrix(K, N, dA.nlimbs + dB.nlimbs + 2)
        g.default_handle().matmul(dC, dA, dB, plan=g.PLAN_CRT_SPLIT)
        assert dC.to_ints() == _exact(K, M, N, A, B)


def test_autotune_table_roundtrip(g, tmp_path):
    rng = random.Random(5)
    jobs = _make_jobs(g, rng, [(64, 64, 64, 2048, 2048), (8, 8, 8, 64, 64)])
    h = g.Handle()
    arr = h.jobs([(j[7], j[5], j[6]) for j in jobs])
    log = str(tmp_path / "timings.jsonl")
    h.autotune(arr, repeats=1, log_path=log)
    rows = [json.loads(l) for l in open(log)]
    assert len(rows) >= 4 and all(r["ms"] > 0 for r in rows)
    table = str(tmp_path / "tune.json")
    g.check(g.lib().gbmm_tune_save(h.h, table.encode()))
    h2 = g.Handle()
    g.check(g.lib().gbmm_tune_load(h2.h, table.encode()))
    chosen = h2.matmul_batched(h2.jobs([(j[7], j[5], j[6]) for j in jobs]))
    best = {}
    for r in rows:
        key = (r["m"], r["la"])
        if key not in best or r["ms"] < best[key][0]:
            best[key] = (r["ms"], r["path"])
    assert chosen == [best[(64, 64)][1], best[(8, 2)][1]]
    assert {r["plan"] for r in rows} >= {g.PLAN_LIMB_NAIVE, g.PLAN_CRT, g.PLAN_CRT_SINGLE, g.PLAN_CRT_PAIR}
    for K, M, N, A, B, dA, dB, dC in jobs:
        assert dC.to_ints() == _exact(K, M, N, A, B)
    h.close()
    h2.close()


def test_batched_uneven_stream_repeated_on_fresh_handles(g):
    """The learned-dispatch workload's 72 products (uneven shapes, A and B of
    independent bit lengths in [64, 16384], eight 1024x64x1024 rectangles), run in
    one batched call on a fresh handle, eight times.  Every result is downloaded
    (which reports any device-side capacity or wait-timeout flag) and sampled
    entries are checked against Python integers.  Products whose result fits one
    reconstruction table tile exercise the hand-over of the fixed-point quotient
    and top-limb slots between the reconstruction's two epilogue halves; an
    unordered hand-over there failed about one batch in five."""
    import numpy as np
    import bench
    evals, _ = bench.gen_jobs(g, bench.WORKLOADS["cfg5"], 2024)
    srng = np.random.default_rng(3)
    for rep in range(8):
        h = g.Handle()
        jobs = h.jobs([(c, a, b) for c, a, b, _ in evals])
        h.matmul_batched(jobs)
        for i, (dC, dA, dB, (Al, As, Bl, Bs, K, M, N)) in enumerate(evals):
            Cl, Cs = dC.download()
            if i % 6 == rep % 6:
                y, x = int(srng.integers(K)), int(srng.integers(N))
                exp = sum(bench.entry_int(Al, As, y * M + k) * bench.entry_int(Bl, Bs, k * N + x) for k in range(M))
                assert bench.entry_int(Cl, Cs, y * N + x) == exp, (rep, i, K, M, N)
        h.close()
