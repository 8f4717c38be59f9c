"""Complete-output parity at the benchmark sizes: every entry of C, limbs and
sizes, bit for bit against the CPU oracle (the reference's naive mat_mul order,
mat-cpu/mat.c:72-82, over GMP arithmetic on all host cores).

- 512 x 512 x 512 at 4096 bits (the headline workload) through gbmm_matmul on
  the CRT path, on the limb path (Winograd, cutoffs 32 and 64) and through
  gbmm_matmul_host (host buffers, pipelined copies);
- 256 x 256 x 256 at 2048 bits with 5% zero and 5% 64-bit entries on the limb
  path (Winograd, cutoff 32) and on the CRT path;
- one seeded 64-product draw of the uneven workload (m, n, k log-uniform in
  [16, 512], bit lengths log-uniform in [64, 16384], 10% zeros) through
  gbmm_matmul_batched: the eager call, the capturing call and a graph replay.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NTHREADS = os.cpu_count() or 1


@pytest.fixture(scope="module")
def g(built_lib):
    import gbmm
    gbmm.default_handle()
    return gbmm


@pytest.fixture(scope="module")
def orc(oracle):
    oracle.set_backend(1 if oracle.gmp_available() else 0)
    yield oracle
    oracle.set_backend(0)


def _expect(orc, K, M, N, A, B, cn):
    return orc.matmul_planes(K, M, N, A, B, cn, method=1, nthreads=NTHREADS)


def _same(got, exp):
    (gl, gs), (el, es) = got, exp
    assert gs.shape == es.shape
    bad = np.flatnonzero(gs != es)
    assert bad.size == 0, f"{bad.size} sizes differ, first at entry {bad[:4]}"
    n = min(gl.shape[0], el.shape[0])
    assert not gl[n:].any() and not el[n:].any()
    bad = np.flatnonzero((gl[:n] != el[:n]).any(axis=0))
    assert bad.size == 0, f"{bad.size} entries differ, first at {bad[:4]}"


def _planes(rng, n, bits, zero=0.0, short=0.0, short_bits=0):
    import bench
    return bench.gen_planes(rng, n, bits, zero, short, short_bits)


@pytest.fixture(scope="module")
def cfg3(g, orc):
    rng = np.random.default_rng(2024)
    K = M = N = 512
    A = _planes(rng, K * M, 4096)
    B = _planes(rng, M * N, 4096)
    cn = g.limbs_needed(128, 128, M, path=g.PATH_CRT)
    return K, M, N, A, B, cn, _expect(orc, K, M, N, A, B, cn)


def test_cfg3_crt_device_full_output(g, cfg3):
    K, M, N, A, B, cn, exp = cfg3
    dA, dB = g.DeviceMatrix(K, M, 128), g.DeviceMatrix(M, N, 128)
    dA.upload(*A)
    dB.upload(*B)
    dC = g.DeviceMatrix(K, N, cn)
    g.default_handle().matmul(dC, dA, dB, path=g.PATH_CRT)
    _same(dC.download(), exp)


@pytest.mark.parametrize("cutoff", [32, 64])
def test_cfg3_limb_winograd_full_output(g, cfg3, cutoff):
    """The plain limb form the CRT path is compared against: Winograd's tree on
    one-limb-longer sums (129 limbs) down to the cutoff."""
    K, M, N, A, B, cn, exp = cfg3
    dA, dB = g.DeviceMatrix(K, M, 128), g.DeviceMatrix(M, N, 128)
    dA.upload(*A)
    dB.upload(*B)
    dC = g.DeviceMatrix(K, N, cn)
    g.default_handle().matmul(dC, dA, dB, path=g.PATH_LIMB, method=g.METHOD_WINOGRAD, cutoff=cutoff)
    _same(dC.download(), exp)


def test_cfg3_crt_host_buffers_full_output(g, cfg3):
    K, M, N, A, B, cn, exp = cfg3
    outs = [(np.zeros((cn, K * N), dtype=np.uint32), np.zeros(K * N, dtype=np.int32)) for _ in range(2)]
    h = g.Handle()
    h.matmul_host(h.host_jobs([(K, M, N, A, B, o) for o in outs], path=g.PATH_CRT))
    for o in outs:
        _same(o, exp)
    h.close()


@pytest.fixture(scope="module")
def cfg2(g, orc):
    rng = np.random.default_rng(77)
    K = M = N = 256
    A = _planes(rng, K * M, 2048, 0.05, 0.05, 64)
    B = _planes(rng, M * N, 2048, 0.05, 0.05, 64)
    cn = g.limbs_needed(64, 64, M, path=g.PATH_LIMB, method=g.METHOD_WINOGRAD, cutoff=32)
    return K, M, N, A, B, cn, _expect(orc, K, M, N, A, B, cn)


@pytest.mark.parametrize("path,method", [("limb", "winograd"), ("limb", "naive"), ("crt", "naive")])
def test_cfg2_full_output(g, cfg2, path, method):
    K, M, N, A, B, cn, exp = cfg2
    dA, dB = g.DeviceMatrix(K, M, 64), g.DeviceMatrix(M, N, 64)
    dA.upload(*A)
    dB.upload(*B)
    dC = g.DeviceMatrix(K, N, cn)
    g.default_handle().matmul(dC, dA, dB, path={"limb": g.PATH_LIMB, "crt": g.PATH_CRT}[path],
                              method={"winograd": g.METHOD_WINOGRAD, "naive": g.METHOD_NAIVE}[method], cutoff=32)
    _same(dC.download(), exp)


def test_cfg4_batched_draw_full_output(g, orc):
    """The uneven workload's own generator and seed; every product checked in
    full after the eager call, after the call that captures the CUDA graph and
    after a replay of that graph."""
    import bench
    W = bench.WORKLOADS["cfg4"]
    mats, _ = bench.gen_jobs(g, W, 2024)
    exps = [_expect(orc, K, M, N, (Al, As), (Bl, Bs), dC.nlimbs) for dC, _, _, (Al, As, Bl, Bs, K, M, N) in mats]
    import torch
    # a stream of its own: on the legacy default stream a batch never captures a graph
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        h = g.Handle()
        jobs = h.jobs([(c, a, b) for c, a, b, _ in mats])
        for call in range(3):
            for dC, _, _, _ in mats:
                dC.limbs_t.fill_(-1)   # stale output must not survive a call
                dC.sizes_t.fill_(7)
            chosen = h.matmul_batched(jobs)
            for i, ((dC, _, _, (_, _, _, _, K, M, N)), exp) in enumerate(zip(mats, exps)):
                try:
                    _same(dC.download(), exp)
                except AssertionError as e:
                    raise AssertionError(f"call {call}, job {i} ({K}x{M}x{N}, path {chosen[i]}): {e}") from None
        h.close()
    torch.cuda.current_stream().wait_stream(s)
