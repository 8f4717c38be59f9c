"""Learned cost model: GPU forward / backward kernels against a float64 numpy
restatement (the oracle for this floating-point part), training, and the gain
of the trained model over the plain heuristic on measured job timings."""
import json
import random

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NF, NH, NO = 8, 64, 8   # features, hidden width, heads (one per gbmm_plan)


def _unpack(w):
    o = 0
    W1 = w[o:o + NF * NH].reshape(NF, NH); o += NF * NH
    b1 = w[o:o + NH]; o += NH
    W2 = w[o:o + NH * NH].reshape(NH, NH); o += NH * NH
    b2 = w[o:o + NH]; o += NH
    W3 = w[o:o + NH * NO].reshape(NH, NO); o += NH * NO
    b3 = w[o:o + NO]
    return W1, b1, W2, b2, W3, b3


def _bf16_to_f64(b):
    return (b.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def _ref_forward(w, X):
    W1, b1, W2, b2, W3, b3 = _unpack(w)
    z1 = X @ W1 + b1
    h1 = np.maximum(z1, 0)
    z2 = h1 @ W2 + b2
    h2 = np.maximum(z2, 0)
    return h1, h2, h2 @ W3 + b3


def _ref_grad(w, X, T):
    W1, b1, W2, b2, W3, b3 = _unpack(w)
    h1, h2, Y = _ref_forward(w, X)
    mask = ~np.isnan(T)
    cnt = mask.sum()
    E = np.where(mask, Y - np.nan_to_num(T), 0.0)
    loss = (E * E).sum() / cnt
    dY = 2 * E / cnt
    gW3 = h2.T @ dY
    gb3 = dY.sum(0)
    dh2 = (dY @ W3.T) * (h2 > 0)
    gW2 = h1.T @ dh2
    gb2 = dh2.sum(0)
    dh1 = (dh2 @ W2.T) * (h1 > 0)
    gW1 = X.T @ dh1
    gb1 = dh1.sum(0)
    return np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3]), loss


@pytest.fixture
def h(built_lib):
    import gbmm
    hh = gbmm.Handle()
    hh.model_init(seed=3)
    yield hh
    hh.close()


def _data(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.uniform(0, 1.2, size=(n, NF)).astype(np.float32)
    T = np.stack([np.sin(3 * X[:, 0]) + X[:, 5], X[:, 1] * X[:, 3] - 0.5, np.cos(2 * X[:, 4]) * X[:, 2],
                  X[:, 6] - X[:, 7], np.sin(X[:, 1] + X[:, 2]), X[:, 0] * X[:, 4], 0.3 * X[:, 3] + 0.1,
                  np.cos(X[:, 5] * X[:, 6])], 1)
    T = T.astype(np.float32)
    T[rng.random(T.shape) < 0.1] = np.nan
    return X, T


def test_forward_matches_float64(h):
    X, _ = _data(300, 1)
    _, w16 = h.model_params()
    _, _, Yref = _ref_forward(_bf16_to_f64(w16), X.astype(np.float64))
    Y = h.model_predict(X)
    assert np.allclose(Y, Yref, rtol=1e-4, atol=1e-4)


def test_backward_matches_float64(h):
    X, T = _data(257, 2)
    _, w16 = h.model_params()
    gref, lref = _ref_grad(_bf16_to_f64(w16), X.astype(np.float64), T.astype(np.float64))
    g, loss = h.model_gradient(X, T)
    assert abs(loss - lref) <= 1e-4 * max(1.0, abs(lref))
    # FP32 accumulation against float64: tolerance relative to the gradient scale
    assert np.max(np.abs(g - gref)) <= 2e-4 * np.max(np.abs(gref)) + 1e-6


def test_training_reduces_loss(h):
    X, T = _data(512, 3)
    _, l0 = h.model_gradient(X, T)
    lf = h.model_train(X, T, epochs=600, lr=3e-3)
    _, l1 = h.model_gradient(X, T)
    assert l1 < 0.2 * l0 and abs(l1 - lf) < 0.05 * l0


def _stream(gbmm, seed, n):
    """n products of uneven shape (dims log-uniform in [8, 384]) and bit length
    (log-uniform in [64, 4096] per matrix), uploaded: [(A, B, C, host planes)]."""
    rng = np.random.default_rng(seed)
    lu = lambda lo, hi: int(round(float(np.exp(rng.uniform(np.log(lo), np.log(hi))))))
    import bench
    mats = []
    for _ in range(n):
        K, M, N, ba, bb = lu(8, 384), lu(8, 384), lu(8, 384), lu(64, 4096), lu(64, 4096)
        Al, As = bench.gen_planes(rng, K * M, ba, 0.05, 0.0, 0)
        Bl, Bs = bench.gen_planes(rng, M * N, bb, 0.05, 0.0, 0)
        dA, dB = gbmm.DeviceMatrix(K, M, Al.shape[0]), gbmm.DeviceMatrix(M, N, Bl.shape[0])
        dA.upload(Al, As)
        dB.upload(Bl, Bs)
        dC = gbmm.DeviceMatrix(K, N, Al.shape[0] + Bl.shape[0] + 2)
        mats.append((dA, dB, dC, (Al, As, Bl, Bs)))
    return mats


def _tune(gbmm, h, mats, log):
    """Times every admissible plan of every product (autotuner); returns
    {(m, k, n, la, lb): [ms per plan, NaN where not timed]}."""
    h.autotune(h.jobs([(c, a, b) for a, b, c, _ in mats]), repeats=2, log_path=log)
    times = {}
    for r in (json.loads(l) for l in open(log)):
        times.setdefault((r["m"], r["k"], r["n"], r["la"], r["lb"]), [np.nan] * NO)[r["plan"]] = r["ms"]
    return times


def test_learned_dispatch_gains_over_heuristic_out_of_sample(built_lib, tmp_path):
    """The model trains on the autotuner's timings of every plan on one seeded
    stream of 96 uneven products.  On a separately drawn stream of 64 every
    admissible plan of every product is timed too; the summed measured time of
    the plans the learned dispatcher picks must be below the summed time of the
    plain heuristic's picks.  Both dispatchers' batched calls stay exact."""
    import gbmm
    import bench
    train = _stream(gbmm, 17, 96)
    ht = gbmm.Handle()
    tt = _tune(gbmm, ht, train, str(tmp_path / "train.jsonl"))
    keys = sorted(tt)
    X = np.stack([gbmm.model_features(*k) for k in keys])
    T = np.log2(np.array([tt[k] for k in keys], dtype=np.float64)).astype(np.float32)
    hl = gbmm.Handle()
    hl.model_init(seed=5)
    hl.model_train(X, T, epochs=2000, lr=3e-3)
    hl.model_use(True)
    del train
    evals = _stream(gbmm, 99, 64)
    he = gbmm.Handle()
    et = _tune(gbmm, he, evals, str(tmp_path / "eval.jsonl"))
    hh = gbmm.Handle()
    pick_h = hh.matmul_batched(hh.jobs([(c, a, b) for a, b, c, _ in evals]), plans=True)
    pick_l = hl.matmul_batched(hl.jobs([(c, a, b) for a, b, c, _ in evals]), plans=True)
    cost_h = cost_l = best = 0.0
    changed = 0
    for (dA, dB, dC, _), (_, qh), (_, ql) in zip(evals, pick_h, pick_l):
        t = et[(dA.rows, dA.cols, dB.cols, dA.nlimbs, dB.nlimbs)]
        assert not np.isnan(t[qh]) and not np.isnan(t[ql])
        cost_h += t[qh]
        cost_l += t[ql]
        best += np.nanmin(t)
        changed += qh != ql
    srng = np.random.default_rng(1)
    for dA, dB, dC, (Al, As, Bl, Bs) in evals:
        Cl, Cs = dC.download()
        y, x = int(srng.integers(dA.rows)), int(srng.integers(dB.cols))
        exp = sum(bench.entry_int(Al, As, y * dA.cols + k) * bench.entry_int(Bl, Bs, k * dB.cols + x)
                  for k in range(dA.cols))
        assert bench.entry_int(Cl, Cs, y * dB.cols + x) == exp
    print(f"held-out stream, summed measured ms of the picked plans: heuristic {cost_h:.3f}, "
          f"learned {cost_l:.3f}, best possible {best:.3f}; {changed} of {len(evals)} picks differ")
    assert cost_l < cost_h
    for x in (ht, hl, he, hh):
        x.close()
