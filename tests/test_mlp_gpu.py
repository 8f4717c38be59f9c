"""Learned cost model: GPU forward / backward kernels against a float64 numpy
restatement (the oracle for this floating-point part), training, and the gain
of the trained model over the plain heuristic on measured job timings."""
import json
import random

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NF, NH, NO = 8, 64, 3


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
    T = np.stack([np.sin(3 * X[:, 0]) + X[:, 5], X[:, 1] * X[:, 3] - 0.5, np.cos(2 * X[:, 4]) * X[:, 2]], 1)
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


def test_learned_dispatch_gains_over_heuristic(built_lib, tmp_path):
    """Times the three candidate plans of a stream of uneven products with the
    autotuner, trains the model on those timings, and compares the measured
    cost of the plans each dispatcher picks."""
    import gbmm
    rng = random.Random(17)
    specs = []
    for _ in range(40):
        dims = [int(round(np.exp(rng.uniform(np.log(8), np.log(160))))) for _ in range(3)]
        bits = [int(round(np.exp(rng.uniform(np.log(64), np.log(4096))))) for _ in range(2)]
        specs.append((*dims, *bits))
    mats = []
    for K, M, N, ba, bb in specs:
        la, lb = (ba + 31) // 32, (bb + 31) // 32
        A = [rng.getrandbits(ba) * rng.choice((-1, 1)) for _ in range(K * M)]
        B = [rng.getrandbits(bb) * rng.choice((-1, 1)) for _ in range(M * N)]
        dA = gbmm.DeviceMatrix.from_ints(K, M, A, la)
        dB = gbmm.DeviceMatrix.from_ints(M, N, B, lb)
        need = gbmm.limbs_needed(la, lb, M, path=gbmm.PATH_LIMB, cutoff=64)
        mats.append((dA, dB, gbmm.DeviceMatrix(K, N, need)))
    hh = gbmm.Handle()
    jobs = hh.jobs([(c, a, b) for a, b, c in mats])
    log = str(tmp_path / "t.jsonl")
    hh.autotune(jobs, repeats=2, log_path=log)
    rows = [json.loads(l) for l in open(log)]
    head = lambda r: 2 if r["path"] == gbmm.PATH_CRT else (0 if r["method"] == gbmm.METHOD_NAIVE else 1)
    times = {}
    for r in rows:
        times.setdefault((r["m"], r["k"], r["n"], r["la"], r["lb"]), [np.nan] * 3)[head(r)] = r["ms"]
    keys = sorted(times)
    X = np.stack([gbmm.model_features(m, k, n, la, lb) for (m, k, n, la, lb) in keys])
    T = np.log2(np.array([times[k] for k in keys], dtype=np.float64)).astype(np.float32)
    hh.model_init(seed=5)
    hh.model_train(X, T, epochs=1500, lr=3e-3)
    pred = hh.model_predict(X)
    tm = np.array([times[k] for k in keys])
    choose_model = np.nanargmin(np.where(np.isnan(T), np.inf, pred), axis=1)
    # the heuristic's choice, as the dispatcher makes it without a model or table
    h0 = gbmm.Handle()
    chosen = h0.matmul_batched(h0.jobs([(c, a, b) for a, b, c in mats]))
    by_key = {(a.rows, a.cols, b.cols, a.nlimbs, b.nlimbs): p for (a, b, c), p in zip(mats, chosen)}
    choose_heur = np.array([2 if by_key[k] == gbmm.PATH_CRT else 1 for k in keys])
    cost = lambda ch: float(np.nansum([tm[i, ch[i]] if not np.isnan(tm[i, ch[i]]) else np.nanmax(tm[i])
                                       for i in range(len(keys))]))
    best = float(np.nansum(np.nanmin(tm, axis=1)))
    t_model, t_heur = cost(choose_model), cost(choose_heur)
    print(f"measured ms: heuristic {t_heur:.3f}, learned {t_model:.3f}, best {best:.3f}")
    assert t_model <= t_heur * 1.02
    hh.close()
    h0.close()
