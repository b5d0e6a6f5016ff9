"""Learned starting radius: the CUDA forward / backward kernels against a
float64 numpy restatement, exactness of the join under any model, a short
training run, and what a trained model saves over the plain BETA schedule."""
import ctypes

import numpy as np
import pytest

import oracle
import hybrid_k_nearest_neighbor_self_join_gb300 as kj
from hybrid_k_nearest_neighbor_self_join_gb300 import _lib, datasets, train_radius

pytestmark = pytest.mark.gpu

NF, NH = 24, 64


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build_library()
    __graft_entry__.build_oracle()
    yield
    kj.set_radius_model(None)


def unpack(m):
    m = m.astype(np.float64)
    o = 0
    mean = m[o:o + NF]; o += NF
    istd = m[o:o + NF]; o += NF
    W1 = m[o:o + NF * NH].reshape(NF, NH); o += NF * NH
    b1 = m[o:o + NH]; o += NH
    W2 = m[o:o + NH * NH].reshape(NH, NH); o += NH * NH
    b2 = m[o:o + NH]; o += NH
    W3 = m[o:o + NH]; o += NH
    b3 = m[o]
    return mean, istd, W1, b1, W2, b2, W3, b3


def np_forward(m, X):
    mean, istd, W1, b1, W2, b2, W3, b3 = unpack(m)
    x = (X.astype(np.float64) - mean) * istd
    a1 = x @ W1 + b1
    h1 = np.maximum(a1, 0)
    a2 = h1 @ W2 + b2
    h2 = np.maximum(a2, 0)
    return x, a1, h1, a2, h2, h2 @ W3 + b3


def np_grad(m, X, Y, q):
    mean, istd, W1, b1, W2, b2, W3, b3 = unpack(m)
    x, a1, h1, a2, h2, y = np_forward(m, X)
    n = len(Y)
    e = Y.astype(np.float64) - y
    loss = np.where(e > 0, q * e, (q - 1) * e).mean()
    dy = np.where(e > 0, -q, 1 - q) / n
    dW3 = h2.T @ dy
    db3 = dy.sum()
    g2 = np.outer(dy, W3) * (a2 > 0)
    dW2 = h1.T @ g2
    db2 = g2.sum(0)
    g1 = (g2 @ W2.T) * (a1 > 0)
    dW1 = x.T @ g1
    db1 = g1.sum(0)
    return np.concatenate([dW1.ravel(), db1, dW2.ravel(), db2, dW3, [db3]]), loss


def random_model(seed):
    rng = np.random.default_rng(seed)
    m = np.zeros(_lib.RADIUS_MODEL_FLOATS, np.float32)
    m[:NF] = rng.normal(0, 0.5, NF)
    m[NF:2 * NF] = rng.uniform(0.5, 2.0, NF)
    m[2 * NF:] = rng.normal(0, 0.3, len(m) - 2 * NF)
    return m


def bf16(a):
    """float32 -> nearest bfloat16 (ties to even), returned as float32."""
    b = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


def np_forward_bf16(m, X):
    """The tensor-core evaluation: BF16 operands (normalised features,
    first-layer activations, W1, W2), FP32 accumulation, biases, ReLU and
    the last layer in FP32."""
    mean, istd = m[:NF], m[NF:2 * NF]
    W1 = m[2 * NF:2 * NF + NF * NH].reshape(NF, NH)
    o = 2 * NF + NF * NH
    b1 = m[o:o + NH]; o += NH
    W2 = m[o:o + NH * NH].reshape(NH, NH); o += NH * NH
    b2 = m[o:o + NH]; o += NH
    W3 = m[o:o + NH]; b3 = m[o + NH]
    x = bf16((X - mean) * istd).astype(np.float64)
    h1 = np.maximum(x @ bf16(W1).astype(np.float64) + b1, 0)
    a2 = np.maximum(bf16(h1.astype(np.float32)).astype(np.float64) @ bf16(W2).astype(np.float64) + b2, 0)
    return a2 @ W3 + b3


def test_forward_matches_numpy(monkeypatch):
    m = random_model(1)
    X = np.random.default_rng(2).normal(0, 1, (3000, NF)).astype(np.float32)
    # the FP32 CUDA-core evaluation: the training forward pass
    monkeypatch.setenv("KNNSJ_RADIUS_MLP", "fp32")
    got = train_radius.predict(m, X)
    want = np_forward(m, X)[-1]
    assert np.allclose(got, want, rtol=1e-4, atol=1e-4)
    # the tensor-core evaluation (tcgen05, BF16 operands), as the join uses
    # it: equal to a BF16 restatement up to FP32 summation order
    monkeypatch.delenv("KNNSJ_RADIUS_MLP")
    got = train_radius.predict(m, X)
    want = np_forward_bf16(m, X)
    # (a BF16 rounding of a first-layer activation can flip with the FP32
    # summation order: one BF16 unit, 2^-8 relative, through W2)
    assert np.allclose(got, want, rtol=5e-3, atol=5e-2), np.abs(got - want).max()
    assert np.corrcoef(got, want)[0, 1] > 0.9999
    assert np.abs(got - np_forward(m, X)[-1]).max() < 0.5  # and close to the FP32 model


@pytest.mark.parametrize("q", [0.5, 0.9])
def test_gradient_matches_numpy(q):
    m = random_model(3)
    rng = np.random.default_rng(4)
    X = rng.normal(0, 1, (1000, NF)).astype(np.float32)
    Y = rng.normal(0, 1, 1000).astype(np.float32)
    g = np.empty(_lib.RADIUS_MODEL_FLOATS - 2 * NF, np.float32)
    loss = ctypes.c_double(0)
    _lib.check(_lib.load().knnsj_radius_grad(m.ctypes.data, X.ctypes.data, Y.ctypes.data, 1000, q,
                                             g.ctypes.data, ctypes.byref(loss)))
    want, wl = np_grad(m, X, Y, q)
    scale = np.abs(want).max()
    assert np.max(np.abs(g - want)) <= 1e-4 * scale + 1e-6
    assert abs(loss.value - wl) <= 1e-5 * abs(wl) + 1e-6
    # deterministic: same bits on a second call
    g2 = np.empty_like(g)
    _lib.check(_lib.load().knnsj_radius_grad(m.ctypes.data, X.ctypes.data, Y.ctypes.data, 1000, q,
                                             g2.ctypes.data, ctypes.byref(loss)))
    assert np.array_equal(g, g2)


@pytest.mark.parametrize("model_seed", [None, 5])
def test_learned_mode_is_exact(model_seed):
    if model_seed is not None:
        kj.set_radius_model(random_model(model_seed))
    try:
        cases = [(datasets.sky_like(200_000, seed=8), 64, 2, 0.025),
                 (datasets.gmm(40_000, 6, 10, 0.1, seed=9, dtype=np.float64), 16, 6, 0.05),
                 (datasets.heldout4d(60_000, seed=10), 128, 4, 0.05),
                 (datasets.gmm(30_000, 5, 8, 0.2, seed=11, dtype=np.float32), 10, 3, 0.05)]
        for x, k, di, beta in cases:
            ids, dists = kj.selfjoin(x, k, num_indexed_dims=di, beta=beta, radius_mode=kj.RADIUS_LEARNED)
            rc, oids, odists, _ = oracle.join(x, k, di=di, beta=beta)
            assert rc == 0
            assert np.array_equal(ids, oids)
            assert np.array_equal(dists, odists)
    finally:
        kj.set_radius_model(None)


def test_training_reduces_loss_and_saves_work():
    # a small training run on seeded sets, evaluated on a held-out set
    rng = np.random.default_rng(0)
    Xs, Ys = [], []
    for i, x, beta in train_radius.training_sets(6, 200_000, seed=21):
        X, Y = train_radius.collect(x, beta, 20_000, rng)
        Xs.append(X)
        Ys.append(Y)
    X, Y = np.concatenate(Xs), np.concatenate(Ys)
    model, loss = train_radius.train(X, Y, epochs=6, quantile=0.9, seed=3)
    assert loss[-1] < loss[0]
    held = datasets.gmm(200_000, 3, 30, 0.2, seed=99, sd_lo=0.002, sd_hi=0.05, dtype=np.float32)
    plain = kj.selfjoin(held, 32, beta=0.05, return_stats=True)
    kj.set_radius_model(model)
    try:
        learned = kj.selfjoin(held, 32, beta=0.05, radius_mode=kj.RADIUS_LEARNED, return_stats=True)
    finally:
        kj.set_radius_model(None)
    assert np.array_equal(plain[0], learned[0]) and np.array_equal(plain[1], learned[1])
    # fewer re-attempts than the plain BETA schedule
    assert learned[2]["queries_run"] < plain[2]["queries_run"]
