"""The surrogate network's kernels against an FP64 CPU MLP, and what the
trained network gains over plain Monte Carlo."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def silu(z):
    return z / (1.0 + np.exp(-z))


def cpu_forward(layers, X):
    """FP64 forward; returns y and the per-layer (A, Z) for backward."""
    A = np.asarray(X, np.float64)
    cache = []
    for W, b in layers[:-1]:
        Z = A @ W.T.astype(np.float64) + b
        cache.append((A, Z))
        A = silu(Z)
    W, b = layers[-1]
    y = A @ W[0].astype(np.float64) + b[0]
    return y, cache, A


def cpu_gradients(layers, X, t):
    """FP64 gradients of mean (y - t)^2 in the library's parameter layout."""
    y, cache, Hl = cpu_forward(layers, X)
    B = len(t)
    dy = 2.0 * (y - t) / B
    grads = [None] * len(layers)
    W, b = layers[-1]
    grads[-1] = (np.outer([1.0], dy @ Hl), np.array([dy.sum()]))
    dH = np.outer(dy, W[0])
    for l in range(len(layers) - 2, -1, -1):
        A, Z = cache[l]
        s = 1.0 / (1.0 + np.exp(-Z))
        dZ = dH * s * (1.0 + Z * (1.0 - s))
        grads[l] = (dZ.T @ A, dZ.sum(0))
        dH = dZ @ layers[l][0].astype(np.float64)
    flat = []
    for gW, gb in grads:
        flat += [np.ravel(gW), np.ravel(gb)]
    return np.concatenate(flat), float(np.mean((y - t) ** 2))


def test_gradients_match_fp64_cpu(dev):
    from axonexa_gb300.surrogate import MLP
    rng = np.random.default_rng(0)
    m = MLP(seed=3, device=dev)
    X = rng.uniform(-1, 1, size=(512, 10))
    t = np.sin(X[:, 0] * 2) * 0.3 + 0.5 + 0.1 * X[:, 1] * X[:, 2]
    g, loss = m.gradients(X, t)
    ref, ref_loss = cpu_gradients(m.layers(), X, t)
    assert abs(loss - ref_loss) <= 2e-2 * ref_loss + 1e-6
    # BF16 operands, FP32 accumulation: agreement to about 1 %
    rel = np.linalg.norm(g - ref) / np.linalg.norm(ref)
    assert rel < 3e-2, rel
    cos = float(g @ ref / (np.linalg.norm(g) * np.linalg.norm(ref)))
    assert cos > 0.999, cos
    # per layer, too
    o = 0
    for W, b in m.layers():
        n = W.size + b.size
        seg, rs = g[o:o + n], ref[o:o + n]
        assert np.linalg.norm(seg - rs) <= 5e-2 * np.linalg.norm(rs) + 1e-8
        o += n


def test_tensor_core_forward_matches_fp64_cpu(dev):
    from axonexa_gb300.surrogate import MLP
    rng = np.random.default_rng(1)
    m = MLP(seed=5, device=dev)
    # make the network non-trivial: a few training steps on a smooth target
    X = rng.uniform(-1, 1, size=(8192, 10))
    t = 0.5 + 0.3 * np.tanh(X[:, 0] + 0.5 * X[:, 3] * X[:, 4])
    m.train(X, t, batch=1024, steps=50, lr=1e-3, seed=1)
    Q = rng.uniform(-1, 1, size=(1000, 10))  # not a multiple of the 128-row tile
    y = m.predict(Q)
    ref, _, _ = cpu_forward(m.layers(), Q)
    err = np.abs(y - ref)
    assert np.all(np.isfinite(y))
    assert err.max() < 2e-2 * max(1.0, np.abs(ref).max()), err.max()
    assert err.mean() < 5e-3, err.mean()


def test_host_memory_chunks_equal_device_inference(dev):
    """Inference from host memory runs as a pipeline of chunks (whole waves
    of the persistent kernel); every row is independent, so the outputs equal
    one device-resident launch over all rows bit for bit, for a ragged row
    count over several chunks, into a caller's array, and again on the kept
    buffers with fewer rows."""
    import torch
    from axonexa_gb300.surrogate import MLP
    rng = np.random.default_rng(4)
    m = MLP(seed=7, device=dev)
    for n in (100_003, 38_913, 1):
        Q = rng.uniform(-1, 1, size=(n, 10)).astype(np.float32)
        X = torch.from_numpy(Q).cuda()
        y = torch.empty(n, device="cuda")
        m.predict_device(X.data_ptr(), n, y.data_ptr())
        torch.cuda.synchronize()
        out = np.full(n, np.nan, np.float32)
        got = m.predict(Q, out=out)
        assert got is out
        np.testing.assert_array_equal(out, y.cpu().numpy())
    with pytest.raises(ValueError):
        m.predict(Q, out=np.zeros(n + 1, np.float32))
    m.close()


def test_training_reduces_loss(dev):
    from axonexa_gb300.surrogate import MLP
    rng = np.random.default_rng(2)
    X = rng.uniform(-1, 1, size=(20000, 10))
    t = 0.5 + 0.25 * np.sin(2 * X[:, 0]) * np.cos(X[:, 1]) + 0.1 * X[:, 5]
    m = MLP(seed=7, device=dev)
    loss = m.train(X, t, batch=4096, steps=600, lr=2e-3, seed=3)
    assert loss[-50:].mean() < 0.05 * loss[:5].mean()
    Q = rng.uniform(-1, 1, size=(4000, 10))
    tq = 0.5 + 0.25 * np.sin(2 * Q[:, 0]) * np.cos(Q[:, 1]) + 0.1 * Q[:, 5]
    assert np.sqrt(np.mean((m.predict(Q) - tq) ** 2)) < 0.02


def test_surrogate_gain_over_plain_monte_carlo(dev):
    """Small version of the surrogate workflow: the network is trained on
    signals the walk produced for random gamma-radius packings; on held-out
    substrates it answers within the Monte Carlo noise, at far more signals/s
    than the walk that made its training data; out-of-range queries fall back
    to the walk."""
    import axonexa_gb300.surrogate as S
    walkers, dt = 32768, 0.01
    t0 = time.perf_counter()
    P, Y = S.generate(48, seed=1, walkers=walkers, timestep=dt, n_cyl=40, device=dev)
    t_mc = time.perf_counter() - t0
    mc_rate = len(Y) / t_mc
    Ph, Yh = S.generate(8, seed=99, walkers=walkers, timestep=dt, n_cyl=40, device=dev)
    sur = S.Surrogate.fit(P, Y, steps=1500, batch=2048, lr=1e-3, seed=0, device=dev)
    pred, fb = sur.predict(Ph)
    assert not fb.any()
    err = np.abs(pred - Yh)
    # Monte Carlo noise of one training signal is about 1/sqrt(walkers) ~ 0.006
    assert err.mean() < 0.03, err.mean()
    # versus the method without the network: a constant guess (training mean)
    assert err.mean() < 0.5 * np.abs(Yh - Y.mean()).mean()
    # throughput: 1e5 queries through the tensor cores
    Q = np.tile(Ph, (100000 // len(Ph) + 1, 1))[:100000]
    sur.mlp.predict(Q[:1000])
    t0 = time.perf_counter()
    sur.mlp.predict(Q)
    t_nn = time.perf_counter() - t0
    nn_rate = len(Q) / t_nn
    assert nn_rate > 100 * mc_rate, (nn_rate, mc_rate)
    # out-of-range queries are simulated instead of predicted
    out = Ph[:2].copy()
    out[:, 0] = 6.0  # mean radius beyond the training range
    val, fb = sur.predict(out, fallback_walkers=4096, timestep=dt, n_cyl=40)
    assert fb.all() and np.all((val > 0) & (val <= 1.0))
