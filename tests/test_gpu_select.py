"""The learned (direction, ordering, kernel) selector: the MLP's hand-written CUDA
forward / backward / Adam kernels against the double-precision oracle, the device graph
statistics, and the selector's gain over the method without it (the reference's cost
function with a fixed kernel) on measured timings."""
import os

import numpy as np
import pytest

import atc
import oracle

pytestmark = pytest.mark.gpu

FIXTURE = os.path.join(os.path.dirname(__file__), "golden", "select_timings.npz")


@pytest.fixture(scope="module", autouse=True)
def _init(gpu_ready):
    yield


def _problem(rng, B, I=6, O=24):
    x = rng.normal(size=(B, I)).astype(np.float32) * 2 + 1
    t = rng.normal(size=(B, O)).astype(np.float32)
    mask = (rng.random((B, O)) > 0.2).astype(np.float32)
    return x, t, mask


@pytest.mark.parametrize("B,H", [(1, 64), (37, 64), (256, 16)])
def test_mlp_gradients_match_oracle(B, H):
    rng = np.random.default_rng(B + H)
    net = atc.MLP(6, H, 24, seed=B)
    mean = rng.normal(size=6).astype(np.float32)
    std = (rng.random(6) + 0.5).astype(np.float32)
    net.scaling(mean, std)
    x, t, mask = _problem(rng, B)
    loss, g = net.gradients(x, t, mask)
    rloss, rg = oracle.mlp_grad(net.params(), 6, H, 24, mean, std, x, t, mask)
    assert abs(loss - rloss) <= 1e-4 * max(1.0, abs(rloss))
    scale = np.abs(rg).max()
    assert np.abs(g - rg).max() <= 2e-4 * scale, (np.abs(g - rg).max(), scale)


def test_mlp_forward_matches_oracle_loss():
    rng = np.random.default_rng(3)
    net = atc.MLP(6, 64, 24, seed=3)
    x, t, _ = _problem(rng, 50)
    y = net.forward(x)
    m, s = net.scaling()
    rloss, _ = oracle.mlp_grad(net.params(), 6, 64, 24, m, s, x, y)  # targets = outputs: zero loss
    assert rloss < 1e-9


def test_mlp_training_reduces_loss():
    rng = np.random.default_rng(5)
    x = rng.normal(size=(2048, 6)).astype(np.float32)
    w = rng.normal(size=(6, 24)).astype(np.float32)
    t = np.tanh(x @ w) + 0.5 * (x[:, :1] ** 2)
    net = atc.MLP(6, 64, 24, seed=5)
    m, s = x.mean(0), x.std(0)
    net.scaling(m, s)
    before, _ = net.gradients(x, t)
    net.train(x, t, epochs=60, batch=256, lr=3e-3, seed=5)
    after, _ = net.gradients(x, t)
    assert after < 0.1 * before, (before, after)
    # deterministic: the same seed trains to the same parameters
    net2 = atc.MLP(6, 64, 24, seed=5)
    net2.train(x, t, epochs=60, batch=256, lr=3e-3, seed=5)
    assert np.array_equal(net.params(), net2.params())


def test_graph_features_known_values():
    import torch
    # a star with 4 leaves plus a triangle on leaves 1,2,3; one self-loop (ignored)
    pairs = np.array([[0, 1], [0, 2], [0, 3], [0, 4], [1, 2], [2, 3], [3, 1], [2, 2]], dtype=np.int32)
    d = torch.from_numpy(pairs).cuda()
    f = atc.graph_features(d.data_ptr(), pairs.shape[0])
    deg = np.array([4, 3, 3, 3, 1], dtype=np.float64)
    n, m = 5, 7
    assert np.allclose(f[:5], np.log1p([n, m, deg.mean(), deg.var(), deg.max()]), rtol=1e-6)
    # degree orientation (lower degree first, ties to the larger id): out-degrees
    dout = np.zeros(5)
    for u, v in pairs:
        if u == v:
            continue
        src = u if (deg[u] < deg[v] or (deg[u] == deg[v] and u > v)) else v
        dout[src] += 1
    avg = m / n
    tail = sum(o - avg for o in dout if o - avg > avg)
    assert np.isclose(f[5], np.log1p(tail), rtol=1e-6)


def test_selector_gains_over_cost_function():
    if not os.path.exists(FIXTURE):
        pytest.skip("timings fixture not generated yet")
    import bench
    d = np.load(FIXTURE)
    feats, times, costs = d["features"], d["times_ms"], d["costs"]
    ntr = int(0.75 * feats.shape[0])
    res = bench.train_and_evaluate(feats, times, costs, ntr, seed=1)
    pol = res["policies"]
    assert pol["learned"]["ms"] < pol["cost_function"]["ms"], pol
    assert pol["learned"]["ms"] <= pol["fixed_default"]["ms"], pol
