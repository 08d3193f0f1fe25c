"""The learned proposal's CPU oracle: autoregressive masks and gradients (finite differences)."""
import numpy as np
import pytest

from oracle.made_oracle import MADE, adam_step, masks


def _params(n, hidden, rng, dtype=np.float32):
    return {"W1": rng.normal(0, 0.5, (hidden, n)).astype(dtype), "b1": rng.normal(0, 0.1, hidden).astype(dtype),
            "W2": rng.normal(0, 0.3, (hidden, hidden)).astype(dtype), "b2": rng.normal(0, 0.1, hidden).astype(dtype),
            "W3": rng.normal(0, 0.3, (n, hidden)).astype(dtype), "b3": rng.normal(0, 0.1, n).astype(dtype)}


def test_output_i_depends_on_earlier_sites_only():
    n, hidden = 7, 12
    rng = np.random.default_rng(0)
    net = MADE(_params(n, hidden, rng), n, hidden)
    x = rng.integers(0, 2, (1, n))
    o, _ = net.forward(x)
    for j in range(n):
        y = x.copy()
        y[0, j] ^= 1
        oy, _ = net.forward(y)
        changed = np.nonzero(np.abs(oy - o)[0] > 0)[0]
        assert (changed > j).all(), (j, changed)


def test_probabilities_sum_to_one():
    n, hidden = 5, 8
    net = MADE(_params(n, hidden, np.random.default_rng(1)), n, hidden)
    allx = np.array([[(k >> i) & 1 for i in range(n)] for k in range(2**n)])
    assert abs(np.exp(net.logq(allx)).sum() - 1) < 1e-5


def test_gradients_match_finite_differences():
    n, hidden = 6, 10
    rng = np.random.default_rng(2)
    net = MADE(_params(n, hidden, rng, np.float64), n, hidden, bf16_weights=False, dtype=np.float64)
    x = rng.integers(0, 2, (9, n))
    _, g = net.loss_and_grads(x)
    m1, m2, m3 = masks(n, hidden)
    mask = {"W1": m1, "W2": m2, "W3": m3}
    h = 1e-6
    for k in ("W1", "b1", "W2", "b2", "W3", "b3"):
        for idx in [tuple(rng.integers(0, s) for s in net.p[k].shape) for _ in range(6)]:
            if k in mask and mask[k][idx] == 0:
                assert g[k][idx] == 0
                continue
            old = net.p[k][idx]
            net.p[k][idx] = old + h
            lp, _ = net.loss_and_grads(x)
            net.p[k][idx] = old - h
            lm, _ = net.loss_and_grads(x)
            net.p[k][idx] = old
            assert abs((lp - lm) / (2 * h) - g[k][idx]) < 1e-6 * max(1, abs(g[k][idx])), (k, idx)


def test_adam_lowers_the_loss():
    n, hidden = 6, 16
    rng = np.random.default_rng(3)
    net = MADE(_params(n, hidden, rng), n, hidden)
    x = (rng.random((64, n)) < np.linspace(0.1, 0.9, n)).astype(int)
    m = {k: np.zeros_like(v) for k, v in net.p.items()}
    v = {k: np.zeros_like(v) for k, v in net.p.items()}
    first, _ = net.loss_and_grads(x)
    for t in range(1, 101):
        _, g = net.loss_and_grads(x)
        adam_step(net.p, g, m, v, t, 1e-2)
    last, _ = net.loss_and_grads(x)
    assert last < first - 0.5
