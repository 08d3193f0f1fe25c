"""Learned proposal on the GPU: the hand-written network kernels against the CPU oracle, the sampling
distribution, and the trained proposal on a 4x4 lattice."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _net(n, hidden, seed, cap):
    from tnsp_gb300.proposal import AutoregressiveProposal
    return AutoregressiveProposal(n, hidden=hidden, seed=seed, batch_capacity=cap)


def test_network_kernels_match_oracle():
    from oracle.made_oracle import MADE, adam_step
    n, hidden = 10, 32
    net = _net(n, hidden, 5, 64)
    p0 = net.params()
    ref = MADE(net.unpack(p0), n, hidden)
    x = np.random.default_rng(7).integers(0, 2, (50, n))
    np.testing.assert_allclose(net.logq(x), ref.logq(x), rtol=0, atol=1e-3)
    loss_ref, g_ref = ref.loss_and_grads(x)
    g = net.unpack(net.gradient(x))
    for k in g_ref:
        scale = max(1e-12, np.abs(g_ref[k]).max())
        assert np.abs(g[k] - g_ref[k]).max() <= 2e-3 * scale, k
    # one Adam step (t = 1, lr = 1e-2): p - lr * g / (|g| + eps), compared where g is clearly nonzero
    loss = net.train_step(x, lr=1e-2)
    assert abs(loss - loss_ref) < 1e-3
    p1 = net.unpack(net.params())
    m = {k: np.zeros_like(v) for k, v in ref.p.items()}
    v = {k: np.zeros_like(v) for k, v in ref.p.items()}
    expect = {k: a.copy() for k, a in ref.p.items()}
    adam_step(expect, g_ref, m, v, 1, 1e-2)
    for k in expect:
        clear = np.abs(g_ref[k]) > 1e-2 * max(1e-12, np.abs(g_ref[k]).max())
        np.testing.assert_allclose(p1[k][clear], expect[k][clear], rtol=0, atol=1e-5, err_msg=k)
        untouched = g_ref[k] == 0
        np.testing.assert_array_equal(p1[k][untouched], net.unpack(p0)[k][untouched])


def test_samples_follow_the_model():
    n, hidden, B = 6, 16, 4096
    net = _net(n, hidden, 1, B)
    conf, lq = net.sample(B)
    np.testing.assert_allclose(lq, net.logq(conf), rtol=0, atol=1e-9)
    states = np.array([[(k >> i) & 1 for i in range(n)] for k in range(2**n)])
    p = np.exp(net.logq(states))
    assert abs(p.sum() - 1) < 1e-4
    idx = (conf * (1 << np.arange(n))).sum(axis=1)
    counts = np.bincount(idx, minlength=2**n)
    chi2 = ((counts - B * p)**2 / (B * p)).sum()
    assert chi2 < 63 + 6 * np.sqrt(2 * 63), chi2  # chi-square with 63 degrees of freedom, 6 sigma


def test_trained_proposal_on_a_4x4_lattice():
    """Trained on plain-sweep configurations, the network lowers its negative log-likelihood and is
    accepted more often than an untrained one as a Metropolis-Hastings independence proposal."""
    from tnsp_gb300.engine import Sampler
    from tnsp_gb300.lattice import neel, random_heisenberg
    from tnsp_gb300.proposal import independence_step
    lat = random_heisenberg(4, 4, 4, seed=20240601)
    B = 256
    s = Sampler(lat, 16)
    s.init_chains(neel(4, 4), np.arange(B, dtype=np.uint64) + np.uint64(11))
    s.sweep(10)
    data = []
    for _ in range(16):
        s.sweep(1)
        data.append(s.read_chains()[0].reshape(B, -1))
    data = np.concatenate(data)
    trained = _net(16, 64, 3, 512)
    untrained = _net(16, 64, 4, 512)
    history = trained.fit(data, epochs=15, batch=512, lr=3e-3)
    assert history[-1] < history[0] - 0.5, history
    rng = np.random.default_rng(0)
    acc_t, acc_u = [], []
    for _ in range(3):
        acc_u.append(independence_step(s, untrained, rng))
        s.sweep(1)
        acc_t.append(independence_step(s, trained, rng))
        s.sweep(1)
    print(f"NLL {history[0]:.3f} -> {history[-1]:.3f}; acceptance trained {np.mean(acc_t):.3f}, "
          f"untrained {np.mean(acc_u):.3f}")
    assert np.mean(acc_t) > np.mean(acc_u)
    assert s.status() == 0
