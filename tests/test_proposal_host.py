"""Host logic of the learned proposal's Metropolis-Hastings move (no device): stand-in sampler and
proposal over all configurations of a 2x2 lattice with known amplitudes."""
import itertools

import numpy as np

from tnsp_gb300.proposal import independence_step

STATES = np.array(list(itertools.product([0, 1], repeat=4)))


class FakeSampler:
    """Chains over 2x2 configurations with amplitude psi(x) = mantissa * 2^exponent."""

    def __init__(self, psi, conf):
        self.psi = psi
        self.conf = np.array(conf, dtype=np.int32)

    def _index(self, c):
        return (np.asarray(c).reshape(len(c), -1) * (1 << np.arange(3, -1, -1))).sum(axis=1)

    def read_chains(self):
        return self.conf.copy(), np.zeros(len(self.conf))

    def amplitude(self, configs):
        v = self.psi[self._index(configs)]
        m, e = np.frexp(v)
        return m, e.astype(np.int32)

    def write_chains(self, configs):
        self.conf = np.array(configs, dtype=np.int32).reshape(self.conf.shape)


class FakeProposal:
    """Independent draws from a fixed distribution q over the 16 configurations."""

    def __init__(self, q, rng):
        self.q = q / q.sum()
        self.rng = rng

    def sample(self, B):
        idx = self.rng.choice(len(self.q), size=B, p=self.q)
        return STATES[idx].astype(np.int32), np.log(self.q[idx])

    def logq(self, configs):
        idx = (np.asarray(configs).reshape(len(configs), -1) * (1 << np.arange(3, -1, -1))).sum(axis=1)
        return np.log(self.q[idx])


def test_chain_converges_to_psi_squared_on_its_sector():
    rng = np.random.default_rng(0)
    psi = rng.normal(size=16) * 3.0
    start = np.array([[[0, 1], [1, 0]]] * 2000)  # two sites up: the chains' sector
    s = FakeSampler(psi, start)
    prop = FakeProposal(rng.random(16) + 0.2, rng)  # q unrelated to psi, covering every configuration
    for _ in range(60):
        independence_step(s, prop, rng)
    conf, _ = s.read_chains()
    assert (conf.reshape(len(conf), -1).sum(axis=1) == 2).all()  # never left the sector
    sector = STATES.sum(axis=1) == 2
    target = np.where(sector, psi**2, 0.0)
    target /= target.sum()
    idx = s._index(conf)
    freq = np.bincount(idx, minlength=16) / len(idx)
    assert 0.5 * np.abs(freq - target).sum() < 0.05


def test_proposal_proportional_to_psi_squared_is_always_accepted():
    rng = np.random.default_rng(1)
    psi = rng.normal(size=16)
    sector = STATES.sum(axis=1) == 2
    q = np.where(sector, psi**2, 0.0)
    s = FakeSampler(psi, np.array([[[1, 1], [0, 0]]] * 500))
    assert independence_step(s, FakeProposal(q, rng), rng) == 1.0


def test_zero_amplitude_proposals_are_rejected():
    rng = np.random.default_rng(2)
    psi = np.where(STATES.sum(axis=1) == 2, 1.0, 0.0) * (1 + np.arange(16))
    psi[3] = 0.0  # a configuration of the sector with zero amplitude
    q = np.zeros(16)
    q[3] = 1.0
    s = FakeSampler(psi, np.array([[[0, 1], [0, 1]]] * 100))
    assert independence_step(s, FakeProposal(q + 1e-300, rng), rng) == 0.0
