"""Learned proposal: an autoregressive network trained on sweep configurations, used as a
Metropolis-Hastings independence proposal with exact PEPS amplitudes.

``AutoregressiveProposal`` owns the device network of ``tnsp_made_*`` (include/tnsp_gb300.h: masked
MLP, bfloat16 weights, float32 accumulation, hand-written training and sampling kernels).
``independence_step`` moves every chain of a ``Sampler`` once: x' ~ q, accepted with probability
min(1, |psi(x')|^2 q(x) / (|psi(x)|^2 q(x'))), psi from the sampler's own amplitude kernel; the chain
stays a valid Markov chain for |psi|^2 whatever q is, so the plain estimator judges its quality.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import ptr

_LN2 = 0.6931471805599453


class ProposalError(RuntimeError):
    pass


class AutoregressiveProposal:

    def __init__(self, n_sites, hidden=256, seed=0, batch_capacity=4096, device=0):
        self.lib = _lib.load()
        self.n, self.hidden, self.capacity = n_sites, hidden, batch_capacity
        self.h = ctypes.c_void_p()
        code = self.lib.tnsp_made_create(ctypes.byref(self.h), device, n_sites, hidden, seed, batch_capacity)
        self._check(code, "tnsp_made_create")
        self.n_params = hidden * n_sites + hidden + hidden * hidden + hidden + n_sites * hidden + n_sites

    def _check(self, code, what):
        if code != 0:
            msg = self.lib.tnsp_made_error(self.h).decode() if self.h else ""
            raise ProposalError(f"{what} failed ({code}): {msg}")

    def close(self):
        if self.h:
            self.lib.tnsp_made_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self):
        """float32 parameters W1 [hidden][n], b1, W2 [hidden][hidden], b2, W3 [n][hidden], b3."""
        p = np.zeros(self.n_params, dtype=np.float32)
        self._check(self.lib.tnsp_made_params(self.h, ptr(p, ctypes.c_float), 0), "tnsp_made_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != self.n_params:
            raise ValueError("parameter count mismatch")
        self._check(self.lib.tnsp_made_params(self.h, ptr(p, ctypes.c_float), 1), "tnsp_made_params")

    def unpack(self, p):
        """The flat parameter vector as a dict of arrays (W1, b1, W2, b2, W3, b3)."""
        n, H = self.n, self.hidden
        out, o = {}, 0
        for k, shape in (("W1", (H, n)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (n, H)), ("b3", (n,))):
            size = int(np.prod(shape))
            out[k] = p[o:o + size].reshape(shape)
            o += size
        return out

    def _configs(self, configs):
        c = np.ascontiguousarray(np.asarray(configs).reshape(-1, self.n), dtype=np.int32)
        if c.shape[0] > self.capacity:
            raise ValueError("more configurations than the batch capacity")
        return c

    def train_step(self, configs, lr=1e-3):
        """One Adam step on the mean negative log-likelihood of the batch; returns that mean (before
        the step)."""
        c = self._configs(configs)
        loss = ctypes.c_double()
        self._check(self.lib.tnsp_made_train(self.h, ptr(c, ctypes.c_int32), c.shape[0], lr, ctypes.byref(loss)),
                    "tnsp_made_train")
        return loss.value

    def fit(self, configs, epochs=20, batch=512, lr=1e-3, seed=0):
        """Maximum-likelihood training on configurations (e.g. of the plain sweep); returns the mean
        loss of every epoch."""
        data = np.asarray(configs).reshape(-1, self.n)
        rng = np.random.default_rng(seed)
        batch = min(batch, self.capacity)
        history = []
        for _ in range(epochs):
            order = rng.permutation(data.shape[0])
            losses = [self.train_step(data[order[k:k + batch]], lr) for k in range(0, data.shape[0], batch)]
            history.append(float(np.mean(losses)))
        return history

    def gradient(self, configs):
        c = self._configs(configs)
        g = np.zeros(self.n_params, dtype=np.float32)
        self._check(self.lib.tnsp_made_gradient(self.h, ptr(c, ctypes.c_int32), c.shape[0], ptr(g, ctypes.c_float)),
                    "tnsp_made_gradient")
        return g

    def logq(self, configs):
        c = self._configs(configs)
        out = np.zeros(c.shape[0])
        self._check(self.lib.tnsp_made_logq(self.h, ptr(c, ctypes.c_int32), c.shape[0], ptr(out, ctypes.c_double)),
                    "tnsp_made_logq")
        return out

    def sample(self, B):
        """B independent configurations (0/1 per site) and their log q."""
        c = np.zeros((B, self.n), dtype=np.int32)
        lq = np.zeros(B)
        self._check(self.lib.tnsp_made_sample(self.h, B, ptr(c, ctypes.c_int32), ptr(lq, ctypes.c_double)),
                    "tnsp_made_sample")
        return c, lq


def _log_abs_psi(m, e):
    with np.errstate(divide="ignore"):
        return np.log(np.abs(m)) + e.astype(np.float64) * _LN2


def independence_step(sampler, proposal, rng, conserve_sum=True):
    """One Metropolis-Hastings independence move of every chain of ``sampler``; returns the
    acceptance rate.  Accepted chains continue from the proposed configuration.

    With ``conserve_sum`` a proposal whose sum of site indices (2 S^z for spins) differs from the
    chain's is rejected: the target stays |psi|^2 on the sector the local moves explore (for U(1)
    lattices the amplitude outside it is zero anyway)."""
    conf, _ = sampler.read_chains()
    B = conf.shape[0]
    prop, lq_prop = proposal.sample(B)
    prop = prop.reshape(conf.shape)
    lq_cur = proposal.logq(conf.reshape(B, -1))
    lp_cur = _log_abs_psi(*sampler.amplitude(conf))
    lp_prop = _log_abs_psi(*sampler.amplitude(prop))
    with np.errstate(invalid="ignore"):
        log_ratio = 2.0 * (lp_prop - lp_cur) + lq_cur - lq_prop
    log_ratio = np.nan_to_num(log_ratio, nan=-np.inf)
    if conserve_sum:
        same = prop.reshape(B, -1).sum(axis=1) == conf.reshape(B, -1).sum(axis=1)
        log_ratio = np.where(same, log_ratio, -np.inf)
    accept = np.log(rng.random(B)) < log_ratio
    sampler.write_chains(np.where(accept[:, None, None], prop, conf))
    return float(accept.mean())
