"""The reference's own gradient_descent (tetragono/tetragono/sampling_lattice/gradient.py:93-445), unchanged,
with its SweepSampling and Observer replaced by tnsp_gb300.reference_driver's adapters.

Here, without a GPU, the oracle (oracle/peps_oracle.py) stands in for the device sampler behind the drop-in
classes (it reproduces the reference's chains bit-exactly).  One gradient step of the adapted driver then
equals one step of the reference's own run: the same energy and the same updated tensors; a longer run
completes.  Needs the reference (TNSP_REFERENCE_ROOT and its CPU module from oracle/build_ref.sh): skipped
otherwise."""
import numpy as np
import pytest

from oracle.peps_oracle import DensePEPS, ObserverAccumulator, SweepChain


class OracleEngine:
    """The engine.Sampler interface the drop-in classes use, on the CPU oracle (test stand-in only)."""

    def __init__(self, lattice, cut, device=0, stream=None):
        self.lattice, self.cut = lattice, cut
        self.B = 0
        self.energy_restricted = False
        self.upload()

    def upload(self):
        lat = self.lattice
        self.peps = DensePEPS([[lat[a, b] for b in range(lat.L2)] for a in range(lat.L1)],
                              list(lat._hamiltonians.items()), self.cut, lat.charges)
        self._uploaded_version = lat.version

    def init_chains(self, configs, seeds, discard=0, precision=0):
        L1, L2 = self.lattice.L1, self.lattice.L2
        configs = np.broadcast_to(np.asarray(configs).reshape(-1, L1, L2), (len(seeds), L1, L2))
        self.chains = [SweepChain(self.peps, c, int(s), discard) for c, s in zip(configs, seeds)]
        self.B = len(seeds)
        self._poss = np.ones(self.B)
        self.reset_observer()

    def set_hopping(self, tables=None, allowed=None):
        if tables is not None or allowed is not None:
            raise NotImplementedError

    def restrict_energy(self, allowed=None):
        if allowed is not None:
            raise NotImplementedError

    def keep_holes(self, enable=True):
        pass

    def reset_observer(self):
        self.acc = ObserverAccumulator(self.peps, natural=True)
        self._rec = None

    def sweep(self, nsweeps=1, observe=False):
        for _ in range(nsweeps):
            rec = []
            for b, ch in enumerate(self.chains):
                poss, conf = ch.sweep()
                self._poss[b] = poss
                if observe:
                    ws, e, _ = self.acc.add(poss, conf, ch.env)
                    rec.append((e, np.log(abs(ws)), ws * ws / poss))
            if observe:
                self._rec = np.array(rec).T

    def read_chains(self):
        return np.array([ch.conf for ch in self.chains]), np.log(self._poss)

    def read_samples(self, nsweeps):
        return self._rec[0][None], self._rec[1][None], self._rec[2][None]

    def read_observer(self, with_gradient=True):
        a = self.acc
        scalars = np.array([a.count, a.total_weight, a.total_weight_square, a.total_log_ws, a.er, a.err, a.eerr,
                            float(sum(ch.accepts for ch in self.chains))])
        flat = lambda x: np.concatenate([t.ravel() for row in x for t in row])
        return scalars, flat(a.Delta), flat(a.EDelta)

    def holes_count(self):
        return len(self.acc.samples)

    def holes_gemv(self, x, transpose=False):
        H = np.array([r for _, _, r in self.acc.samples])
        return H.T @ x if transpose else H @ x

    def holes_gram(self):
        H = np.array([r for _, _, r in self.acc.samples])
        return H @ H.T

    def status(self):
        return 0


def _lattice(make_golden, seed):
    return make_golden.build_lattice("u1", 4, 4, (1, 1, 1), seed)


def test_reference_gradient_descent_runs_on_the_drop_in_sampler(monkeypatch):
    from test_checkpoint import _reference_modules
    TAT, tetragono = _reference_modules()  # skips without the reference
    import make_golden
    from tetragono.sampling_lattice import gradient
    from tnsp_gb300 import reference_driver, sampling
    monkeypatch.setattr(sampling, "Sampler", OracleEngine)
    neel = np.fromfunction(lambda a, b: (a + b) % 2, (4, 4)).astype(np.int64)[:, :, None]
    kwargs = dict(sampling_total_step=6, grad_total_step=1, grad_step_size=0.02, sampling_method="sweep",
                  configuration_cut_dimension=5)

    def run(driver):
        TAT.random.seed(2718)  # the driver's SeedDiffer draws the chain seed from the global engine
        state = _lattice(make_golden, 4321)
        out = list(driver(state, sampling_configurations=neel.copy(), **kwargs))
        return state, out

    ref_state, ref_out = run(gradient.gradient_descent)
    our_state, our_out = run(reference_driver.run_gradient_descent)
    start = _lattice(make_golden, 4321)
    moved = max(np.abs(np.array(ref_state[a, b].storage) - np.array(start[a, b].storage)).max()
                for a in range(4) for b in range(4))
    assert moved > 1e-4  # the step changed the tensors
    assert abs(our_out[0][0]["energy"][0] - ref_out[0][0]["energy"][0]) < 1e-12
    for l1 in range(4):
        for l2 in range(4):
            a, b = np.array(our_state[l1, l2].storage), np.array(ref_state[l1, l2].storage)
            assert np.abs(a - b).max() <= 1e-10 * np.abs(b).max()
    # several steps with the natural gradient run through the same interfaces
    TAT.random.seed(3)
    state = _lattice(make_golden, 4321)
    out = list(reference_driver.run_gradient_descent(state, sampling_configurations=neel.copy(), sampling_total_step=4,
                                                     grad_total_step=2, grad_step_size=0.02, sampling_method="sweep",
                                                     configuration_cut_dimension=5, use_natural_gradient=True,
                                                     conjugate_gradient_method_step=5))
    assert len(out) == 2 and all(np.isfinite(o[0]["energy"][0]) for o in out)
