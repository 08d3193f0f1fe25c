"""The drop-in Observer's diagonal observer set (long-range Sz and SzSz) against the reference's own
``result`` / ``whole_result`` on the golden chains (tests/golden/heis_no_3x3_D3_dc4_observe.npz, made by
tests/golden/make_golden.py): the per-sample accumulation and the reference's expect/deviation formula,
fed with the golden samples through a stand-in engine (no GPU)."""
import json
import os

import numpy as np
import pytest

from golden_cases import GOLDEN

from tnsp_gb300.sampling import Observer


class _Owner:
    L1 = L2 = 3
    site_number = 9
    _active_observer = None


class _Engine:
    def __init__(self, scalars):
        self.scalars = scalars

    def keep_holes(self, enable=True):
        pass

    def reset_observer(self):
        pass

    def read_observer(self, with_gradient=True):
        return self.scalars.copy(), None, None


def _tables(z, meta):
    sets = {}
    for k, (name, positions) in enumerate(zip(meta["names"], meta["positions"])):
        table = {}
        for row in z[f"table_{k}"]:
            body = (len(row) - 1) // 2
            s_in = tuple(int(x) for x in row[:body])
            s_out = tuple(int(x) for x in row[body:2 * body])
            table.setdefault(s_in, []).append((s_out, float(row[-1])))
        sets.setdefault(name, {})[tuple(tuple(p) for p in positions)] = table
    return sets


def test_diagonal_observer_set_matches_reference():
    g = np.load(os.path.join(GOLDEN, "heis_no_3x3_D3_dc4.npz"))
    z = np.load(os.path.join(GOLDEN, "heis_no_3x3_D3_dc4_observe.npz"))
    meta = json.loads(str(z["meta"]))
    n_therm = g["confs"].shape[1] - g["ws"].shape[1]
    confs = g["confs"][:, n_therm:].reshape(-1, 3, 3)
    w = (g["ws"]**2 / g["possibility"][:, n_therm:]).reshape(-1)
    e = g["eloc"].reshape(-1)
    scalars = np.array([len(w), w.sum(), (w * w).sum(), 0.0, (e * w).sum(), (e * w * w).sum(), (e * e * w * w).sum(), 0])
    obs = Observer(_Owner(), observer_set=_tables(z, meta), enable_energy=True)
    obs.__enter__()
    obs._bind(_Engine(scalars))
    for c, rw in zip(confs, w):
        obs._observe_set([c], [rw])
    obs.__exit__(None, None, None)
    result, whole = obs.result, obs.whole_result
    for k, (name, positions) in enumerate(zip(meta["names"], meta["positions"])):
        np.testing.assert_allclose(result[name][tuple(tuple(p) for p in positions)], z[f"result_{k}"], rtol=1e-12,
                                   atol=1e-14)
    for name in set(meta["names"]):
        np.testing.assert_allclose(whole[name], z[f"whole_{name}"], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(whole["energy"], np.array(z["energy"]) * 9, rtol=1e-10)  # total = 9 x per site


class _AmplitudeEngine(_Engine):
    """A stand-in engine whose ``amplitude`` is the oracle's hole(()) (oracle/peps_oracle.py), as the
    device amplitude entry returns it (mantissa, exponent)."""

    def __init__(self, scalars, peps):
        super().__init__(scalars)
        self.peps = peps
        self.calls = 0

    def amplitude(self, configs):
        from oracle.peps_oracle import Environment
        self.calls += 1
        m = np.array([Environment(self.peps, c).amplitude() for c in np.asarray(configs)])
        return m, np.zeros(len(m), dtype=np.int32)


def _oracle_peps(name):
    from golden_cases import Golden
    from oracle.peps_oracle import DensePEPS
    g = Golden(name)
    return DensePEPS(g.dense_sites(), g.terms(), g.cut)


def test_off_diagonal_observer_set_matches_reference():
    """Off-diagonal long-range operators (Sx, SxSx, SS at distance 2) on the golden chains: the drop-in
    Observer's per-sample values from replaced configurations' amplitudes (here the oracle's, on the
    device the amplitude kernel's) against the reference's ConfigurationPool results
    (tests/golden/heis_no_3x3_D3_dc4_offdiag.npz)."""
    z = np.load(os.path.join(GOLDEN, "heis_no_3x3_D3_dc4_offdiag.npz"))
    meta = json.loads(str(z["meta"]))
    confs, w = z["confs"], z["weights"]
    scalars = np.array([len(w), w.sum(), (w * w).sum(), 0.0, 0.0, 0.0, 0.0, 0])
    engine = _AmplitudeEngine(scalars, _oracle_peps("heis_no_3x3_D3_dc4"))
    obs = Observer(_Owner(), observer_set=_tables(z, meta), enable_energy=True, cache_configuration=True)
    obs.__enter__()
    obs._bind(engine)
    obs._observe_set(confs[:7], w[:7])  # two sweeps' worth of samples, amplitudes batched per sweep
    obs._observe_set(confs[7:], w[7:])
    obs.__exit__(None, None, None)
    assert engine.calls == 4
    result, whole = obs.result, obs.whole_result
    for k, (name, positions) in enumerate(zip(meta["names"], meta["positions"])):
        np.testing.assert_allclose(result[name][tuple(tuple(p) for p in positions)], z[f"result_{k}"], rtol=1e-10,
                                   atol=1e-13)
    for name in set(meta["names"]):
        np.testing.assert_allclose(whole[name], z[f"whole_{name}"], rtol=1e-10, atol=1e-13)


def test_off_diagonal_observers_respect_the_restriction():
    """A restriction that forbids changing site (1, 1) (observer.py:364-367, asked for every element,
    the diagonal one included): Sx there vanishes, SS across it keeps only its diagonal SzSz part, and
    terms away from it keep the reference's values."""
    z = np.load(os.path.join(GOLDEN, "heis_no_3x3_D3_dc4_offdiag.npz"))
    meta = json.loads(str(z["meta"]))
    confs, w = z["confs"], z["weights"]
    scalars = np.array([len(w), w.sum(), (w * w).sum(), 0.0, 0.0, 0.0, 0.0, 0])
    engine = _AmplitudeEngine(scalars, _oracle_peps("heis_no_3x3_D3_dc4"))
    owner = _Owner()
    owner.P, owner.charges = 2, None

    def fixed_center(configuration, replacement):
        return all(configuration[p] == v for p, v in replacement.items() if p == (1, 1, 0))

    obs = Observer(owner, observer_set=_tables(z, meta), enable_energy=True, restrict_subspace=fixed_center)
    obs.__enter__()
    obs._engine = engine  # bound without the device-side energy restriction
    obs._observe_set(confs, w)
    obs.__exit__(None, None, None)
    result = obs.result
    assert result["Sx"][((1, 1, 0),)] == (0.0, 0.0)
    szsz = (0.5 - confs[:, 0, 0]) * (0.5 - confs[:, 1, 1])
    np.testing.assert_allclose(result["SS"][((0, 0, 0), (1, 1, 0))][0], (szsz * w).sum() / w.sum(), rtol=1e-12)
    for k, (name, positions) in enumerate(zip(meta["names"], meta["positions"])):
        positions = tuple(tuple(p) for p in positions)
        if (1, 1, 0) not in positions:
            np.testing.assert_allclose(result[name][positions], z[f"result_{k}"], rtol=1e-10, atol=1e-13)
