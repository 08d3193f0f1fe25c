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
        obs._observe_diagonal([c], [rw])
    obs.__exit__(None, None, None)
    result, whole = obs.result, obs.whole_result
    for k, (name, positions) in enumerate(zip(meta["names"], meta["positions"])):
        np.testing.assert_allclose(result[name][tuple(tuple(p) for p in positions)], z[f"result_{k}"], rtol=1e-12,
                                   atol=1e-14)
    for name in set(meta["names"]):
        np.testing.assert_allclose(whole[name], z[f"whole_{name}"], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(whole["energy"], np.array(z["energy"]) * 9, rtol=1e-10)  # total = 9 x per site


def test_off_diagonal_observers_are_refused():
    flip = {(0, 1): [((1, 0), 0.5)], (1, 0): [((0, 1), 0.5)]}
    with pytest.raises(NotImplementedError):
        Observer(_Owner(), observer_set={"flip": {((0, 0, 0), (2, 2, 0)): flip}})
