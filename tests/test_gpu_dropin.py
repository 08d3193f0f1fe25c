"""The reference's gradient_descent sampling loop, run unchanged against the drop-in classes."""
import numpy as np
import pytest

from golden_cases import Golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["heis_no_3x3_D3_dc4", "heis_u1_4x4_D111_dc5"])
def test_driver_loop_matches_reference(name):
    from test_gpu_parity import make_lattice
    from tnsp_gb300.sampling import Observer, SweepSampling
    g = Golden(name)
    state = make_lattice(g, charged=True)
    seeds = g.meta["chain_seeds"]
    chains = len(seeds)
    nt, ns = g.meta["n_therm"], g.meta["n_samples"]
    observer = Observer(state, enable_energy=True, enable_gradient=True)
    # thermalisation (gm_conf_eq): sweeps without an observer
    sampling = SweepSampling(state, g.cut, None, None, chains=chains, seeds=seeds)
    sampling.configuration.import_configuration(g.neel()[:, :, None])
    for k in range(nt * chains):
        possibility, configuration = sampling()
        ci = k % chains
        np.testing.assert_array_equal(configuration.export_configuration()[:, :, 0], g.z["confs"][ci][k // chains])
    # gradient.py:331-358
    with observer:
        for k in range(ns * chains):
            possibility, configuration = sampling()
            observer(possibility, configuration)
            ci = k % chains
            assert abs(possibility / g.z["possibility"][ci][nt + k // chains] - 1) < 1e-10
    energy, error = observer.energy
    assert abs(energy - g.z["energy"][0]) < 1e-12
    grad = observer.gradient
    for l1 in range(g.L1):
        for l2 in range(g.L2):
            ref = g.z[f"grad_{l1}_{l2}"]
            assert np.abs(grad[l1][l2] - ref).max() <= 1e-10 * max(1.0, np.abs(ref).max())
    # apply_gradient + normalize_lattice as gradient.py:399-433 does
    norm0 = state.lattice_dot()
    state.apply_gradient(grad, 0.01)
    observer.normalize_lattice()
    assert state.lattice_dot() != norm0


@pytest.mark.parametrize("name", ["heis_no_3x3_D3_dc4", "heis_u1_4x4_D111_dc5"])
def test_natural_gradient_matches_reference(name):
    """Observer(enable_natural_gradient=True) + natural_gradient_by_conjugate_gradient(step, error)
    against the reference's own outputs (fixed step count, and error-based stop)."""
    import os
    from golden_cases import GOLDEN
    from test_gpu_parity import make_lattice
    from tnsp_gb300.sampling import Observer, SweepSampling
    g = Golden(name)
    nat = np.load(os.path.join(GOLDEN, f"{name}_natgrad.npz"))
    state = make_lattice(g, charged=True)
    seeds = g.meta["chain_seeds"]
    chains = len(seeds)
    nt, ns = g.meta["n_therm"], g.meta["n_samples"]
    sampling = SweepSampling(state, g.cut, None, None, chains=chains, seeds=seeds)
    sampling.configuration.import_configuration(g.neel()[:, :, None])
    for _ in range(nt * chains):
        sampling()
    observer = Observer(state, enable_energy=True, enable_gradient=True, enable_natural_gradient=True)
    with observer:
        for _ in range(ns * chains):
            possibility, configuration = sampling()
            observer(possibility, configuration)
    for k, (steps, error) in enumerate(nat["runs"]):
        grad = observer.natural_gradient_by_conjugate_gradient(int(steps), float(error))
        scale = max(np.abs(nat[f"natgrad{k}_{l1}_{l2}"]).max() for l1 in range(g.L1) for l2 in range(g.L2))
        for l1 in range(g.L1):
            for l2 in range(g.L2):
                ref = nat[f"natgrad{k}_{l1}_{l2}"]
                assert np.abs(grad[l1][l2] - ref).max() <= 1e-8 * scale, (k, l1, l2)


def center_fixed(configuration, replacement):
    """The restricted subspace of the golden case: site (1, 1) keeps its value (EdgePoint index), the
    same callable the reference ran (tests/golden/make_golden.py)."""
    return replacement.get((1, 1, 0), configuration[1, 1, 0])[1] == configuration[1, 1, 0][1]


@pytest.mark.parametrize("precision", ["fp64", "dd"])
def test_restricted_subspace_and_hopping_hamiltonians_match_reference(precision):
    """SweepSampling(state, cut, restrict_subspace, hopping_hamiltonians) and Observer(restrict_subspace=...)
    as the reference runs them (sampling.py:81-91, 117-143; observer.py:364-367): spin-flip-only hopping
    tables and a restriction that keeps site (1, 1) fixed; configurations bit-exact after every sweep,
    possibilities, energy and gradient within the golden tolerances."""
    import os
    from golden_cases import GOLDEN
    from test_gpu_parity import TOL, make_lattice
    from tnsp_gb300.sampling import Observer, SweepSampling
    tol = TOL[precision]
    z = np.load(os.path.join(GOLDEN, "heis_no_3x3_D3_dc4_restricted.npz"))
    g = Golden("heis_no_3x3_D3_dc4")
    state = make_lattice(g)
    hopping = {}
    for positions, table in state._hamiltonians.items():
        hopping[positions] = {s: [(o, v) for o, v in outs if tuple(o) != tuple(s)] for s, outs in table.items()}
        hopping[positions] = {s: outs for s, outs in hopping[positions].items() if outs}
    seeds = [11, 12]
    chains = len(seeds)
    nt, ns = 3, 5
    sampling = SweepSampling(state, g.cut, center_fixed, hopping, chains=chains, seeds=seeds, precision=precision)
    sampling.configuration.import_configuration(g.neel()[:, :, None])
    for k in range(nt * chains):
        possibility, configuration = sampling()
        ci = k % chains
        np.testing.assert_array_equal(configuration.export_configuration()[:, :, 0], z["confs"][ci][k // chains])
    observer = Observer(state, enable_energy=True, enable_gradient=True, restrict_subspace=center_fixed)
    with observer:
        for k in range(ns * chains):
            possibility, configuration = sampling()
            observer(possibility, configuration)
            ci = k % chains
            np.testing.assert_array_equal(configuration.export_configuration()[:, :, 0], z["confs"][ci][nt + k // chains])
            assert abs(possibility / z["possibility"][ci][nt + k // chains] - 1) < tol["val"]
    energy, _ = observer.energy
    assert abs(energy - z["energy"][0]) < tol["energy"]
    grad = observer.gradient
    for l1 in range(g.L1):
        for l2 in range(g.L2):
            ref = z[f"grad_{l1}_{l2}"]
            assert np.abs(grad[l1][l2] - ref).max() <= tol["grad"] * max(1.0, np.abs(ref).max())


def test_hole_row_gram_product_and_pseudo_inverse():
    """tnsp_holes_gram (H H^T over the device-kept hole rows, one launch) equals the products built from
    tnsp_holes_gemv, and the pseudo-inverse natural gradient built on it equals the single-process equation
    (observer.py:902-907) evaluated from the rows read back."""
    from test_gpu_parity import make_lattice
    from tnsp_gb300.sampling import Observer, SweepSampling
    g = Golden("heis_u1_4x4_D111_dc5")
    state = make_lattice(g, charged=True)
    seeds = g.meta["chain_seeds"]
    sampling = SweepSampling(state, g.cut, None, None, chains=len(seeds), seeds=seeds)
    sampling.configuration.import_configuration(g.neel()[:, :, None])
    for _ in range(3 * len(seeds)):
        sampling()
    observer = Observer(state, enable_energy=True, enable_gradient=True, enable_natural_gradient=True)
    with observer:
        for _ in range(5 * len(seeds)):
            possibility, configuration = sampling()
            observer(possibility, configuration)
    eng = observer._engine
    n = eng.holes_count()
    H = np.stack([eng.holes_gemv(np.eye(n)[j], transpose=True) for j in range(n)])
    G = eng.holes_gram()
    np.testing.assert_allclose(G, H @ H.T, rtol=1e-12, atol=1e-12 * np.abs(H @ H.T).max())
    r_pinv, a_pinv = 1e-6, 1e-9
    x = np.concatenate([a.ravel() for row in observer.natural_gradient_by_direct_pseudo_inverse(r_pinv, a_pinv)
                        for a in row])
    scal = observer._read()
    delta = np.asarray(observer._delta) / scal[1]
    D = H - delta
    E = np.asarray(observer._samples_e) - scal[4] / scal[1]
    L, U = np.linalg.eigh(D @ D.T)
    num = r_pinv * L.max() + a_pinv
    Linv = np.array([0.0 if l <= 0 else 1.0 / (l * (1 + (num / l)**6)) for l in L])
    want = 2 * D.T @ (U @ (Linv * (U.T @ E)))
    np.testing.assert_allclose(x, want, rtol=0, atol=1e-8 * np.abs(want).max())


def test_off_diagonal_observer_set_matches_reference():
    """Long-range operators with off-diagonal elements (Sx, SxSx and SS at distance 2) observed in the
    driver loop: the replaced configurations' amplitudes come from the device amplitude entry, against
    the reference's ConfigurationPool results on the same chains
    (tests/golden/heis_no_3x3_D3_dc4_offdiag.npz)."""
    import json
    import os
    from golden_cases import GOLDEN
    from test_gpu_parity import make_lattice
    from test_observer_set import _tables
    from tnsp_gb300.sampling import Observer, SweepSampling
    g = Golden("heis_no_3x3_D3_dc4")
    z = np.load(os.path.join(GOLDEN, "heis_no_3x3_D3_dc4_offdiag.npz"))
    meta = json.loads(str(z["meta"]))
    state = make_lattice(g, charged=True)
    seeds = g.meta["chain_seeds"]
    nt, ns = g.meta["n_therm"], g.meta["n_samples"]
    sampling = SweepSampling(state, g.cut, None, None, chains=len(seeds), seeds=seeds)
    sampling.configuration.import_configuration(g.neel()[:, :, None])
    for _ in range(nt * len(seeds)):
        sampling()
    observer = Observer(state, observer_set=_tables(z, meta), enable_energy=True, cache_configuration=True)
    with observer:
        for _ in range(ns * len(seeds)):
            observer(*sampling())
    result, whole = observer.result, observer.whole_result
    for k, (name, positions) in enumerate(zip(meta["names"], meta["positions"])):
        np.testing.assert_allclose(result[name][tuple(tuple(p) for p in positions)], z[f"result_{k}"], rtol=1e-10,
                                   atol=1e-13)
    for name in set(meta["names"]):
        np.testing.assert_allclose(whole[name], z[f"whole_{name}"], rtol=1e-10, atol=1e-13)
    np.testing.assert_allclose(observer.energy[0], z["energy"][0], rtol=1e-10)
