"""The oracle (CPU restatement) against the reference's own outputs (tests/golden/)."""
import os
import numpy as np
import pytest

from golden_cases import CASES, GOLDEN, WORKLOAD_CASES, Golden
from oracle.peps_oracle import DensePEPS, ObserverAccumulator, SweepChain, sweep_order
from oracle.rng import MT19937_64, uniform_int, uniform_real01


def test_mt19937_64_known_answer():
    # The C++ standard requires the 10000th output of a default-constructed mt19937_64
    # (seed 5489) to be 9981545732273789042 ([rand.predef]).
    g = MT19937_64(5489)
    for _ in range(9999):
        g()
    assert g() == 9981545732273789042


def test_distributions_edge_cases():
    g = MT19937_64(1)
    assert all(uniform_int(g, 0, 0) == 0 for _ in range(10))
    vals = [uniform_int(g, 0, 2) for _ in range(3000)]
    assert set(vals) == {0, 1, 2}
    r = [uniform_real01(g) for _ in range(1000)]
    assert min(r) >= 0.0 and max(r) < 1.0


def golden_charges(g):
    """(legs, phys, flux) of a golden case from the reference's edge segments."""
    from tnsp_gb300.lattice import site_charges
    legs = [[None] * g.L2 for _ in range(g.L1)]
    flux = [[0] * g.L2 for _ in range(g.L1)]
    phys = None
    for l1 in range(g.L1):
        for l2 in range(g.L2):
            meta = g.meta["sites"][f"{l1},{l2}"]
            legs[l1][l2], phys, flux[l1][l2] = site_charges([m["name"] for m in meta],
                                                            [[tuple(x) for x in m["segments"]] for m in meta])
    return legs, phys, flux


@pytest.mark.parametrize("charged", [False, True])
@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference(name, charged):
    g = Golden(name)
    peps = DensePEPS(g.dense_sites(), g.terms(), g.cut, golden_charges(g) if charged else None)
    order = [peps.terms[i][0] for i in sweep_order(peps)]
    assert order == [tuple(tuple(p) for p in ps) for ps in g.meta["sweep_order"]]
    acc = ObserverAccumulator(peps)
    z = g.z
    for ci, seed in enumerate(g.meta["chain_seeds"]):
        chain = SweepChain(peps, g.neel(), seed)
        for k in range(g.meta["n_therm"] + g.meta["n_samples"]):
            poss, conf = chain.sweep()
            # sampled configurations are bit-exact
            np.testing.assert_array_equal(conf, z["confs"][ci][k])
            assert abs(poss / z["possibility"][ci][k] - 1) < 1e-10
            if k >= g.meta["n_therm"]:
                j = k - g.meta["n_therm"]
                ws, eloc, holes = acc.add(poss, conf, chain.env)
                assert abs(ws / z["ws"][ci][j] - 1) < 1e-10
                assert abs(eloc - z["eloc"][ci][j]) < 1e-10
                for l1 in range(g.L1):
                    for l2 in range(g.L2):
                        ref = z[f"holes_{l1}_{l2}"][ci][j]
                        mine = np.zeros_like(ref)
                        mine[conf[l1, l2]] = holes[l1][l2]
                        assert np.abs(mine - ref).max() <= 1e-10 * np.abs(ref).max()
    e, err = acc.energy()
    assert abs(e - z["energy"][0]) < 1e-12
    assert abs(err - z["energy"][1]) < 1e-10
    grad = acc.gradient()
    for l1 in range(g.L1):
        for l2 in range(g.L2):
            ref = z[f"grad_{l1}_{l2}"]
            assert np.abs(grad[l1][l2] - ref).max() <= 1e-10 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("name", WORKLOAD_CASES)
def test_oracle_matches_reference_on_benchmark_lattices(name):
    """The oracle on the benchmark-size lattices (8x8 U(1) D=6 Dcut 36; 6x6 U(1) D=4 Dcut 16), where the
    truncation keeps Dcut of up to D*Dcut singular values over many sectors: configurations bit-exact,
    values to 1e-10 relative, the gradient on its allowed entries."""
    g = Golden(name)
    dense = g.dense_sites()
    peps = DensePEPS(dense, g.terms(), g.cut, golden_charges(g))
    acc = ObserverAccumulator(peps)
    z = g.z
    for ci, seed in enumerate(g.meta["chain_seeds"]):
        chain = SweepChain(peps, g.neel(), seed)
        for k in range(g.meta["n_therm"] + g.meta["n_samples"]):
            poss, conf = chain.sweep()
            np.testing.assert_array_equal(conf, z["confs"][ci][k])
            assert abs(poss / z["possibility"][ci][k] - 1) < 1e-10
            if k >= g.meta["n_therm"]:
                j = k - g.meta["n_therm"]
                ws, eloc, _ = acc.add(poss, conf, chain.env)
                assert abs(ws / z["ws"][ci][j] - 1) < 1e-10
                assert abs(eloc - z["eloc"][ci][j]) < 1e-10 * max(1.0, abs(z["eloc"][ci][j]))
    e, err = acc.energy()
    assert abs(e - z["energy"][0]) < 1e-12
    grad = acc.gradient()
    for l1 in range(g.L1):
        for l2 in range(g.L2):
            ref = g.gradient(l1, l2, dense)
            assert np.abs(grad[l1][l2] - ref).max() <= 1e-10 * max(1.0, np.abs(ref).max())


NATURAL_CASES = ["heis_no_3x3_D3_dc4", "heis_u1_4x4_D111_dc5"]


@pytest.mark.parametrize("name", NATURAL_CASES)
def test_oracle_natural_gradient_matches_reference(name):
    """Conjugate-gradient natural gradient of the oracle against the reference's own
    natural_gradient_by_conjugate_gradient (observer.py:576-675), fixed step count and error stop."""
    g = Golden(name)
    nat = np.load(os.path.join(GOLDEN, f"{name}_natgrad.npz"))
    peps = DensePEPS(g.dense_sites(), g.terms(), g.cut)
    acc = ObserverAccumulator(peps, natural=True)
    for seed in g.meta["chain_seeds"]:
        chain = SweepChain(peps, g.neel(), seed)
        for k in range(g.meta["n_therm"] + g.meta["n_samples"]):
            poss, conf = chain.sweep()
            if k >= g.meta["n_therm"]:
                acc.add(poss, conf, chain.env)
    for k, (steps, error) in enumerate(nat["runs"]):
        grad, _ = acc.natural_gradient(int(steps), float(error))
        scale = max(np.abs(nat[f"natgrad{k}_{l1}_{l2}"]).max() for l1 in range(g.L1) for l2 in range(g.L2))
        for l1 in range(g.L1):
            for l2 in range(g.L2):
                ref = nat[f"natgrad{k}_{l1}_{l2}"]
                assert np.abs(grad[l1][l2] - ref).max() <= 1e-8 * scale, (k, l1, l2)


def test_direct_sampling_matches_reference():
    """DirectSampling with exact cuts: the reference's sampled configurations (bit-exact) and
    possibilities, for alpha 1 and 0.5, from the enumeration oracle replaying the same draws."""
    from oracle.peps_oracle import DensePEPS, DirectSamplerExact
    from oracle.rng import MT19937_64
    g = Golden("heis_no_3x3_D3_dc4")
    z = np.load(os.path.join(GOLDEN, "heis_no_3x3_D3_dc4_direct.npz"))
    peps = DensePEPS(g.dense_sites(), g.terms(), int(z["cuts"][0]))
    for k, (seed, alpha, n) in enumerate(z["runs"]):
        sampler = DirectSamplerExact(peps, MT19937_64(int(seed)), alpha)
        for i in range(int(n)):
            p, conf = sampler()
            np.testing.assert_array_equal(conf, z[f"confs{k}"][i])
            assert p == pytest.approx(z[f"possibility{k}"][i], rel=1e-12)


def test_ergodic_energy_and_gradient_match_reference():
    """ErgodicSampling (every configuration, possibility 1, sampling.py:196-249) with the truncating cut
    of the golden case: the oracle's exact enumeration of E/site, its error bar and the gradient against
    the reference's, free of sampling noise."""
    import itertools
    g = Golden("heis_no_3x3_D3_dc4")
    z = np.load(os.path.join(GOLDEN, "heis_no_3x3_D3_dc4_ergodic.npz"))
    peps = DensePEPS(g.dense_sites(), g.terms(), int(z["cut"]))
    acc = ObserverAccumulator(peps)
    for idx in itertools.product(range(2), repeat=9):
        acc.add(1.0, np.array(idx).reshape(3, 3))  # the order of the sum does not matter
    assert acc.count == int(z["total_steps"])
    np.testing.assert_allclose(acc.energy(), z["energy"], rtol=1e-11)
    grad = acc.gradient()
    for l1 in range(3):
        for l2 in range(3):
            np.testing.assert_allclose(grad[l1][l2], z[f"grad_{l1}_{l2}"], rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("name", ["heis_no_3x3_D3_dc4_trunc", "heis_no_3x3_D3_dc4_trunc2"])
def test_direct_sampling_with_truncation_matches_reference(name):
    """DirectSampling with truncating single- and double-layer cuts, (4, 6) and (2, 4)
    (oracle/direct_oracle.py): the reference's samples, configurations bit-exact and possibilities to
    1e-12, alpha 1 and 0.5."""
    from oracle.direct_oracle import DirectSampler
    g = Golden("heis_no_3x3_D3_dc4")
    z = np.load(os.path.join(GOLDEN, f"{name}_direct.npz"))
    cuts = tuple(int(x) for x in z["cuts"])
    peps = DensePEPS(g.dense_sites(), g.terms(), cuts[0])
    for k, (seed, alpha, n) in enumerate(z["runs"]):
        sampler = DirectSampler(peps, MT19937_64(int(seed)), cuts[1], alpha)
        for i in range(int(n)):
            p, conf = sampler()
            np.testing.assert_array_equal(conf, z[f"confs{k}"][i])
            assert p == pytest.approx(z[f"possibility{k}"][i], rel=1e-12)


def test_pseudo_inverse_natural_gradient_meets_the_reference_conjugate_gradient():
    """The pseudo-inverse natural gradient (observer.py:697-907, by its single-process equation; the
    reference's ScaLAPACK path cannot run here) and the reference's own conjugate-gradient natural
    gradient solve the same least-squares problem (reweights 1, fewer samples than parameters: both give
    the least-norm solution); they agree to the conjugate gradient's stopping tolerance of 1e-3."""
    g = Golden("heis_no_3x3_D3_dc4")
    nat = np.load(os.path.join(GOLDEN, "heis_no_3x3_D3_dc4_natgrad.npz"))
    peps = DensePEPS(g.dense_sites(), g.terms(), g.cut)
    acc = ObserverAccumulator(peps, natural=True)
    for seed in g.meta["chain_seeds"]:
        chain = SweepChain(peps, g.neel(), seed)
        for k in range(g.meta["n_therm"] + g.meta["n_samples"]):
            poss, conf = chain.sweep()
            if k >= g.meta["n_therm"]:
                acc.add(poss, conf, chain.env)
    k = [i for i, (s, e) in enumerate(nat["runs"]) if e > 0][0]
    pinv = acc.natural_gradient_pinv(1e-8, 0.0)
    scale = max(np.abs(nat[f"natgrad{k}_{a}_{b}"]).max() for a in range(g.L1) for b in range(g.L2))
    err = max(np.abs(pinv[a][b] - nat[f"natgrad{k}_{a}_{b}"]).max() for a in range(g.L1) for b in range(g.L2))
    assert err <= 2e-3 * scale
