"""GPU sampler (through the C ABI) against the reference's golden vectors and the oracle."""
import numpy as np
import pytest

from golden_cases import CASES, Golden

pytestmark = pytest.mark.gpu


def make_lattice(g, charged=False):
    """Lattice of a golden case; ``charged`` declares the reference's block structure so the device
    factorises per charge sector."""
    from tnsp_gb300.lattice import SamplingLattice, site_charges
    dense = g.dense_sites()
    charges = None
    if charged:
        legs = [[None] * g.L2 for _ in range(g.L1)]
        flux = [[0] * g.L2 for _ in range(g.L1)]
        phys = None
        for l1 in range(g.L1):
            for l2 in range(g.L2):
                meta = g.meta["sites"][f"{l1},{l2}"]
                legs[l1][l2], phys, flux[l1][l2] = site_charges([m["name"] for m in meta],
                                                                [[tuple(x) for x in m["segments"]] for m in meta])
        charges = (legs, phys, flux)
    return SamplingLattice(g.L1, g.L2, dense[0][0].shape[0], dense, {pos: t for pos, t in g.terms()}, charges)


@pytest.fixture(scope="module")
def engine_mod():
    from tnsp_gb300 import engine
    return engine


@pytest.mark.parametrize("charged", [False, True])
@pytest.mark.parametrize("name", CASES)
def test_sweeps_and_observer_match_reference(name, charged, engine_mod):
    g = Golden(name)
    lat = make_lattice(g, charged)
    z = g.z
    seeds = np.array(g.meta["chain_seeds"], dtype=np.uint64)
    B = len(seeds)
    s = engine_mod.Sampler(lat, g.cut)
    s.init_chains(g.neel(), seeds)
    nt, ns = g.meta["n_therm"], g.meta["n_samples"]
    for k in range(nt):
        s.sweep(1)
        conf, logp = s.read_chains()
        for b in range(B):
            np.testing.assert_array_equal(conf[b], z["confs"][b][k], err_msg=f"chain {b} sweep {k}")
            assert abs(logp[b] - np.log(z["possibility"][b][k])) < 1e-10
    s.reset_observer()
    elocs = np.zeros((ns, B))
    for k in range(ns):
        s.sweep(1, observe=True)
        conf, logp = s.read_chains()
        e, logws, rw = s.read_samples(1)
        elocs[k] = e[0]
        for b in range(B):
            np.testing.assert_array_equal(conf[b], z["confs"][b][nt + k], err_msg=f"chain {b} sample {k}")
            assert abs(logp[b] - np.log(z["possibility"][b][nt + k])) < 1e-10
            assert abs(logws[0][b] - np.log(abs(z["ws"][b][k]))) < 1e-10
            assert abs(e[0][b] - z["eloc"][b][k]) < 1e-10
    scalars, delta, edelta = s.read_observer()
    assert scalars[0] == B * ns
    energy, err = engine_mod.estimators(scalars, lat.site_number)
    assert abs(energy - z["energy"][0]) < 1e-12
    assert abs(err - z["energy"][1]) < 1e-10
    grad = lat.unflatten(engine_mod.gradient_from(scalars, delta, edelta))
    for l1 in range(g.L1):
        for l2 in range(g.L2):
            ref = z[f"grad_{l1}_{l2}"]
            assert np.abs(grad[l1][l2] - ref).max() <= 1e-10 * max(1.0, np.abs(ref).max()), (l1, l2)
    assert s.status() == 0


@pytest.mark.parametrize("name", CASES[:2])
def test_amplitude_entry(name, engine_mod):
    g = Golden(name)
    lat = make_lattice(g)
    s = engine_mod.Sampler(lat, g.cut)
    confs = g.z["confs"][0][g.meta["n_therm"]:]
    m, e = s.amplitude(confs)
    ws = m * np.exp2(e.astype(np.float64))
    np.testing.assert_allclose(ws, g.z["ws"][0], rtol=1e-10, atol=0)


@pytest.mark.parametrize("charged", [False, True])
def test_fp32_mode_close_to_fp64(charged, engine_mod):
    """Mixed mode: the same chains in float32 arithmetic; amplitudes and E_loc within 1e-3 relative."""
    g = Golden("heis_u1_4x4_D222_dc8")
    lat = make_lattice(g, charged)
    confs = g.z["confs"][0][g.meta["n_therm"]:]
    s64 = engine_mod.Sampler(lat, g.cut)
    m64, e64 = s64.amplitude(confs)
    s32 = engine_mod.Sampler(lat, g.cut)
    s32.init_chains(g.neel(), np.array([1], dtype=np.uint64), precision=engine_mod.TNSP_FP32)
    m32, e32 = s32.amplitude(confs)
    a64 = m64 * np.exp2(e64.astype(float))
    a32 = m32 * np.exp2(e32.astype(float))
    np.testing.assert_allclose(a32, a64, rtol=1e-3)
