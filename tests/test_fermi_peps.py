"""Fermionic (spinless t-V) amplitudes and local energies in the oracle against the reference's own
outputs (tests/golden/tv_*.npz, made by tests/golden/make_fermi_golden.py): the exact graded
contraction, and the same lattice evaluated as a bosonic network (per-site sign tables, a prefix
parity on one leg, a configuration sign) through the dense boundary-MPS oracle, with the
truncation active."""
import json
import os

import numpy as np
import pytest

from oracle import fermi_peps as fp
from oracle.fermi_tensor import FermiTensor

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    z = np.load(os.path.join(GOLDEN, f"tv_{name}.npz"))
    meta = json.loads(bytes(z["meta"]).decode())

    def mk(desc, st):
        return FermiTensor(desc["names"], [([tuple(x) for x in segs], a) for segs, a in desc["edges"]]).set_storage(st)

    sites = [[mk(meta["sites"][f"{a},{b}"], z[f"site_{a}_{b}"]) for b in range(meta["L2"])] for a in range(meta["L1"])]
    terms = [([tuple(p) for p in t["positions"]], mk(t["tensor"], z[f"term_{k}"])) for k, t in enumerate(meta["terms"])]
    return z, meta, sites, terms


def test_exact_graded_contraction_matches_reference():
    """3x3, cut 16: the reference's boundary MPS is exact, so its amplitude (sign included, in its own
    leg order) and E_loc equal the exact graded contraction."""
    z, meta, sites, terms = _load("3x3_D1_T4_dc16")
    for i, conf in enumerate(z["confs"]):
        ws = fp.amplitude(sites, conf)
        assert fp.value(ws, meta["ws_names"][i]) == pytest.approx(z["ws"][i], rel=1e-12, abs=0)
        assert fp.local_energy(sites, terms, conf) == pytest.approx(z["eloc"][i], rel=1e-12, abs=1e-12)


@pytest.mark.parametrize("name", ["3x3_D1_T4_dc16", "4x4_D2_T8_dc2", "3x4_D2_T5_dc3", "4x4_D1odd_T8_dc3"])
def test_bosonized_boundary_mps_matches_reference(name):
    """The bosonized lattice through the dense oracle reproduces the reference's amplitudes and E_loc,
    including with a cut of 2 where truncation changes the amplitudes by percents."""
    z, meta, sites, terms = _load(name)
    lat = fp.BosonizedLattice(sites, meta["cut"])
    for i, conf in enumerate(z["confs"]):
        envs = lat.environments(conf)
        assert fp.value(lat.amplitude(envs), meta["ws_names"][i]) == pytest.approx(z["ws"][i], rel=1e-12, abs=0)
        assert lat.local_energy(terms, conf) == pytest.approx(z["eloc"][i], rel=1e-12, abs=1e-12)


@pytest.mark.parametrize("name", ["4x4_D2_T8_dc2", "3x4_D2_T5_dc3", "4x4_D1odd_T8_dc3"])
def test_truncation_is_active_in_the_truncated_cases(name):
    z, meta, sites, terms = _load(name)
    rel = [abs(fp.value(fp.amplitude(sites, c), meta["ws_names"][i]) / z["ws"][i] - 1) for i, c in enumerate(z["confs"])]
    assert max(rel) > 1e-4   # truncation moves the amplitudes by far more than the 1e-12 parity tolerance


def test_column_family_is_exact_without_truncation():
    """The column-major sign rule: the column-strip amplitude equals the exact one on the 3x3 case."""
    z, meta, sites, terms = _load("3x3_D1_T4_dc16")
    lat = fp.BosonizedLattice(sites, meta["cut"])
    T = lat.T_symmetry
    for i, conf in enumerate(z["confs"]):
        envs = lat.environments(conf)
        E, F = envs[fp.COL].col_envs(0)
        v = float(F[0].reshape(-1)[0]) * fp.configuration_sign(conf, lat.p_T, fp.COL)
        v *= fp.order_sign(conf, fp.canonical_names(3, 3, fp.COL), meta["ws_names"][i], T)
        assert v == pytest.approx(z["ws"][i], rel=1e-12, abs=0)


def test_projection_is_the_stored_slice_times_minus_one_to_the_occupation():
    _, _, sites, _ = _load("3x3_D1_T4_dc16")
    for a in range(3):
        for b in range(3):
            s = sites[a][b]
            legs = [x for x in ["T", "U", "D", "L", "R"] if x in s.names]
            raw = s.transpose(["P0"] + legs).data
            for n in (0, 1):
                want = ((-1.0)**n) * raw[n].reshape(fp.projected_dense(s, a, b, n).shape)
                assert np.array_equal(fp.projected_dense(s, a, b, n), want)


def test_closed_form_term_sign_equals_the_graded_pairing():
    _, _, sites, terms = _load("4x4_D2_T8_dc2")
    T = sites[0][0].edge_by_name("T")[0][0][0]
    rng = np.random.default_rng(3)
    checked = 0
    for _ in range(100):
        conf = np.zeros(16, int)
        conf[rng.choice(16, size=-T, replace=False)] = 1
        conf = conf.reshape(4, 4)
        ws = fp.amplitude_tensor(conf, 1.0, T, fp.ROW)
        for positions, H in terms:
            table = fp.element_table(H)
            here = tuple(fp.point(conf[a][b]) for a, b, _ in positions)
            for out, elem in table.get(here, {}).items():
                new = [sym for sym, _ in out]
                after = conf.copy()
                for (a, b, _), s in zip(positions, new):
                    after[a, b] = s
                wss = fp.amplitude_tensor(after, 1.0, T, fp.ROW)
                pn = [f"P_{a}_{b}_0" for a, b, _ in positions]
                v = ws.contract(elem, {(pn[i], f"I{i}") for i in range(2)})
                v = v.edge_rename({f"O{i}": pn[i] for i in range(2)})
                pairing = float(v.contract(wss.conjugate(), {(n, n) for n in ws.names}).scalar())
                h = float(elem.data.reshape(-1)[0])
                assert pairing == h * fp.hop_sign(conf, [p[:2] for p in positions], new)
                checked += 1
    assert checked > 1000


def test_exact_graded_holes_match_reference():
    z, meta, sites, _ = _load("3x3_D1_T4_dc16")

    def mk(desc, st):
        return FermiTensor(desc["names"], [([tuple(x) for x in segs], a) for segs, a in desc["edges"]]).set_storage(st)

    for i, conf in enumerate(z["confs"][:4]):
        hs = fp.holes(sites, conf)
        for a in range(3):
            for b in range(3):
                ref = mk(meta["holes"][f"{a},{b}"], z[f"holes_{a}_{b}"][i])
                mine = hs[a][b].transpose(ref.names)
                assert mine.edges == ref.edges
                assert np.abs(mine.data - ref.data).max() <= 1e-12 * np.abs(ref.data).max()


@pytest.mark.parametrize("name", ["3x3_D1_T4_dc16", "4x4_D2_T8_dc2", "3x4_D2_T5_dc3", "4x4_D1odd_T8_dc3"])
def test_gradient_from_bosonic_holes_matches_reference(name):
    z, meta, sites, _ = _load(name)

    def mk(desc, st):
        return FermiTensor(desc["names"], [([tuple(x) for x in segs], a) for segs, a in desc["edges"]]).set_storage(st)

    lat = fp.BosonizedLattice(sites, meta["cut"])
    samples = [(np.asarray(c), z["ws"][i]**2 / z["possibility"][i], z["eloc"][i]) for i, c in enumerate(z["confs"])]
    mine = fp.site_gradients(lat, samples)
    refs = []
    for a in range(meta["L1"]):
        for b in range(meta["L2"]):
            ref = mk(meta["gradient"][f"{a},{b}"], z[f"grad_{a}_{b}"])
            legs = [x for x in ["T", "U", "D", "L", "R"] if x in ref.names]
            refs.append((a, b, ref.transpose(["P0"] + legs).data.reshape(mine[a][b].shape)))
    scale = max(np.abs(r).max() for _, _, r in refs)
    for a, b, r in refs:
        assert np.abs(mine[a][b] - r).max() <= 1e-12 * scale, (a, b)


@pytest.mark.parametrize("name", ["3x3_D1_T4_dc16", "4x4_D2_T8_dc2", "3x4_D2_T5_dc3", "4x4_D1odd_T8_dc3"])
def test_local_energy_from_strip_values_and_integer_signs(name):
    """The form a dense kernel evaluates: strip values of the bosonized lattice times signs computed
    from particle counts alone."""
    z, meta, sites, terms = _load(name)
    lat = fp.BosonizedLattice(sites, meta["cut"])
    for i, conf in enumerate(z["confs"]):
        assert fp.local_energy_signs(lat, terms, conf) == pytest.approx(z["eloc"][i], rel=1e-12, abs=1e-12)


def test_order_inversions_is_the_leg_reordering_sign():
    rng = np.random.default_rng(11)
    for _ in range(50):
        conf = (rng.random((3, 4)) < 0.5).astype(int)
        s = fp.order_sign(conf, fp.canonical_names(3, 4, fp.COL), fp.canonical_names(3, 4, fp.ROW), -int(conf.sum()))
        assert s == (-1.0)**fp.order_inversions(conf)


@pytest.mark.parametrize("name", ["3x3_D1_T4_dc16", "4x4_D2_T8_dc2", "3x4_D2_T5_dc3"])
def test_order_sign_by_count_equals_the_tensor_transpose(name):
    """The count form of the amplitude's leg-reordering sign (no rank-L1*L2 tensor, so it works on 8x8)
    equals the graded transpose on every reference sample's leg order."""
    z, meta, _, _ = _load(name)
    canon = fp.canonical_names(meta["L1"], meta["L2"], fp.ROW)
    T = -int(np.asarray(z["confs"][0]).sum())
    for i, conf in enumerate(z["confs"]):
        names = meta["ws_names"][i]
        assert fp.order_sign_by_count(conf, canon, names, T) == fp.order_sign(conf, canon, names, T)
        assert fp.order_sign_by_count(conf, names, canon, T) == fp.order_sign(conf, names, canon, T)


def test_natural_gradient_matches_reference():
    """observer.py:576-675 on the bosonic rows, folded like the gradient, against the reference's
    natural gradient (4x4, cut 2) for a fixed step count and for an error-bounded run."""
    z, meta, sites, _ = _load("4x4_D2_T8_dc2")
    ng = np.load(os.path.join(GOLDEN, "tv_4x4_D2_T8_dc2_natgrad.npz"))
    ng_meta = json.loads(bytes(ng["meta"]).decode())

    def mk(desc, st):
        return FermiTensor(desc["names"], [([tuple(x) for x in segs], a) for segs, a in desc["edges"]]).set_storage(st)

    lat = fp.BosonizedLattice(sites, meta["cut"])
    samples = [(np.asarray(c), z["ws"][i]**2 / z["possibility"][i], z["eloc"][i]) for i, c in enumerate(z["confs"])]
    for k, (steps, error) in enumerate(ng["runs"]):
        mine = fp.natural_gradient(lat, samples, int(steps), float(error))
        refs = []
        for a in range(4):
            for b in range(4):
                ref = mk(ng_meta[f"{a},{b}"], ng[f"natgrad{k}_{a}_{b}"])
                legs = [x for x in ["T", "U", "D", "L", "R"] if x in ref.names]
                refs.append((a, b, ref.transpose(["P0"] + legs).data.reshape(mine[a][b].shape)))
        scale = max(np.abs(r).max() for _, _, r in refs)
        for a, b, r in refs:
            assert np.abs(mine[a][b] - r).max() <= 1e-12 * scale, (k, a, b)


@pytest.mark.parametrize("name", ["3x3_D1_T4_dc16", "4x4_D2_T8_dc2", "3x4_D2_T5_dc3", "4x4_D1odd_T8_dc3"])
def test_sweep_chains_reproduce_the_reference(name):
    """The reference's own chains (seeded engines, thermalisation, proposals, acceptance) replayed on
    the bosonized amplitudes: configurations bit-exact, sampling weights to 1e-12."""
    z, meta, sites, terms = _load(name)
    lat = fp.BosonizedLattice(sites, meta["cut"])
    start = np.array(meta["start"])
    k = 0
    for seed in meta["chain_seeds"]:
        chain = fp.FermionSweepChain(lat, terms, start, seed)
        for step in range(meta["n_therm"] + meta["n_samples"]):
            poss, conf = chain.sweep()
            if step < meta["n_therm"]:
                continue
            np.testing.assert_array_equal(conf, z["confs"][k])
            assert poss == pytest.approx(z["possibility"][k], rel=1e-12, abs=0)
            k += 1
    assert k == len(z["confs"])
