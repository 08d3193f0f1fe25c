"""Host side of fermionic lattices (tnsp_gb300/fermion.py): the reference's t-V lattice file read
without the reference, the sign-folded slices and count-based signs checked against the oracle, and
the whole data flow a dense sampler would run (slices -> boundary MPS -> amplitude, E_loc, gradient)
emulated through the dense oracle and compared with the reference's own outputs."""
import io
import json
import os

import numpy as np
import pytest

from oracle import fermi_peps as fp
from oracle.fermi_tensor import FermiTensor
from oracle.peps_oracle import DensePEPS, Environment
from tnsp_gb300 import fermion as F
from tnsp_gb300.checkpoint import load_lattice, save_lattice

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _golden(name):
    z = np.load(os.path.join(GOLDEN, f"tv_{name}.npz"))
    meta = json.loads(bytes(z["meta"]).decode())

    def mk(desc, st):
        return FermiTensor(desc["names"], [([tuple(x) for x in segs], a) for segs, a in desc["edges"]]).set_storage(st)

    sites = [[mk(meta["sites"][f"{a},{b}"], z[f"site_{a}_{b}"]) for b in range(meta["L2"])] for a in range(meta["L1"])]
    return z, meta, sites, mk


def _host(sites, terms=None):
    """A FermionLattice from oracle site tensors (same block storage the reference holds)."""
    L1, L2 = len(sites), len(sites[0])
    from tnsp_gb300.lattice import site_charges, site_from_blocks
    tensors, legs, edges, names = [], [], [], []
    T = 0
    for a in range(L1):
        rt, rl, re, rn = [], [], [], []
        for b in range(L2):
            s = sites[a][b]
            segs = [list(e[0]) for e in s.edges]
            rt.append(site_from_blocks(s.storage(), s.names, segs))
            rl.append(site_charges(s.names, segs)[0])
            re.append([(list(e[0]), e[1]) for e in s.edges])
            rn.append(list(s.names))
            if "T" in s.names:
                T = s.edge_by_name("T")[0][0][0]
        tensors.append(rt), legs.append(rl), edges.append(re), names.append(rn)
    return F.FermionLattice(L1, L2, tensors, legs, T, terms or {}, edges, names)


def test_reference_lattice_file_reads_without_the_reference():
    z, meta, sites, _ = _golden("3x3_D1_T4_dc16")
    lat = F.from_reference_lattice(load_lattice(os.path.join(GOLDEN, "tv_3x3_D1_T4_dc16_lattice.pkl")))
    assert (lat.L1, lat.L2, lat.particles) == (3, 3, 4)
    host = _host(sites)
    for a in range(3):
        for b in range(3):
            np.testing.assert_array_equal(lat.tensors[a][b], host.tensors[a][b])
            assert lat.names[a][b] == meta["sites"][f"{a},{b}"]["names"]
            assert [(list(map(tuple, segs)), arrow) for segs, arrow in meta["sites"][f"{a},{b}"]["edges"]] == \
                [(list(map(tuple, segs)), arrow) for segs, arrow in lat.edges[a][b]]
    positions = [tuple(tuple(p) for p in t["positions"]) for t in meta["terms"]]
    assert list(lat.terms.keys()) == positions
    for table in lat.terms.values():
        assert table == F.tv_element_table()
    built = F.random_tv(3, 3, 1, 4, seed=0)
    assert list(built.terms.keys()) == positions
    assert built.names == lat.names and built.edges == lat.edges


def test_fermionic_lattice_file_round_trip():
    path = os.path.join(GOLDEN, "tv_3x3_D1_T4_dc16_lattice.pkl")
    ref = load_lattice(path)
    buf = io.BytesIO()
    save_lattice(ref, buf)
    buf.seek(0)
    back = load_lattice(buf)
    for a in range(3):
        for b in range(3):
            t0, t1 = ref.state["_lattice"][a][b], back.state["_lattice"][a][b]
            assert t0.dumps() == t1.dumps()
            assert t1.arrows == t0.arrows


def test_sign_folded_slices_equal_the_oracle():
    _, _, sites, _ = _golden("4x4_D2_T8_dc2")
    host = _host(sites)
    for a in range(4):
        for b in range(4):
            sl = host.sign_folded_slices(a, b)
            for family in (F.ROW, F.COL):
                for n in (0, 1):
                    for m in (0, 1):
                        want = fp.bosonized_site(sites[a][b], a, b, n, m, family)
                        np.testing.assert_array_equal(sl[family, n, m], want)


def test_count_based_signs_equal_the_oracle():
    rng = np.random.default_rng(5)
    for _ in range(200):
        conf = (rng.random((4, 5)) < 0.5).astype(np.int64)
        pT = int(rng.integers(0, 2))
        for family in (F.ROW, F.COL):
            assert F.configuration_sign(conf, pT, family) == fp.configuration_sign(conf, pT, family)
        assert F.order_inversions(conf) == fp.order_inversions(conf)
        a, b = int(rng.integers(0, 4)), int(rng.integers(0, 4))
        pos = [(a, b), (a, b + 1)] if rng.random() < 0.5 else [(a, b), (a + 1, b)] if a < 3 else [(a, b), (a, b + 1)]
        new = [int(conf[pos[1]]), int(conf[pos[0]])]
        assert F.hop_sign(conf, pos, new) == fp.hop_sign(conf, pos, new)


class _Emulator:
    """The sampler's data flow on the host tables: per configuration the slices [family][n][M parity]
    of every site, dense row / column boundaries (the oracle's), count-based signs."""

    def __init__(self, host, cut):
        self.h, self.cut = host, cut

    def _peps(self, conf, family):
        M = (np.cumsum(conf, axis=1) - conf) if family == F.ROW else (np.cumsum(conf, axis=0) - conf)
        A = [[None] * self.h.L2 for _ in range(self.h.L1)]
        for a in range(self.h.L1):
            for b in range(self.h.L2):
                sl = self.h.sign_folded_slices(a, b)
                n = int(conf[a, b])
                full = np.zeros((2,) + sl.shape[3:])
                full[n] = sl[family, n, M[a, b] & 1]
                A[a][b] = full
        return DensePEPS(A, [], self.cut, charges=self.h.charges())

    def observe(self, conf):
        conf = np.asarray(conf)
        envs = {f: Environment(self._peps(conf, f), conf) for f in (F.ROW, F.COL)}
        psi = envs[F.ROW].amplitude()
        eloc = 0.0
        for positions, table in self.h.terms.items():
            pos = [p[:2] for p in positions]
            here = tuple(int(conf[p]) for p in pos)
            for new, h in table.get(here, []):
                changed = [(p, s) for p, s in zip(pos, new) if conf[p] != s]
                if not changed:
                    eloc += h
                    continue
                (p0, s0), (p1, s1) = sorted(changed)
                after = conf.copy()
                after[p0], after[p1] = s0, s1
                family = F.ROW if p0[0] == p1[0] else F.COL
                env = envs[family]
                M = (np.cumsum(after, axis=1) - after) if family == F.ROW else (np.cumsum(after, axis=0) - after)
                for (a, b), s in ((p0, s0), (p1, s1)):
                    env.peps.A[a][b][s] = self.h.sign_folded_slices(a, b)[family, s, M[a, b] & 1]
                if family == F.ROW:
                    wss, sigma = env.replace_horizontal(p0[0], p0[1], s0, s1), 1.0
                else:
                    wss = env.replace_vertical(p0[0], p0[1], s0, s1)
                    sigma = F.vertical_pair_sign(conf, after, self.h.p_T)
                eloc += h * F.hop_sign(conf, pos, new) * sigma * wss / psi
        M = np.cumsum(conf, axis=1) - conf
        holes = [[None] * self.h.L2 for _ in range(self.h.L1)]
        for a in range(self.h.L1):
            for b in range(self.h.L2):
                hb = envs[F.ROW].site_hole(a, b) / psi
                if M[a, b] & 1:
                    hb = hb * self.h.prefix_sign(a, b, F.ROW)
                holes[a][b] = hb
        return psi * F.configuration_sign(conf, self.h.p_T, F.ROW), eloc, holes


@pytest.mark.parametrize("name", ["3x3_D1_T4_dc16", "4x4_D2_T8_dc2", "3x4_D2_T5_dc3", "4x4_D1odd_T8_dc3"])
def test_host_tables_reproduce_the_reference_through_a_dense_sampler(name):
    z, meta, sites, mk = _golden(name)
    lat = load_lattice(os.path.join(GOLDEN, f"tv_{name}_lattice.pkl")) if name.startswith("3x3") else None
    host = F.from_reference_lattice(lat) if lat is not None else _host(sites)
    if lat is None:
        host.terms = {tuple(tuple(p) for p in t["positions"]): F.tv_element_table() for t in meta["terms"]}
    em = _Emulator(host, meta["cut"])
    L1, L2 = meta["L1"], meta["L2"]
    W, EW = 0.0, 0.0
    D = [[np.zeros((2,) + host.tensors[a][b].shape[1:]) for b in range(L2)] for a in range(L1)]
    ED = [[np.zeros_like(D[a][b]) for b in range(L2)] for a in range(L1)]
    for i, conf in enumerate(z["confs"]):
        conf = np.asarray(conf)
        psi, eloc, holes = em.observe(conf)
        canon = fp.canonical_names(L1, L2, fp.ROW)
        assert psi * fp.order_sign(conf, canon, meta["ws_names"][i], host.T_charge) == \
            pytest.approx(z["ws"][i], rel=1e-12, abs=0)
        assert eloc == pytest.approx(z["eloc"][i], rel=1e-12, abs=1e-12)
        rw = z["ws"][i]**2 / z["possibility"][i]
        W += rw
        EW += rw * eloc
        for a in range(L1):
            for b in range(L2):
                D[a][b][conf[a, b]] += rw * holes[a][b]
                ED[a][b][conf[a, b]] += rw * eloc * holes[a][b]
    E = EW / W
    scale = 0.0
    errs = []
    for a in range(L1):
        for b in range(L2):
            g = host.fold_gradient(a, b, 2 * (ED[a][b] / W - E * D[a][b] / W))
            mine = FermiTensor(host.names[a][b], host.edges[a][b]).set_storage(host.to_blocks(a, b, g))
            ref = mk(meta["gradient"][f"{a},{b}"], z[f"grad_{a}_{b}"])
            diff = mine.transpose(ref.names).storage() - ref.storage()
            scale = max(scale, np.abs(ref.storage()).max())
            errs.append(np.abs(diff).max())
    assert max(errs) <= 1e-12 * scale


def test_fermionic_workload_layout():
    """The 8x8 t-V workload: 32 particles, sectors {Q-1:2, Q:4, Q+1:2} on R bonds and column-0 D bonds
    with tetraku's charge flow Q, {-1:2, 0:4, +1:2} on interior D bonds, U/L legs the conjugates."""
    lat = F.random_tv(8, 8, (2, 4, 2), 32, seed=3, interior=[(-1, 2), (0, 4), (1, 2)])
    assert lat.particles == 32 and lat.names[0][0] == ["P0", "T", "D", "R"]
    e00 = dict(zip(lat.names[0][0], lat.edges[0][0]))
    assert e00["T"] == ([(-32, 1)], False)
    assert e00["D"] == ([(27, 2), (28, 4), (29, 2)], False)   # Q = int(32 * 7 / 8)
    assert e00["R"] == ([(2, 2), (3, 4), (4, 2)], False)      # Q = int(4 * 7 / 8)
    e33 = dict(zip(lat.names[3][3], lat.edges[3][3]))
    assert e33["D"] == ([(-1, 2), (0, 4), (1, 2)], False)
    assert e33["U"] == ([(1, 2), (0, 4), (-1, 2)], True)
    assert e33["L"] == ([(-1, 2), (-2, 4), (-3, 2)], True)
    for a in range(8):
        for b in range(8):
            t = lat.tensors[a][b]
            assert t.shape == (2,) + tuple(len(lat.legs[a][b][x]) for x in F.LEGS)
    # every element outside the charge-conserving blocks is zero
    for a in range(8):
        for b in range(8):
            q = lat.legs[a][b]
            flux = lat.flux()[a][b]
            tot = (np.arange(2)[:, None, None, None, None] + np.array(q["U"])[None, :, None, None, None] +
                   np.array(q["D"])[None, None, :, None, None] + np.array(q["L"])[None, None, None, :, None] +
                   np.array(q["R"])[None, None, None, None, :])
            assert not lat.tensors[a][b][tot != flux].any()


def test_sampler_inputs_of_a_fermionic_lattice():
    """What engine.Sampler uploads for a fermionic lattice: the dense tensors with U(1) charges and the
    element tables (tnsp_lattice_upload / _charges / tnsp_model_upload), then every site's eight
    slices in site order (tnsp_lattice_fermion); the drop-in Observer folds flat gradients."""
    fl = F.random_tv(3, 4, 2, 5, seed=9)
    lat = fl.sampling_lattice()
    assert lat.fermion is fl and lat.P == 2
    q, qp, flux = lat.charge_arrays()
    assert qp.tolist() == [0, 1] and flux.reshape(3, 4)[0, 0] == 5 and not flux.reshape(3, 4)[1:].any()
    flat = fl.slices_flat()
    assert flat.size == 8 * sum(t[0].size for row in fl.tensors for t in row)
    pos = 0
    for a in range(3):
        for b in range(4):
            sl = fl.sign_folded_slices(a, b)
            np.testing.assert_array_equal(flat[pos:pos + sl.size], sl.ravel())
            pos += sl.size
    g = np.arange(lat.flat_tensors().size, dtype=np.float64)
    folded = lat.unflatten(fl.fold_flat(g))
    raw = lat.unflatten(g)
    for a in range(3):
        for b in range(4):
            np.testing.assert_array_equal(folded[a][b], fl.fold_gradient(a, b, raw[a][b]))
    n, sites, offs, cnts, outs, vals = lat.term_arrays()
    assert n == len(fl.terms) == 3 * 3 + 2 * 4


def test_fermionic_lattice_file_write_back():
    """New dense tensors written into a reference t-V lattice file come back from our reader, and the
    reference's own loader reads the file (when the reference is present)."""
    path = os.path.join(GOLDEN, "tv_3x4_D2_T5_dc3_lattice.pkl")
    ref = load_lattice(path)
    lat = F.from_reference_lattice(ref)
    new = [[-0.5 * lat.tensors[a][b] for b in range(lat.L2)] for a in range(lat.L1)]
    F.set_reference_tensors(ref, new)
    buf = io.BytesIO()
    save_lattice(ref, buf)
    buf.seek(0)
    back = F.from_reference_lattice(load_lattice(buf))
    for a in range(lat.L1):
        for b in range(lat.L2):
            np.testing.assert_array_equal(back.tensors[a][b], new[a][b])
            assert back.edges[a][b] == lat.edges[a][b]
    bad = [[t.copy() for t in row] for row in new]
    zero = np.argwhere(bad[1][1] == 0)[0]
    bad[1][1][tuple(zero)] = 1.0
    with pytest.raises(ValueError):
        F.set_reference_tensors(load_lattice(path), bad)
    from test_checkpoint import _reference_modules
    _reference_modules()   # skips when the reference is not available
    import pickle
    theirs = pickle.loads(buf.getvalue())
    for a in range(lat.L1):
        for b in range(lat.L2):
            np.testing.assert_array_equal(np.array(theirs[a, b].storage), ref.state["_lattice"][a][b].storage)


def test_tv_builder_sector_dimensions():
    """An int D and the equal triple (D, D, D) build the same layout (tetraku's [(0, D)] interior bonds)."""
    a = F.random_tv(3, 3, 2, 4, seed=1)
    b = F.random_tv(3, 3, (2, 2, 2), 4, seed=1)
    assert a.edges == b.edges
    for r1, r2 in zip(a.tensors, b.tensors):
        for t1, t2 in zip(r1, r2):
            np.testing.assert_array_equal(t1, t2)
