"""The fermionic tensor oracle (oracle/fermi_tensor.py) against the reference's TAT: golden outputs of
every sign-carrying edge operation (tests/golden/fermi_ops.npz, made by
tests/golden/make_fermi_golden.py), the known answers of TAT's own fermion tests restated, and a
live comparison when the reference's CPU build is present."""
import itertools
import json
import os
import sys

import numpy as np
import pytest

from oracle.fermi_tensor import FermiTensor

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "fermi_ops.npz")


def _tensor(group, desc, storage):
    t = FermiTensor(desc["names"], [([tuple(sd) for sd in segs], arrow) for segs, arrow in desc["edges"]], group)
    return t.set_storage(storage)


def _apply(case, ins):
    op, a = case["op"], case["args"]
    t = ins[0]
    if op == "transpose":
        return t.transpose(a["names"])
    if op == "reverse_edge":
        return t.reverse_edge(set(a["names"]), a["apply_parity"], set(a["exclude"]))
    if op == "conjugate":
        return t.conjugate(a["trivial_metric"])
    if op == "merge_edge":
        return t.merge_edge(a["merge"], a["apply_parity"], set(a["exclude_merge"]), set(a["exclude_reverse"]))
    if op == "split_edge":
        plan = {k: [(n, [tuple(sd) for sd in segs]) for n, segs in v] for k, v in a["split"].items()}
        return t.split_edge(plan, a["apply_parity"])
    if op == "contract":
        return t.contract(ins[1], {tuple(p) for p in a["pairs"]})
    raise ValueError(op)


def test_golden_edge_operations():
    z = np.load(GOLDEN)
    cases = json.loads(bytes(z["meta"]).decode())
    seen = set()
    for c, case in enumerate(cases):
        ins = [_tensor(case["group"], d, z[f"in{c}_{k}"]) for k, d in enumerate(case["inputs"])]
        out = _apply(case, ins)
        want = _tensor(case["group"], case["out"], z[f"out{c}"])
        assert out.names == want.names, (c, case["op"])
        assert out.edges == want.edges, (c, case["op"])
        tol = 1e-12 if case["op"] == "contract" else 0.0
        assert np.abs(out.storage() - want.storage()).max(initial=0.0) <= tol, (c, case["op"])
        seen.add((case["group"], case["op"]))
    assert len(seen) == 12


def test_transpose_sign_rank6_z2():
    """TAT's own rank-6 Z2 transpose known answer: the sign is the parity of the exchanged odd pairs."""
    edge = ([(0, 2), (1, 2)], False)
    a = FermiTensor(list("ijklmn"), [edge] * 6, "Z2").range_()
    b = a.transpose(list("ljinkm"))
    for idx in itertools.product(range(4), repeat=6):
        p = [x >= 2 for x in idx]
        if sum(p) % 2:
            continue
        i, j, k, l, m, n = p
        flip = (l and (i ^ j ^ k)) ^ (j and i) ^ (n and (k ^ m))
        where = {name: (int(x >= 2), x % 2) for name, x in zip("ijklmn", idx)}
        assert b[where] == (-a[where] if flip else a[where])


def test_merge_sign_counts_odd_edges():
    """FermiU1 merge with parity applied equals the bosonic merge up to the sign (n_odd & 2)."""
    edge = [(-1, 1), (0, 1), (1, 1)]
    a = FermiTensor(list("12345"), [edge] * 5).range_()
    for i in range(5):
        for j in range(i, 5):
            names = a.names[i:j]
            merged = a.merge_edge({"m": names}, True)
            plain = a.merge_edge({"m": names}, False)
            back = merged.split_edge({"m": [(n, edge) for n in names]}, True)
            assert np.array_equal(back.data, a.data)
            for s in itertools.product([-1, 0, 1], repeat=5):
                if sum(s):
                    continue
                count = sum(s[x] != 0 for x in range(i, j))
                item = a[{str(q + 1): (s[q], 0) for q in range(5)}]
                pos = np.flatnonzero(plain.storage() == item)
                assert pos.size == 1
                assert merged.storage()[pos[0]] == (-item if count & 2 else item)


def test_conjugate_norms_and_involution():
    seg = [(-1, 2), (0, 2), (1, 2)]
    a = FermiTensor(["i", "j"], [seg, seg]).range_(-8, 1)
    assert a.contract(a.conjugate(), {("i", "i"), ("j", "j")}).scalar() > 0
    assert (a.conjugate().conjugate() - a).norm_max() == 0
    b = FermiTensor(["i", "j"], [(seg, False), (seg, True)]).range_(-8, 1)
    assert b.contract(b.conjugate(), {("i", "i"), ("j", "j")}).scalar() < 0
    assert b.contract(b.conjugate(True), {("i", "i"), ("j", "j")}).scalar() > 0
    assert (b.conjugate(True).conjugate(True) - b).norm_max() == 0


def _bosonic_contract(a, b, pairs):
    ia = [a.names.index(x) for x, _ in pairs]
    ib = [b.names.index(y) for _, y in pairs]
    data = np.tensordot(a.data, b.data, (ia, ib))
    names = [n for n in a.names if n not in {x for x, _ in pairs}] + [n for n in b.names if n not in {y for _, y in pairs}]
    edges = [e for n, e in zip(a.names, a.edges) if n in names] + [e for n, e in zip(b.names, b.edges) if n in names]
    return FermiTensor(names, edges, a.group, data)


def test_contract_matches_bosonic_and_either_order():
    """TAT's fermi example 0: contracting in either order agrees, and with these arrows the result
    equals the bosonic U(1) contraction of the same storages."""
    e1 = [(-1, 2), (0, 2), (1, 2)]
    e2 = [(1, 2), (0, 2), (-1, 2)]
    a = FermiTensor(list("abcd"), [(e1, True), e2, (e1, True), (e2, True)]).range_()
    b = FermiTensor(list("efgh"), [e1, e2, (e1, True), e2]).range_()
    c = a.contract(b, {("d", "e"), ("c", "f")})
    d = b.contract(a, {("e", "d"), ("f", "c")})
    assert (c - d).norm_max() == 0
    assert np.array_equal(c.storage(), _bosonic_contract(a, b, [("d", "e"), ("c", "f")]).storage())


def test_contract_commutes_with_merge_and_reverse():
    edge1 = ([(-1, 2), (0, 2), (1, 2)], False)
    edge2 = ([(1, 2), (0, 2), (-1, 2)], True)
    a = FermiTensor(list("abcd"), [edge1, edge2, edge1, edge2]).range_()
    b = FermiTensor(list("efgh"), [edge1, edge2, edge1, edge2]).range_()
    c = a.contract(b, {("a", "f"), ("b", "g"), ("c", "h")})
    am = a.merge_edge({"m": ["b", "a"]}, False)
    bm = b.merge_edge({"m": ["g", "f"]}, True)
    assert (c - am.contract(bm, {("m", "m"), ("c", "h")})).norm_max() == 0
    ar = a.reverse_edge({"b", "a"}, False)
    br = b.reverse_edge({"g", "f"}, True)
    assert (c - ar.contract(br, {("a", "f"), ("b", "g"), ("c", "h")})).norm_max() == 0


def _reference_tat():
    ref = os.path.join(ROOT, "oracle", "_ref")
    if not (os.path.isdir(ref) and any(f.startswith("TAT") and f.endswith(".so") for f in os.listdir(ref))):
        pytest.skip("the reference's CPU build is not present")
    sys.path.insert(0, ref)
    import TAT
    return TAT


def test_live_against_reference_tat():
    TAT = _reference_tat()
    rng = np.random.default_rng(7)

    def to_tat(f):
        t = TAT.FermiU1.D.Tensor(f.names, [(list(e[0]), e[1]) for e in f.edges]).zero_()
        t.storage[:] = f.storage()
        return t

    def check(f, t):
        edges = []
        for n in t.names:
            e = t.edge_by_name(n)
            edges.append((tuple((int(s.fermi), int(d)) for s, d in list(e.segments)), bool(e.arrow)))
        assert list(t.names) == f.names and edges == f.edges
        assert np.abs(np.array(t.storage) - f.storage()).max(initial=0.0) <= 1e-12

    def rand_edge():
        segs = [(q, int(rng.integers(1, 3))) for q in range(-2, 3) if rng.random() < 0.7] or [(0, 1)]
        rng.shuffle(segs)
        return ([tuple(x) for x in segs], bool(rng.random() < 0.5))

    for _ in range(40):
        r = int(rng.integers(2, 5))
        names = [f"e{i}" for i in range(r)]
        f = FermiTensor(names, [rand_edge() for _ in range(r)])
        f.set_storage(rng.normal(size=f.storage().size))
        t = to_tat(f)
        perm = [str(x) for x in rng.permutation(names)]
        check(f.transpose(perm), t.transpose(perm))
        check(f.conjugate(True), t.conjugate(True))
        check(f.merge_edge({"m": perm[:2]}, True), t.merge_edge({"m": perm[:2]}, True))
        other = FermiTensor(["x", "y"], [([(-s, d) for s, d in f.edges[0][0]], not f.edges[0][1]), rand_edge()])
        other.set_storage(rng.normal(size=other.storage().size))
        check(f.contract(other, {("e0", "x")}), t.contract(to_tat(other), {("e0", "x")}))
