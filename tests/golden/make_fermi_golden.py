"""Generates tests/golden/fermi_ops.npz: random fermionic tensors put through the reference's own
TAT (the CPU build of ``oracle/build_ref.sh``) by every edge operation whose parity sign the oracle
restates (transpose, reverse_edge, merge_edge, split_edge, conjugate, contract), for Fermi U(1) and
Fermi Z2.

    python tests/golden/make_fermi_golden.py

Inputs are drawn from numpy's seeded generator; each case stores the input tensors (names, edges,
block storage), the operation's arguments and the reference's output tensor.  Tests read the file
without the reference.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle", "_ref"))

import TAT  # noqa: E402  (the reference's tensor library, built by oracle/build_ref.sh)


def _module(group):
    return TAT.FermiU1 if group == "U1" else TAT.FermiZ2


def _sym_out(group, s):
    return int(s.fermi) if group == "U1" else int(s.parity)


def _sym_in(group, s):
    return int(s) if group == "U1" else bool(s)


def to_tat(group, names, edges, storage):
    t = _module(group).D.Tensor(names, [([(_sym_in(group, s), d) for s, d in segs], arrow)
                                         for segs, arrow in edges]).zero_()
    t.storage[:] = storage
    return t


def describe(group, t):
    edges = []
    for n in t.names:
        e = t.edge_by_name(n)
        edges.append(([[_sym_out(group, s), int(d)] for s, d in list(e.segments)], bool(e.arrow)))
    return {"names": list(t.names), "edges": edges}, np.array(t.storage, dtype=np.float64)


def storage_size(group, edges):
    t = _module(group).D.Tensor([f"x{i}" for i in range(len(edges))],
                                [([(_sym_in(group, s), d) for s, d in segs], arrow) for segs, arrow in edges])
    return t.storage.size


def main():
    rng = np.random.default_rng(20261204)
    cases, arrays = [], {}

    def rand_edge(group):
        if group == "U1":
            segs = [[q, int(rng.integers(1, 3))] for q in range(-2, 3) if rng.random() < 0.7] or [[0, 1]]
            rng.shuffle(segs)
        else:
            segs = [[0, int(rng.integers(1, 3))], [1, int(rng.integers(1, 3))]]
            if rng.random() < 0.5:
                segs.reverse()
        return [segs, bool(rng.random() < 0.5)]

    def new_tensor(group, names, edges):
        n = storage_size(group, edges)
        st = np.round(rng.normal(size=n), 6)
        return {"names": names, "edges": edges}, st

    def add(op, group, inputs, args, out_tensor):
        c = len(cases)
        ins = []
        for k, (desc, st) in enumerate(inputs):
            arrays[f"in{c}_{k}"] = st
            ins.append(desc)
        desc, st = describe(group, out_tensor)
        arrays[f"out{c}"] = st
        cases.append({"op": op, "group": group, "inputs": ins, "args": args, "out": desc})

    for group in ["U1", "Z2"]:
        for trial in range(24):
            r = int(rng.integers(2, 5))
            names = [f"e{i}" for i in range(r)]
            desc, st = new_tensor(group, names, [rand_edge(group) for _ in range(r)])
            t = to_tat(group, names, desc["edges"], st)
            perm = [str(x) for x in rng.permutation(names)]
            add("transpose", group, [(desc, st)], {"names": perm}, t.transpose(perm))
            rv = sorted(str(x) for x in rng.choice(names, size=int(rng.integers(1, r + 1)), replace=False))
            ap = bool(rng.random() < 0.5)
            ex = sorted(str(x) for x in rng.choice(names, size=int(rng.integers(0, r)), replace=False))
            add("reverse_edge", group, [(desc, st)], {"names": rv, "apply_parity": ap, "exclude": ex},
                t.reverse_edge(set(rv), ap, set(ex)))
            tm = bool(rng.random() < 0.5)
            add("conjugate", group, [(desc, st)], {"trivial_metric": tm}, t.conjugate(tm))
            k = int(rng.integers(1, r))
            g1, g2 = perm[:k], perm[k:]
            ap = bool(rng.random() < 0.5)
            exm = ["a"] if rng.random() < 0.5 else []
            exr = sorted(str(x) for x in rng.choice(names, size=int(rng.integers(0, r)), replace=False))
            merged = t.merge_edge({"a": g1, "b": g2}, ap, set(exm), set(exr))
            add("merge_edge", group, [(desc, st)], {"merge": {"a": g1, "b": g2}, "apply_parity": ap,
                                                   "exclude_merge": exm, "exclude_reverse": exr}, merged)
            mdesc, mst = describe(group, merged)
            plan = {"a": [[n, desc["edges"][names.index(n)][0]] for n in g1]}
            ap2 = bool(rng.random() < 0.5)
            tplan = {"a": [(n, [(_sym_in(group, s), d) for s, d in segs]) for n, segs in plan["a"]]}
            add("split_edge", group, [(mdesc, mst)], {"split": plan, "apply_parity": ap2},
                merged.split_edge(tplan, ap2))
        for trial in range(24):
            r1, r2 = int(rng.integers(1, 5)), int(rng.integers(1, 5))
            nc = int(rng.integers(0, min(r1, r2) + 1))
            n1, n2 = [f"a{i}" for i in range(r1)], [f"b{i}" for i in range(r2)]
            e1 = [rand_edge(group) for _ in range(r1)]
            e2 = [rand_edge(group) for _ in range(r2)]
            p1, p2 = list(rng.permutation(r1))[:nc], list(rng.permutation(r2))[:nc]
            for i, j in zip(p1, p2):
                e2[j] = [[[(-s if group == "U1" else s), d] for s, d in e1[i][0]], not e1[i][1]]
            d1, s1 = new_tensor(group, n1, e1)
            d2, s2 = new_tensor(group, n2, e2)
            pairs = [[n1[i], n2[j]] for i, j in zip(p1, p2)]
            out = to_tat(group, n1, e1, s1).contract(to_tat(group, n2, e2, s2), {tuple(p) for p in pairs})
            add("contract", group, [(d1, s1), (d2, s2)], {"pairs": pairs}, out)

    arrays["meta"] = np.frombuffer(json.dumps(cases).encode(), dtype=np.uint8)
    path = os.path.join(HERE, "fermi_ops.npz")
    np.savez_compressed(path, **arrays)
    print(f"{len(cases)} cases -> {path}")


if __name__ == "__main__":
    main()
