"""Generates the fermionic golden vectors with the reference itself (its CPU build from
``oracle/build_ref.sh`` and its tetragono / tetraku sources):

* ``tests/golden/fermi_ops.npz``: random fermionic tensors put through the reference's TAT by every
  edge operation whose parity sign the oracle restates (transpose, reverse_edge, merge_edge,
  split_edge, conjugate, contract), for Fermi U(1) and Fermi Z2.  Each case stores the input tensors
  (names, edges, block storage), the operation's arguments and the reference's output tensor.
* ``tests/golden/tv_<case>.npz``: spinless-fermion t-V lattices built by tetraku's own plugin
  (tetraku/tetraku/models/tV/__init__.py:23-76), seeded random site tensors, sweep chains of the
  reference's ``SweepSampling`` and, per sample, the reference's amplitude tensor ``hole(())`` (its
  leg order and element), E_loc from its ``Observer`` and the holes ``Configuration.holes()``; per
  case the energy and the gradient; for some cases also the lattice file the reference pickles
  (``tv_<case>_lattice.pkl``) and its natural gradient by conjugate gradient (``tv_<case>_natgrad.npz``).

    python tests/golden/make_fermi_golden.py [--ops] [--tv] [REFERENCE_ROOT]

Tests read the files without the reference.
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


def make_ops():
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


def _tensor_record(t):
    names = [str(n) for n in t.names]
    edges = []
    for n in t.names:
        e = t.edge_by_name(n)
        edges.append(([[int(sym.fermi), int(d)] for sym, d in list(e.segments)], bool(e.arrow)))
    return {"names": names, "edges": edges}, np.array(t.storage, dtype=np.float64).copy()


def run_tv_case(name, L1, L2, D, T, cut, tensor_seed, chain_seeds, n_therm, n_samples, save_lattice=False,
                interior=None, dims=None, holes=True):
    """Sweep chains of the reference on a t-V lattice (t = V = 1); records per sample the amplitude
    tensor hole(()) and E_loc (observer.py:313-415).  ``dims`` = (d-, d0, d+) replaces tetraku's equal
    sector dimensions D on the R bonds and the column-0 D bonds (the 8x8 workload's (2, 4, 2));
    ``holes`` False leaves out the per-sample holes (benchmark-size lattices)."""
    sys.argv = sys.argv[:1] + [a for a in sys.argv[1:] if not a.startswith("--")]
    import make_golden  # noqa: F401  (mpi4py stand-in and the reference's paths)
    import tetragono as tet
    from tetraku.models import tV

    state = tV.abstract_lattice(L1, L2, D, T, 1.0, 1.0)
    if dims is not None:
        # tetraku's charge flow Q on these bonds, with per-sector dimensions
        for l1 in range(L1 - 1):
            Q = int(T * (L1 - l1 - 1) / L1)
            state.virtual_bond[l1, 0, "D"] = [(Q - 1, dims[0]), (Q, dims[1]), (Q + 1, dims[2])]
        for l1 in range(L1):
            for l2 in range(L2 - 1):
                Q = int(T / L1 * (L2 - l2 - 1) / L2)
                state.virtual_bond[l1, l2, "R"] = [(Q - 1, dims[0]), (Q, dims[1]), (Q + 1, dims[2])]
    if interior is not None:
        # interior D bonds with odd charges (the 8x8 workload's {-1, 0, +1} layout, scaled down)
        for l1 in range(L1 - 1):
            for l2 in range(1, L2):
                state.virtual_bond[l1, l2, "D"] = interior
    TAT.random.seed(tensor_seed)
    lattice = tet.SamplingLattice(state)
    for l1 in range(L1):
        for l2 in range(L2):
            t = lattice[l1, l2]
            z = sum(1 for n in t.names if str(n) in ("U", "D", "L", "R"))
            bond = sum(dims) if dims is not None else 3 * D
            lattice[l1, l2] = t * (1.0 / np.sqrt(2.0 * bond**z))
    out, meta = {}, {"name": name, "L1": L1, "L2": L2, "D": D, "T": T, "cut": cut, "tensor_seed": tensor_seed,
                     "chain_seeds": chain_seeds, "n_therm": n_therm, "n_samples": n_samples, "sites": {},
                     "terms": []}
    for l1 in range(L1):
        for l2 in range(L2):
            desc, st = _tensor_record(lattice[l1, l2])
            meta["sites"][f"{l1},{l2}"] = desc
            out[f"site_{l1}_{l2}"] = st
    for k, (positions, H) in enumerate(lattice._hamiltonians.items()):
        desc, st = _tensor_record(H)
        meta["terms"].append({"positions": [list(p) for p in positions], "tensor": desc})
        out[f"term_{k}"] = st
    # a start with T particles and nonzero amplitude: the first of a seeded run of random fillings
    rng = np.random.default_rng(tensor_seed)
    probe = tet.SweepSampling(lattice, cut, None, None)
    while True:
        occ = np.zeros(L1 * L2, dtype=np.int64)
        occ[rng.choice(L1 * L2, size=T, replace=False)] = 1
        start = occ.reshape(L1, L2, 1)
        probe.configuration.import_configuration(start)
        if probe.configuration.hole(()).norm_max() != 0:
            break
    observer = tet.Observer(lattice, enable_energy=True, enable_gradient=True)
    confs, poss, ws_names, ws_value, eloc = [], [], [], [], []
    want_holes = holes
    holes = {f"{a},{b}": [] for a in range(L1) for b in range(L2)}
    with observer:
        for seed in chain_seeds:
            TAT.random.seed(seed)
            sampling = tet.SweepSampling(lattice, cut, None, None)
            sampling.configuration.import_configuration(start)
            for step in range(n_therm + n_samples):
                possibility, configuration = sampling()
                if step < n_therm:
                    continue
                before = observer._whole_result_reweight["energy"]
                observer(possibility, configuration)
                ws = configuration.hole(())
                w = float(ws.storage[0])
                reweight = w * w / possibility
                confs.append(configuration.export_configuration()[:, :, 0].copy())
                poss.append(possibility)
                ws_names.append([str(n) for n in ws.names])
                ws_value.append(w)
                eloc.append((observer._whole_result_reweight["energy"] - before) / reweight)
                if not want_holes:
                    continue
                hs = configuration.holes()
                for a in range(L1):
                    for b in range(L2):
                        desc, st = _tensor_record(hs[a][b])
                        meta.setdefault("holes", {})[f"{a},{b}"] = desc
                        holes[f"{a},{b}"].append(st)
    meta["start"] = start[:, :, 0].tolist()
    meta["ws_names"] = ws_names
    out["confs"] = np.array(confs, dtype=np.int64)
    out["possibility"] = np.array(poss)
    out["ws"] = np.array(ws_value)
    out["eloc"] = np.array(eloc)
    energy, error = observer.energy
    out["energy"] = np.array([energy, error])
    out["total_weight"] = np.array(observer._total_weight)
    grad = observer.gradient
    meta["gradient"] = {}
    for a in range(L1):
        for b in range(L2):
            if want_holes:
                out[f"holes_{a}_{b}"] = np.array(holes[f"{a},{b}"])
            desc, st = _tensor_record(grad[a][b])
            meta["gradient"][f"{a},{b}"] = desc
            out[f"grad_{a}_{b}"] = st
    out["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    if save_lattice:
        import pickle
        with open(os.path.join(HERE, f"tv_{name}_lattice.pkl"), "wb") as f:
            pickle.dump(lattice, f)
    path = os.path.join(HERE, f"tv_{name}.npz")
    np.savez_compressed(path, **out)
    print(f"tv_{name}: {len(confs)} samples, E/site = {energy:.10f} +- {error:.2e}, {os.path.getsize(path)} bytes")


def run_tv_natural(name, L1, L2, D, T, cut, tensor_seed, chain_seeds, n_therm, n_samples, runs):
    """The chains of t-V case ``name`` again, observed with enable_natural_gradient; saves the
    reference's natural_gradient_by_conjugate_gradient(step, error) (observer.py:576-675) for every
    (step, error) in ``runs`` to tv_<name>_natgrad.npz (one observed run per setting, since the
    reference releases its per-sample deltas after one call)."""
    sys.argv = sys.argv[:1] + [a for a in sys.argv[1:] if not a.startswith("--")]
    import make_golden  # noqa: F401
    import tetragono as tet
    from tetraku.models import tV

    state = tV.abstract_lattice(L1, L2, D, T, 1.0, 1.0)
    TAT.random.seed(tensor_seed)
    lattice = tet.SamplingLattice(state)
    for l1 in range(L1):
        for l2 in range(L2):
            t = lattice[l1, l2]
            z = sum(1 for n in t.names if str(n) in ("U", "D", "L", "R"))
            lattice[l1, l2] = t * (1.0 / np.sqrt(2.0 * (3 * D)**z))
    start = np.load(os.path.join(HERE, f"tv_{name}.npz"))
    meta = json.loads(bytes(start["meta"]).decode())
    conf0 = np.array(meta["start"], dtype=np.int64)[:, :, None]
    out, desc = {"runs": np.array(runs, dtype=np.float64)}, {}
    for k, (steps, error) in enumerate(runs):
        observer = tet.Observer(lattice, enable_energy=True, enable_gradient=True, enable_natural_gradient=True)
        with observer:
            for seed in chain_seeds:
                TAT.random.seed(seed)
                sampling = tet.SweepSampling(lattice, cut, None, None)
                sampling.configuration.import_configuration(conf0)
                for step in range(n_therm + n_samples):
                    possibility, configuration = sampling()
                    if step >= n_therm:
                        observer(possibility, configuration)
        grad = observer.natural_gradient_by_conjugate_gradient(int(steps), float(error))
        for l1 in range(L1):
            for l2 in range(L2):
                d, st = _tensor_record(grad[l1][l2])
                desc[f"{l1},{l2}"] = d
                out[f"natgrad{k}_{l1}_{l2}"] = st
    out["meta"] = np.frombuffer(json.dumps(desc).encode(), dtype=np.uint8)
    path = os.path.join(HERE, f"tv_{name}_natgrad.npz")
    np.savez_compressed(path, **out)
    print(f"tv_{name}: natural gradient for {len(runs)} settings, {os.path.getsize(path)} bytes")


if __name__ == "__main__" and "--workloads" in sys.argv:
    # the 8x8 fermionic workload: 32 particles, {Q-1:2, Q:4, Q+1:2} on the R and column-0 D bonds,
    # {-1:2, 0:4, +1:2} on the interior D bonds, Dcut 64 (seconds per sample here: one chain, few sweeps)
    sys.path.insert(0, HERE)
    run_tv_case("8x8_D242_T32_dc24", 8, 8, 2, 32, 24, 919, [93, 94], 1, 2, interior=[(-1, 2), (0, 4), (1, 2)],
                dims=(2, 4, 2), holes=False)
    run_tv_case("8x8_D242_T32_dc64", 8, 8, 2, 32, 64, 919, [93], 1, 1, interior=[(-1, 2), (0, 4), (1, 2)],
                dims=(2, 4, 2), holes=False)
    sys.exit(0)
if __name__ == "__main__":
    sys.path.insert(0, HERE)
    both = "--ops" not in sys.argv and "--tv" not in sys.argv
    if both or "--ops" in sys.argv:
        make_ops()
    if both or "--tv" in sys.argv:
        run_tv_case("3x3_D1_T4_dc16", 3, 3, 1, 4, 16, 515, [61, 62], 3, 6, save_lattice=True)
        run_tv_case("4x4_D2_T8_dc2", 4, 4, 2, 8, 2, 616, [71, 72], 3, 6)
        run_tv_case("3x4_D2_T5_dc3", 3, 4, 2, 5, 3, 717, [81, 82], 3, 6, save_lattice=True)
        run_tv_natural("4x4_D2_T8_dc2", 4, 4, 2, 8, 2, 616, [71, 72], 3, 6, [(6, 0.0), (50, 1e-3)])
        run_tv_case("4x4_D1odd_T8_dc3", 4, 4, 1, 8, 3, 818, [91, 92], 3, 6,
                    interior=[(-1, 1), (0, 2), (1, 1)])
