"""Generates the golden vectors in tests/golden/*.npz by running the reference itself.

Run in a container that has the reference checkout and the reference CPU build
(``oracle/build_ref.sh``):

    python tests/golden/make_golden.py [REFERENCE_ROOT]   (default: $TNSP_REFERENCE_ROOT)

Each case builds a seeded random PEPS with the reference's own classes, runs independent sweep
chains with ``SweepSampling`` and measures every sample with ``Observer`` (energy + gradient),
exactly as ``gradient_descent`` does (tetragono/tetragono/sampling_lattice/gradient.py:331-358),
one chain per simulated MPI rank (each chain re-seeds ``TAT.random``).  It records

* the site tensors: raw block storage in the reference's core order plus edge metadata, and the
  dense array the reference itself produces with ``clear_symmetry`` (names P0, U, D, L, R);
* the Hamiltonian terms in dictionary order, with the reference's ``tensor_element`` tables;
* the reference's sweep order;
* per chain and per sweep: the configuration and the sampling weight ``possibility``;
* per sample: ws = hole(()), E_loc, and the dense holes of every site;
* the final energy per site (with its error bar) and the gradient.

The generated files are committed; tests never need the reference at run time.
"""
import os
import sys
import types
import json
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
_ARGS = [a for a in sys.argv[1:] if not a.startswith("--")]
REF = _ARGS[0] if _ARGS else os.environ.get("TNSP_REFERENCE_ROOT", "")
if not REF and __name__ == "__main__":
    sys.exit("usage: make_golden.py REFERENCE_ROOT (or set TNSP_REFERENCE_ROOT)")


def install_mpi_stub():
    """A one-process stand-in for mpi4py (the reference imports it unconditionally)."""
    mpi4py = types.ModuleType("mpi4py")
    MPI = types.ModuleType("mpi4py.MPI")

    class Comm:

        def Get_rank(self):
            return 0

        def Get_size(self):
            return 1

        def Allreduce(self, *args, **kwargs):
            pass

        def Allgather(self, send, recv):
            recv[...] = send

        def Iallreduce(self, *args, **kwargs):
            return None

        def Bcast(self, *args, **kwargs):
            pass

        def Ibcast(self, *args, **kwargs):
            return None

        def bcast(self, value, root=0):
            return value

        def allreduce(self, value, op=None):
            return value

        def Barrier(self):
            pass

    class Request:

        @staticmethod
        def Waitall(requests):
            pass

    MPI.COMM_WORLD = Comm()
    MPI.IN_PLACE = object()
    MPI.SUM = "sum"
    MPI.Request = Request
    mpi4py.MPI = MPI
    sys.modules["mpi4py"] = mpi4py
    sys.modules["mpi4py.MPI"] = MPI


def setup_paths():
    sys.path.insert(0, os.path.join(REPO, "oracle", "_ref"))
    for sub in ("tetragono", "tetraku", "lazy_graph", "PyScalapack"):
        sys.path.insert(0, os.path.join(REF, sub))


install_mpi_stub()
setup_paths()
import TAT  # noqa: E402
import tetragono as tet  # noqa: E402
from tetragono.tensor_element import tensor_element  # noqa: E402

ORDER = ["P0", "U", "D", "L", "R"]


def dense_site(tensor):
    """Dense array (P0, U, D, L, R) with extent 1 for absent legs, via the reference's own
    ``clear_symmetry`` (which concatenates segments in edge order).  The one-dimensional
    total-symmetry leg T of site (0, 0) carries no index and is dropped."""
    names = [str(n) for n in tensor.names]
    t = tensor if isinstance(tensor, TAT.No.D.Tensor) else tensor.clear_symmetry()
    present = [n for n in ORDER if n in names]
    extra = [n for n in names if n not in ORDER]
    for n in extra:
        assert t.edge_by_name(n).dimension == 1, n
    arr = np.array(t.blocks[present + extra])
    arr = arr.reshape(arr.shape[:len(present)])
    shape = [arr.shape[present.index(n)] if n in present else 1 for n in ORDER]
    return arr.reshape(shape).copy()


def edge_meta(tensor):
    meta = []
    for i, name in enumerate(tensor.names):
        edge = tensor.edges[i]
        segs = [(int(getattr(sym, "u1", 0)) if not isinstance(sym, TAT.No.Symmetry) else 0, int(dim))
                for sym, dim in edge.segments]
        meta.append({"name": str(name), "arrow": bool(edge.arrow), "segments": segs})
    return meta


def point_index(edge, point):
    sym, idx = point
    return int(edge.index_by_point((sym, idx)))


def build_lattice(kind, L1, L2, D, seed):
    """Heisenberg antiferromagnet H = S.S (J=1) in the reference's own conventions."""
    if kind == "no":
        from tetraku.models import heisenberg
        state = tet.AbstractLattice(heisenberg.abstract_state(L1, L2, J=-1))
        state.virtual_bond["R"] = D
        state.virtual_bond["D"] = D
    elif kind == "u1":
        # A Bose-U(1) Heisenberg model; tetraku ships none, so it is built here: physical charge
        # 2Sz in {+1, -1}; H = Sz Sz + (S+ S- + S- S+)/2.
        state = tet.AbstractState(TAT.BoseU1.D.Tensor, L1, L2)
        state.physics_edges[...] = [(1, 1), (-1, 1)]
        phys = state.physics_edges[0, 0, 0]
        SS = TAT.BoseU1.D.Tensor(["I0", "I1", "O0", "O1"], [phys.conjugate(), phys.conjugate(), phys, phys]).zero_()
        charges = [1, -1]
        for a in range(2):
            for b in range(2):
                sa, sb = charges[a], charges[b]
                SS[{"I0": (-sa, 0), "I1": (-sb, 0), "O0": (sa, 0), "O1": (sb, 0)}] = 0.25 * sa * sb
                if a != b:
                    SS[{"I0": (-sa, 0), "I1": (-sb, 0), "O0": (sb, 0), "O1": (sa, 0)}] = 0.5
        state.hamiltonians["vertical_bond"] = SS
        state.hamiltonians["horizontal_bond"] = SS
        state = tet.AbstractLattice(state)
        segs = [(-1, D[0]), (0, D[1]), (1, D[2])]
        state.virtual_bond["R"] = segs
        state.virtual_bond["D"] = segs
    else:
        raise ValueError(kind)
    TAT.random.seed(seed)
    lattice = tet.SamplingLattice(state)
    # scale by 1/sqrt(2 D^z): z = number of virtual bonds at the site
    for l1 in range(L1):
        for l2 in range(L2):
            t = lattice[l1, l2]
            z = sum(1 for n in t.names if str(n) in ("U", "D", "L", "R"))
            dim = D if isinstance(D, int) else sum(D)
            lattice[l1, l2] = t * (1.0 / np.sqrt(2.0 * dim**z))
    return lattice


def run_case(name, kind, L1, L2, D, cut, tensor_seed, chain_seeds, n_therm, n_samples, compact=False):
    """``compact`` (the benchmark-size lattices): site tensors as block storage only (the dense form
    follows from the edges), no per-sample holes, and the gradient as the values of its allowed
    entries only (those where the dense site tensor is nonzero, in row-major order)."""
    lattice = build_lattice(kind, L1, L2, D, tensor_seed)
    out = {}
    meta = {"name": name, "kind": kind, "L1": L1, "L2": L2, "D": D, "cut": cut, "tensor_seed": tensor_seed,
            "chain_seeds": chain_seeds, "n_therm": n_therm, "n_samples": n_samples, "sites": {}, "terms": [],
            "compact": compact}
    for l1 in range(L1):
        for l2 in range(L2):
            t = lattice[l1, l2]
            if not compact:
                out[f"site_{l1}_{l2}_dense"] = dense_site(t)
            out[f"site_{l1}_{l2}_storage"] = np.array(t.storage).copy()
            meta["sites"][f"{l1},{l2}"] = edge_meta(t)
    phys = lattice.physics_edges[0, 0, 0]
    for ti, (positions, H) in enumerate(lattice._hamiltonians.items()):
        table = tensor_element(H)
        rows = []
        for s_in, outs in table.items():
            for s_out, value in outs.items():
                rows.append([point_index(phys, p) for p in s_in] + [point_index(phys, p) for p in s_out] +
                            [float(value.storage[0])])
        out[f"term_{ti}_table"] = np.array(rows)
        out[f"term_{ti}_storage"] = np.array(H.storage).copy()
        meta["terms"].append({"positions": [list(p) for p in positions], "edges": edge_meta(H)})

    # chains
    neel = np.zeros((L1, L2, 1), dtype=np.int64)
    for l1 in range(L1):
        for l2 in range(L2):
            neel[l1, l2, 0] = (l1 + l2) % 2
    observer = tet.Observer(lattice, enable_energy=True, enable_gradient=True)
    confs, poss, ws_list, eloc_list, holes_list = [], [], [], [], []
    sweep_order = None
    with observer:
        for seed in chain_seeds:
            TAT.random.seed(seed)
            sampling = tet.SweepSampling(lattice, cut, None, None)
            if sweep_order is None:
                sweep_order = [[list(p) for p in ps] for ps in sampling._sweep_order]
            sampling.configuration.import_configuration(neel)
            c_confs, c_poss, c_ws, c_eloc, c_holes = [], [], [], [], []
            for step in range(n_therm + n_samples):
                possibility, configuration = sampling()
                c_confs.append(configuration.export_configuration()[:, :, 0].copy())
                c_poss.append(possibility)
                if step >= n_therm:
                    before = observer._whole_result_reweight["energy"]
                    observer(possibility, configuration)
                    ws = float(configuration.hole(()).storage[0])
                    reweight = ws * ws / possibility
                    eloc = (observer._whole_result_reweight["energy"] - before) / reweight
                    c_ws.append(ws)
                    c_eloc.append(eloc)
                    if not compact:
                        holes = configuration.holes()
                        c_holes.append(np.stack([
                            np.stack([dense_site(holes[l1][l2]) for l2 in range(L2)]) for l1 in range(L1)
                        ]) if _same_shapes(holes, L1, L2) else _pack_holes(holes, L1, L2))
            confs.append(c_confs)
            poss.append(c_poss)
            ws_list.append(c_ws)
            eloc_list.append(c_eloc)
            holes_list.append(c_holes)
    out["confs"] = np.array(confs, dtype=np.int64)
    out["possibility"] = np.array(poss)
    out["ws"] = np.array(ws_list)
    out["eloc"] = np.array(eloc_list)
    if not compact:
        for l1 in range(L1):
            for l2 in range(L2):
                out[f"holes_{l1}_{l2}"] = np.array([[h[l1][l2] for h in c] for c in holes_list])
    energy, error = observer.energy
    out["energy"] = np.array([energy, error])
    out["total_weight"] = np.array(observer._total_weight)
    grad = observer.gradient
    for l1 in range(L1):
        for l2 in range(L2):
            g = dense_site(grad[l1][l2])
            if compact:
                mask = dense_site(lattice[l1, l2]) != 0
                assert not g[~mask].any()
                out[f"grad_{l1}_{l2}_allowed"] = g[mask]
            else:
                out[f"grad_{l1}_{l2}"] = g
    meta["sweep_order"] = sweep_order
    out["meta"] = np.array(json.dumps(meta))
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **out)
    print(f"{name}: E/site = {energy:.12f} +- {error:.3e}, saved {os.path.getsize(path)} bytes")


def center_fixed(configuration, replacement):
    """A restricted subspace for the tests: site (1, 1) keeps its value (EdgePoint index)."""
    return replacement.get((1, 1, 0), configuration[1, 1, 0])[1] == configuration[1, 1, 0][1]


def run_restricted_case(name, base, kind, L1, L2, D, cut, tensor_seed, chain_seeds, n_therm, n_samples):
    """The lattice of case ``base`` sampled with custom hopping Hamiltonians (the spin-flip part of every
    bond's term, no diagonal proposals) and a restricted subspace (``center_fixed``) in both SweepSampling
    and Observer (sampling.py:81-91, 117-143; observer.py:224-233, 364-367); saves per chain and sweep the
    configuration and possibility, per sample ws and E_loc, the energy and the gradient to
    <name>.npz."""
    lattice = build_lattice(kind, L1, L2, D, tensor_seed)
    hopping = {}
    for positions, H in lattice._hamiltonians.items():
        Hf = H.copy()
        for a in range(2):
            Hf[{"I0": a, "I1": a, "O0": a, "O1": a}] = 0
            Hf[{"I0": a, "I1": 1 - a, "O0": a, "O1": 1 - a}] = 0
        hopping[positions] = Hf
    neel = np.zeros((L1, L2, 1), dtype=np.int64)
    for l1 in range(L1):
        for l2 in range(L2):
            neel[l1, l2, 0] = (l1 + l2) % 2
    observer = tet.Observer(lattice, enable_energy=True, enable_gradient=True, restrict_subspace=center_fixed)
    confs, poss, ws_list, eloc_list = [], [], [], []
    with observer:
        for seed in chain_seeds:
            TAT.random.seed(seed)
            sampling = tet.SweepSampling(lattice, cut, center_fixed, hopping)
            sampling.configuration.import_configuration(neel)
            c_confs, c_poss, c_ws, c_eloc = [], [], [], []
            for step in range(n_therm + n_samples):
                possibility, configuration = sampling()
                c_confs.append(configuration.export_configuration()[:, :, 0].copy())
                c_poss.append(possibility)
                if step >= n_therm:
                    before = observer._whole_result_reweight["energy"]
                    observer(possibility, configuration)
                    ws = float(configuration.hole(()).storage[0])
                    c_ws.append(ws)
                    c_eloc.append((observer._whole_result_reweight["energy"] - before) / (ws * ws / possibility))
            confs.append(c_confs)
            poss.append(c_poss)
            ws_list.append(c_ws)
            eloc_list.append(c_eloc)
    out = {"confs": np.array(confs, dtype=np.int64), "possibility": np.array(poss), "ws": np.array(ws_list),
           "eloc": np.array(eloc_list), "energy": np.array(observer.energy)}
    grad = observer.gradient
    for l1 in range(L1):
        for l2 in range(L2):
            out[f"grad_{l1}_{l2}"] = dense_site(grad[l1][l2])
    meta = {"name": name, "base": base, "cut": cut, "chain_seeds": chain_seeds, "n_therm": n_therm,
            "n_samples": n_samples, "L1": L1, "L2": L2}
    out["meta"] = np.array(json.dumps(meta))
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **out)
    print(f"{name}: E/site = {observer.energy[0]:.12f}, saved {os.path.getsize(path)} bytes")


def run_natural_case(name, kind, L1, L2, D, cut, tensor_seed, chain_seeds, n_therm, n_samples, runs):
    """The chains of case `name` again, observed with enable_natural_gradient; saves the reference's
    natural_gradient_by_conjugate_gradient(step, error) (observer.py:576-675) for every (step, error)
    in `runs` to <name>_natgrad.npz."""
    lattice = build_lattice(kind, L1, L2, D, tensor_seed)
    neel = np.zeros((L1, L2, 1), dtype=np.int64)
    for l1 in range(L1):
        for l2 in range(L2):
            neel[l1, l2, 0] = (l1 + l2) % 2
    out = {"runs": np.array(runs, dtype=np.float64)}
    # the reference releases its per-sample deltas after one natural-gradient call: one observed run
    # of the (deterministic) chains per (step, error) setting
    for k, (steps, error) in enumerate(runs):
        observer = tet.Observer(lattice, enable_energy=True, enable_gradient=True, enable_natural_gradient=True)
        with observer:
            for seed in chain_seeds:
                TAT.random.seed(seed)
                sampling = tet.SweepSampling(lattice, cut, None, None)
                sampling.configuration.import_configuration(neel)
                for step in range(n_therm + n_samples):
                    possibility, configuration = sampling()
                    if step >= n_therm:
                        observer(possibility, configuration)
        grad = observer.natural_gradient_by_conjugate_gradient(int(steps), float(error))
        for l1 in range(L1):
            for l2 in range(L2):
                out[f"natgrad{k}_{l1}_{l2}"] = dense_site(grad[l1][l2])
    path = os.path.join(HERE, f"{name}_natgrad.npz")
    np.savez_compressed(path, **out)
    print(f"{name}: natural gradient for {len(runs)} (step, error) settings, saved {os.path.getsize(path)} bytes")


def run_checkpoint_case(name, kind, L1, L2, D, tensor_seed):
    """The lattice of case `name` pickled by the reference (as gm_save does, utility.py:219-224) to
    <name>_lattice.pkl: a checkpoint file for tests/test_checkpoint.py."""
    import pickle
    lattice = build_lattice(kind, L1, L2, D, tensor_seed)
    path = os.path.join(HERE, f"{name}_lattice.pkl")
    with open(path, "wb") as f:
        pickle.dump(lattice, f)
    print(f"{name}: lattice file saved {os.path.getsize(path)} bytes")


def run_direct_case(name, kind, L1, L2, D, tensor_seed, cut, double_cut, runs):
    """The reference's DirectSampling (tetragono/tetragono/sampling_lattice/sampling.py:252-371) on the
    lattice of case ``name`` with cuts large enough to be exact; ``runs`` = [(seed, alpha, n_samples)].
    Saves per run the sampled configurations and possibilities to <name>_direct.npz."""
    lattice = build_lattice(kind, L1, L2, D, tensor_seed)
    out = {"runs": np.array(runs, dtype=np.float64), "cuts": np.array([cut, double_cut])}
    for k, (seed, alpha, n) in enumerate(runs):
        lattice.attribute["alpha"] = alpha
        TAT.random.seed(int(seed))
        sampling = tet.DirectSampling(lattice, cut, None, double_cut)
        confs, poss = [], []
        for _ in range(int(n)):
            p, conf = sampling()
            confs.append(conf.export_configuration()[:, :, 0].copy())
            poss.append(p)
        out[f"confs{k}"] = np.array(confs, dtype=np.int64)
        out[f"possibility{k}"] = np.array(poss)
    path = os.path.join(HERE, f"{name}_direct.npz")
    np.savez_compressed(path, **out)
    print(f"{name}: direct sampling, {len(runs)} runs, saved {os.path.getsize(path)} bytes")


def run_observe_case(name, kind, L1, L2, D, cut, tensor_seed, chain_seeds, n_therm, n_samples):
    """The chains of case ``name`` observed with an ``observer_set`` of long-range diagonal operators
    (Sz on single sites, SzSz on distant pairs; tetragono/tetragono/common_tensor/No.py) besides the
    energy; saves the reference's ``result`` / ``whole_result`` (observer.py:473-503) and the operators'
    element tables to <name>_observe.npz."""
    lattice = build_lattice(kind, L1, L2, D, tensor_seed)
    No = tet.common_tensor.No
    Sz, SzSz = No.Sz.to(float), No.SzSz.to(float)
    observer_set = {
        "SzSz": {((0, 0, 0), (2, 2, 0)): SzSz, ((0, 1, 0), (2, 1, 0)): SzSz, ((1, 0, 0), (1, 2, 0)): SzSz},
        "Sz": {((1, 1, 0),): Sz, ((0, 2, 0),): Sz},
    }
    neel = np.zeros((L1, L2, 1), dtype=np.int64)
    for l1 in range(L1):
        for l2 in range(L2):
            neel[l1, l2, 0] = (l1 + l2) % 2
    observer = tet.Observer(lattice, observer_set={k: dict(v) for k, v in observer_set.items()}, enable_energy=True)
    with observer:
        for seed in chain_seeds:
            TAT.random.seed(seed)
            sampling = tet.SweepSampling(lattice, cut, None, None)
            sampling.configuration.import_configuration(neel)
            for step in range(n_therm + n_samples):
                possibility, configuration = sampling()
                if step >= n_therm:
                    observer(possibility, configuration)
    phys = lattice.physics_edges[0, 0, 0]
    out, meta = {}, {"names": [], "positions": []}
    result, whole = observer.result, observer.whole_result
    k = 0
    for nm, terms in observer_set.items():
        for positions, H in terms.items():
            rows = []
            for s_in, outs in tensor_element(H).items():
                for s_out, value in outs.items():
                    rows.append([point_index(phys, p) for p in s_in] + [point_index(phys, p) for p in s_out] +
                                [float(value.storage[0])])
            out[f"table_{k}"] = np.array(rows)
            out[f"result_{k}"] = np.array(result[nm][positions])
            meta["names"].append(nm)
            meta["positions"].append([list(p) for p in positions])
            k += 1
        out[f"whole_{nm}"] = np.array(whole[nm])
    out["energy"] = np.array(observer.energy)
    out["meta"] = np.array(json.dumps(meta))
    path = os.path.join(HERE, f"{name}_observe.npz")
    np.savez_compressed(path, **out)
    print(f"{name}: observer set of {k} terms, saved {os.path.getsize(path)} bytes")


def run_offdiag_case(name, kind, L1, L2, D, cut, tensor_seed, chain_seeds, n_therm, n_samples):
    """The chains of case ``name`` observed with an ``observer_set`` of long-range operators with
    off-diagonal elements (Sx on one site, SxSx and SS = SxSx + SySy + SzSz on distant pairs;
    tetragono/tetragono/common_tensor/No.py), which the reference evaluates through its
    ConfigurationPool (``cache_configuration=True``, observer.py:325-331, 368-369; lattice.py:473-696);
    saves ``result`` / ``whole_result``, the operators' element tables and, per observed sample, the
    configuration and its weight to <name>_offdiag.npz."""
    lattice = build_lattice(kind, L1, L2, D, tensor_seed)
    No = tet.common_tensor.No
    Sx, SxSx, SS = No.Sx.to(float), No.SxSx.to(float), No.SS.to(float)
    observer_set = {
        "SxSx": {((0, 0, 0), (2, 2, 0)): SxSx, ((0, 1, 0), (2, 1, 0)): SxSx},
        "SS": {((1, 0, 0), (1, 2, 0)): SS, ((0, 0, 0), (1, 1, 0)): SS},
        "Sx": {((1, 1, 0),): Sx},
    }
    neel = np.zeros((L1, L2, 1), dtype=np.int64)
    for l1 in range(L1):
        for l2 in range(L2):
            neel[l1, l2, 0] = (l1 + l2) % 2
    observer = tet.Observer(lattice, observer_set={k: dict(v) for k, v in observer_set.items()}, enable_energy=True,
                            cache_configuration=True)
    phys = lattice.physics_edges[0, 0, 0]
    confs, weights = [], []
    with observer:
        for seed in chain_seeds:
            TAT.random.seed(seed)
            sampling = tet.SweepSampling(lattice, cut, None, None)
            sampling.configuration.import_configuration(neel)
            for step in range(n_therm + n_samples):
                possibility, configuration = sampling()
                if step >= n_therm:
                    observer(possibility, configuration)
                    ws = float(configuration.hole(()))
                    confs.append([[point_index(phys, configuration[l1, l2, 0]) for l2 in range(L2)]
                                  for l1 in range(L1)])
                    weights.append(ws * ws / possibility)
    out, meta = {"confs": np.array(confs), "weights": np.array(weights)}, {"names": [], "positions": []}
    result, whole = observer.result, observer.whole_result
    k = 0
    for nm, terms in observer_set.items():
        for positions, H in terms.items():
            rows = []
            for s_in, outs in tensor_element(H).items():
                for s_out, value in outs.items():
                    rows.append([point_index(phys, p) for p in s_in] + [point_index(phys, p) for p in s_out] +
                                [float(value.storage[0])])
            out[f"table_{k}"] = np.array(rows)
            out[f"result_{k}"] = np.array(result[nm][positions])
            meta["names"].append(nm)
            meta["positions"].append([list(p) for p in positions])
            k += 1
        out[f"whole_{nm}"] = np.array(whole[nm])
    out["energy"] = np.array(observer.energy)
    out["meta"] = np.array(json.dumps(meta))
    path = os.path.join(HERE, f"{name}_offdiag.npz")
    np.savez_compressed(path, **out)
    print(f"{name}: off-diagonal observer set of {k} terms, saved {os.path.getsize(path)} bytes")


def run_ergodic_case(name, kind, L1, L2, D, cut, tensor_seed):
    """The reference's ErgodicSampling (tetragono/tetragono/sampling_lattice/sampling.py:196-249) over every
    configuration of the lattice of case ``name`` with an energy Observer: the exact energy of the
    truncated-contraction PEPS (no sampling noise).  Saves it to <name>_ergodic.npz."""
    lattice = build_lattice(kind, L1, L2, D, tensor_seed)
    sampling = tet.ErgodicSampling(lattice, cut, None)
    observer = tet.Observer(lattice, enable_energy=True, enable_gradient=True)
    with observer:
        for _ in range(sampling.total_step):
            possibility, configuration = sampling()
            observer(possibility, configuration)
    out = {"energy": np.array(observer.energy), "total_energy": np.array(observer.total_energy),
           "total_steps": np.array(sampling.total_step), "cut": np.array(cut)}
    grad = observer.gradient
    for l1 in range(L1):
        for l2 in range(L2):
            out[f"grad_{l1}_{l2}"] = dense_site(grad[l1][l2])
    path = os.path.join(HERE, f"{name}_ergodic.npz")
    np.savez_compressed(path, **out)
    print(f"{name}: ergodic E/site = {observer.energy[0]:.12f}, saved {os.path.getsize(path)} bytes")


def _same_shapes(holes, L1, L2):
    return False


def _pack_holes(holes, L1, L2):
    return [[dense_site(holes[l1][l2]) for l2 in range(L2)] for l1 in range(L1)]


if __name__ == "__main__" and "--offdiag" in sys.argv:
    run_offdiag_case("heis_no_3x3_D3_dc4", "no", 3, 3, 3, 4, 1234, [11, 12], 3, 5)
    sys.exit(0)
if __name__ == "__main__" and "--restricted" in sys.argv:
    run_restricted_case("heis_no_3x3_D3_dc4_restricted", "heis_no_3x3_D3_dc4", "no", 3, 3, 3, 4, 1234, [11, 12], 3, 5)
    sys.exit(0)
if __name__ == "__main__" and "--workloads" in sys.argv:
    # the benchmark-size lattices: 8x8 Bose U(1) D=6 {-1:2, 0:2, +1:2} with Dcut 36, and 6x6 Bose U(1)
    # D=4 {-1:1, 0:2, +1:1} with Dcut 16 (a few chains and sweeps each: seconds per sample here)
    run_case("heis_u1_8x8_D222_dc36", "u1", 8, 8, (2, 2, 2), 36, 20260101, [101, 102], 2, 3, compact=True)
    run_case("heis_u1_6x6_D121_dc16", "u1", 6, 6, (1, 2, 1), 16, 20260102, [111, 112], 3, 4, compact=True)
    sys.exit(0)
if __name__ == "__main__" and "--direct-only" in sys.argv:
    run_direct_case("heis_no_3x3_D3_dc4", "no", 3, 3, 3, 1234, 64, 256, [(5, 1.0, 12), (6, 0.5, 12)])
    run_direct_case("heis_no_3x3_D3_dc4_trunc", "no", 3, 3, 3, 1234, 4, 6, [(5, 1.0, 12), (6, 0.5, 12)])
    run_direct_case("heis_no_3x3_D3_dc4_trunc2", "no", 3, 3, 3, 1234, 2, 4, [(7, 1.0, 12), (8, 0.5, 12)])
    run_observe_case("heis_no_3x3_D3_dc4", "no", 3, 3, 3, 4, 1234, [11, 12], 3, 5)
    run_ergodic_case("heis_no_3x3_D3_dc4", "no", 3, 3, 3, 4, 1234)
if __name__ == "__main__" and "--direct-only" in sys.argv:
    sys.exit(0)
if __name__ == "__main__" and "--natural-only" not in sys.argv and "--checkpoint-only" not in sys.argv:
    run_case("heis_no_3x3_D3_dc4", "no", 3, 3, 3, 4, 1234, [11, 12], 3, 5)
    run_case("heis_no_4x4_D4_dc16", "no", 4, 4, 4, 16, 2024, [21, 22], 4, 6)
    run_case("heis_no_4x4_D3_dc5", "no", 4, 4, 3, 5, 77, [31], 3, 5)
    run_case("heis_u1_4x4_D111_dc5", "u1", 4, 4, (1, 1, 1), 5, 4321, [41, 42], 3, 5)
    run_case("heis_u1_4x4_D222_dc8", "u1", 4, 4, (2, 2, 2), 8, 8765, [51], 2, 4)
if __name__ == "__main__" and "--checkpoint-only" in sys.argv:
    run_checkpoint_case("heis_no_3x3_D3_dc4", "no", 3, 3, 3, 1234)
    run_checkpoint_case("heis_u1_4x4_D111_dc5", "u1", 4, 4, (1, 1, 1), 4321)
if __name__ == "__main__" and "--checkpoint-only" not in sys.argv:
    run_natural_case("heis_no_3x3_D3_dc4", "no", 3, 3, 3, 4, 1234, [11, 12], 3, 5, [(6, 0.0), (50, 1e-3)])
    run_natural_case("heis_u1_4x4_D111_dc5", "u1", 4, 4, (1, 1, 1), 5, 4321, [41, 42], 3, 5, [(6, 0.0), (50, 1e-3)])
