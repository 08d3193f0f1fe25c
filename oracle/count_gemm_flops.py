"""Algorithmic block-GEMM work per sample of the reference's sampling path, measured on the reference.

MEASUREMENT ONLY (runs the reference itself, in a checkout that has it; see oracle/build_ref.sh and
tests/golden/make_golden.py for the set-up): every ``Tensor.contract`` the reference calls during
``SweepSampling.__call__`` and ``Observer.__call__`` (energy + gradient) is counted as the block-sparse
GEMM it performs (TAT/include/TAT/implement/contract.hpp:306-620): with the common legs merged into one
index k and the free legs of each side into i and j, a pair (i, k, j) is a multiply-add when both
blocks exist, so the count is 2 * sum_k n_A(k) n_B(k) with n_A(k) the allowed free-index combinations
of A at k.  A block exists when the charges of its legs sum to zero (U(1); Fermi U(1) by its fermion
number), so n_A(k) is a histogram lookup.  Without symmetry this is 2 m k n.  QR and SVD are not
counted here (the sampler counts them per sector with the Golub-Van Loan operation counts).

    TNSP_REFERENCE_ROOT=<reference checkout> python -m oracle.count_gemm_flops <workload> [samples]

Workloads are the lattices bench.py measures, built here with the reference's own classes: heis8x8u1,
heis6x6u1d4, heis12x12u1, heis10x10u1 (Bose U(1) Heisenberg), tv8x8 (Fermi U(1) t-V), heis4x4 (no
symmetry).  Prints the GEMM flops per sample, split into sweep and observation.
"""
import collections
import itertools
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _charges(edge):
    out = []
    for sym, dim in edge.segments:
        q = getattr(sym, "u1", None)
        if q is None:
            q = getattr(sym, "fermi", 0)
        out += [int(q)] * int(dim)
    return np.array(out, dtype=np.int64)


def _hist(charge_lists):
    """Histogram {total charge: count} over the index combinations of several legs."""
    h = collections.Counter({0: 1})
    for q in charge_lists:
        vals = collections.Counter(q.tolist())
        nh = collections.Counter()
        for a, ca in h.items():
            for b, cb in vals.items():
                nh[a + b] += ca * cb
        h = nh
    return h


def contract_flops(a, b, pairs):
    """2 * multiply-adds of the block-sparse product a x b over the leg pairs (name_a, name_b)."""
    an = [str(n) for n in a.names]
    bn = [str(n) for n in b.names]
    ca = [str(x) for x, _ in pairs]
    cb = [str(y) for _, y in pairs]
    qa = {n: _charges(a.edge_by_name(n)) for n in an}
    qb = {n: _charges(b.edge_by_name(n)) for n in bn}
    free_a = _hist([qa[n] for n in an if n not in ca])
    free_b = _hist([qb[n] for n in bn if n not in cb])
    common = _hist([qa[n] for n in ca])   # charge of the common legs on a's side
    total = 0
    for c, nk in common.items():
        # a's blocks: free + common == 0; b's common legs carry the opposite charges
        total += nk * free_a.get(-c, 0) * free_b.get(c, 0)
    return 2.0 * total


class Counter:

    def __init__(self):
        self.flops = 0.0
        self.enabled = True

    def wrap(self, cls):
        orig = cls.contract
        counter = self

        def contract(a, b, pairs, *args, **kwargs):
            if counter.enabled:
                counter.flops += contract_flops(a, b, list(pairs))
            return orig(a, b, pairs, *args, **kwargs)

        cls.contract = contract


def main():
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    name = sys.argv[1] if len(sys.argv) > 1 else "heis8x8u1"
    samples = int(sys.argv[2]) if len(sys.argv) > 2 else 4
    saved = sys.argv
    sys.argv = [saved[0]]
    import make_golden  # noqa: F401  (mpi4py stand-in, the reference's paths)
    sys.argv = saved
    import TAT
    import tetragono as tet
    counter = Counter()
    for cls in (TAT.No.D.Tensor, TAT.BoseU1.D.Tensor, TAT.FermiU1.D.Tensor):
        counter.wrap(cls)
    heis = {"heis8x8u1": (8, 8, (2, 2, 2), 36), "heis6x6u1d4": (6, 6, (1, 2, 1), 16),
            "heis12x12u1": (12, 12, (2, 4, 2), 64), "heis10x10u1": (10, 10, (2, 2, 2), 36),
            "heis4x4": (4, 4, 4, 16)}
    if name in heis:
        L1, L2, D, cut = heis[name]
        lattice = make_golden.build_lattice("no" if name == "heis4x4" else "u1", L1, L2, D, 12345)
        if L1 * L2 > 100:
            # the 1/sqrt(2 D^z) scaling leaves a 12x12 amplitude below float64's range in the reference,
            # which carries no exponent on this path: scale the sites back up (the counts do not change)
            for l1, l2 in itertools.product(range(L1), range(L2)):
                lattice[l1, l2] = lattice[l1, l2] * 10.0
        start = np.fromfunction(lambda a, b: (a + b) % 2, (L1, L2)).astype(np.int64)[:, :, None]
    elif name == "tv8x8":
        import make_fermi_golden  # noqa: F401
        from tetraku.models import tV
        L1 = L2 = 8
        cut, T = 64, 32
        state = tV.abstract_lattice(L1, L2, 2, T, 1.0, 1.0)
        for l1 in range(L1 - 1):
            Q = int(T * (L1 - l1 - 1) / L1)
            state.virtual_bond[l1, 0, "D"] = [(Q - 1, 2), (Q, 4), (Q + 1, 2)]
            for l2 in range(1, L2):
                state.virtual_bond[l1, l2, "D"] = [(-1, 2), (0, 4), (1, 2)]
        for l1 in range(L1):
            for l2 in range(L2 - 1):
                Q = int(T / L1 * (L2 - l2 - 1) / L2)
                state.virtual_bond[l1, l2, "R"] = [(Q - 1, 2), (Q, 4), (Q + 1, 2)]
        TAT.random.seed(12345)
        lattice = tet.SamplingLattice(state)
        for l1, l2 in itertools.product(range(L1), range(L2)):
            t = lattice[l1, l2]
            z = sum(1 for n in t.names if str(n) in ("U", "D", "L", "R"))
            lattice[l1, l2] = t * (1.0 / np.sqrt(2.0 * 8**z))
        rng = np.random.default_rng(5)
        probe = tet.SweepSampling(lattice, cut, None, None)
        while True:
            occ = np.zeros(L1 * L2, dtype=np.int64)
            occ[rng.choice(L1 * L2, size=T, replace=False)] = 1
            start = occ.reshape(L1, L2, 1)
            probe.configuration.import_configuration(start)
            if probe.configuration.hole(()).norm_max() != 0:
                break
    else:
        raise SystemExit(f"unknown workload {name}")
    TAT.random.seed(777)
    sampling = tet.SweepSampling(lattice, cut, None, None)
    sampling.configuration.import_configuration(start)
    counter.enabled = False
    sampling()  # one sweep of thermalisation, not counted
    observer = tet.Observer(lattice, enable_energy=True, enable_gradient=True)
    sweep, obs = 0.0, 0.0
    with observer:
        for _ in range(samples):
            counter.enabled, counter.flops = True, 0.0
            possibility, configuration = sampling()
            sweep += counter.flops
            counter.flops = 0.0
            observer(possibility, configuration)
            obs += counter.flops
            counter.enabled = False
    print(f"{name}: {samples} samples; GEMM flops per sample {(sweep + obs) / samples:.4e} "
          f"(sweep {sweep / samples:.4e}, observation {obs / samples:.4e})")


if __name__ == "__main__":
    main()
