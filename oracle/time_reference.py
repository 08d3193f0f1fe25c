"""Seconds per sample of the reference's own CPU path against the oracle port, one thread each.

MEASUREMENT ONLY (runs the reference itself, in a checkout that has it; set-up as for
tests/golden/make_golden.py): one chain of the reference's ``SweepSampling`` + ``Observer`` (energy and
gradient) and one chain of the oracle (oracle/peps_oracle.py) on the same tensors (the 8x8 U(1) D=6
lattice built by the reference, Dcut 36), after one untimed sweep each; prints both rates and their
ratio, which converts the CPU baseline that bench.py times (the oracle port) into the reference's own
speed on the same cores.

    TNSP_REFERENCE_ROOT=<reference checkout> OMP_NUM_THREADS=1 OPENBLAS_NUM_THREADS=1 \\
        python -m oracle.time_reference [samples]
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def main():
    samples = int(sys.argv[1]) if len(sys.argv) > 1 else 6
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    saved = sys.argv
    sys.argv = [saved[0]]
    import make_golden
    sys.argv = saved
    import TAT
    import tetragono as tet
    from oracle.peps_oracle import DensePEPS, ObserverAccumulator, SweepChain
    from tnsp_gb300.lattice import SamplingLattice, heisenberg_table, nearest_neighbour_terms, neel, site_charges

    L, D, cut = 8, (2, 2, 2), 36
    ref = make_golden.build_lattice("u1", L, L, D, 20240601)
    dense, legs, flux, phys = [], [], [], None
    for l1 in range(L):
        drow, lrow, frow = [], [], []
        for l2 in range(L):
            t = ref[l1, l2]
            meta = make_golden.edge_meta(t)
            q, phys, f = site_charges([m["name"] for m in meta], [[tuple(x) for x in m["segments"]] for m in meta])
            drow.append(make_golden.dense_site(t))
            lrow.append(q)
            frow.append(f)
        dense.append(drow)
        legs.append(lrow)
        flux.append(frow)
    ours = SamplingLattice(L, L, 2, dense, nearest_neighbour_terms(L, L, heisenberg_table()), (legs, phys, flux))
    start = neel(L, L).astype(np.int64)[:, :, None]
    TAT.random.seed(99)
    sampling = tet.SweepSampling(ref, cut, None, None)
    sampling.configuration.import_configuration(start)
    sampling()
    observer = tet.Observer(ref, enable_energy=True, enable_gradient=True)
    t0 = time.perf_counter()
    with observer:
        for _ in range(samples):
            p, c = sampling()
            observer(p, c)
    t_ref = (time.perf_counter() - t0) / samples
    peps = DensePEPS([[ours[a, b] for b in range(L)] for a in range(L)], list(ours._hamiltonians.items()), cut,
                     ours.charges)
    chain = SweepChain(peps, neel(L, L), 99)
    acc = ObserverAccumulator(peps)
    chain.sweep()
    t0 = time.perf_counter()
    for _ in range(samples):
        p, c = chain.sweep()
        acc.add(p, c, chain.env)
    t_port = (time.perf_counter() - t0) / samples
    print(f"8x8 U(1) D=6 Dcut 36 (reference-built tensors), {samples} samples, one thread: reference "
          f"{t_ref:.3f} s/sample ({1 / t_ref:.3f} samples/s), oracle port {t_port:.3f} s/sample "
          f"({1 / t_port:.3f} samples/s), port / reference time {t_port / t_ref:.2f}")


if __name__ == "__main__":
    main()
