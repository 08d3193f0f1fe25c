"""What lower-precision tensor products do to the sampler's amplitudes and local energies.

TEST INFRASTRUCTURE / MEASUREMENT ONLY: this study runs the numpy oracle (oracle/peps_oracle.py) with its
contraction functions replaced by emulations of tensor-core product schemes, while every QR and SVD
stays in float64 (numpy / LAPACK), and compares with the float64 oracle on the same configurations.
It decides whether the boundary-MPS contractions may run as split products on tensor cores at the
throughput metric's error bar (|dE/site| <= 1e-6 against float64).

Schemes (every product of two operand slices is exact in float32; sums are float32 GEMMs, i.e.
float32 accumulation as in a tensor-core MMA):

* ``fp32``    operands rounded to float32, one float32 GEMM;
* ``tf32x3``  a = hi + lo with hi = TF32(a), lo = TF32(a - hi) (10 explicit mantissa bits each),
  hi*hi + hi*lo + lo*hi (Ootomo and Yokota, "Recovering single precision accuracy from Tensor Cores
  while surpassing the FP32 theoretical peak performance", IJHPCA 2022);
* ``bf16x3``  the same with BF16 slices (7 explicit mantissa bits);
* ``bf16x6``  three BF16 slices a = a0 + a1 + a2 and the six products a_i b_j with i + j <= 2
  (the float32-faithful BF16 split);
* ``fp64``    the oracle itself (reference values).

Run:  python -m oracle.precision_study [--configs N] [--schemes fp32,tf32x3,bf16x3,bf16x6]
on the 8x8 Heisenberg lattice with U(1) bonds {-1:2, 0:2, +1:2} (D = 6), Dcut 36, seeded as bench.py's
default workload; configurations are the states of float64 sweep chains from the Neel state.
"""
import argparse
import json
import time

import numpy as np

from . import peps_oracle as po

_F64_CONTRACT = po.contract
_F64_MATMUL = po.matmul
_F64_DOT = po.full_dot


def _round_bits(x32, drop):
    """float32 array rounded to nearest even after clearing its ``drop`` low mantissa bits."""
    b = np.ascontiguousarray(x32, dtype=np.float32).view(np.uint32).astype(np.uint64)
    half = np.uint64((1 << (drop - 1)) - 1)
    b = b + half + ((b >> np.uint64(drop)) & np.uint64(1))
    b = b & np.uint64((0xFFFFFFFF >> drop) << drop)
    return b.astype(np.uint32).view(np.float32)


def tf32(x):
    return _round_bits(np.asarray(x, dtype=np.float32), 13)


def bf16(x):
    return _round_bits(np.asarray(x, dtype=np.float32), 16)


def slices(a, rnd, k):
    """k slices of a (float64) in the format rnd, a ~ s0 + s1 + ... (each float32-representable)."""
    out, r = [], np.asarray(a, dtype=np.float64)
    for _ in range(k):
        s = rnd(r)
        out.append(s)
        r = r - s.astype(np.float64)
    return out


def make_scheme(name):
    """(contract, matmul) emulating ``name`` with float32 accumulation."""
    if name == "fp32":
        parts, pairs = (lambda a: [np.asarray(a, dtype=np.float32)]), [(0, 0)]
    elif name == "tf32x3":
        parts, pairs = (lambda a: slices(a, tf32, 2)), [(0, 0), (0, 1), (1, 0)]
    elif name == "bf16x3":
        parts, pairs = (lambda a: slices(a, bf16, 2)), [(0, 0), (0, 1), (1, 0)]
    elif name == "bf16x6":
        parts, pairs = (lambda a: slices(a, bf16, 3)), [(0, 0), (0, 1), (1, 0), (0, 2), (1, 1), (2, 0)]
    else:
        raise ValueError(name)

    def product(f, a, b, **kw):
        pa, pb = parts(a), parts(b)
        acc = None
        # smallest terms first, as a split-product kernel accumulates them
        for i, j in sorted(pairs, key=lambda ij: -(ij[0] + ij[1])):
            t = f(pa[i], pb[j], **kw)
            acc = t if acc is None else (acc + t).astype(np.float32)
        return acc.astype(np.float64)

    def contract(a, b, axes):
        return product(np.tensordot, a, b, axes=axes)

    def matmul(a, b):
        return product(np.matmul, a, b)

    def full_dot(a, b):
        return float(product(np.tensordot, a, b, axes=3))

    return contract, matmul, full_dot


def use(name):
    """Switch the oracle's contractions to scheme ``name`` ("fp64" restores float64)."""
    if name == "fp64":
        po.contract, po.matmul, po.full_dot = _F64_CONTRACT, _F64_MATMUL, _F64_DOT
    else:
        po.contract, po.matmul, po.full_dot = make_scheme(name)


def workload_peps():
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from tnsp_gb300.lattice import random_heisenberg
    lat = random_heisenberg(8, 8, 6, seed=20240601, scale=False, sectors=(2, 2, 2))
    A = [[lat[l1, l2] for l2 in range(8)] for l1 in range(8)]
    return po.DensePEPS(A, list(lat._hamiltonians.items()), 36, lat.charges), lat


def sample_configurations(peps, n, seed0=4242, sweeps=3):
    from tnsp_gb300.lattice import neel
    confs = []
    for k in range(n):
        ch = po.SweepChain(peps, neel(peps.L1, peps.L2), seed0 + k)
        for _ in range(sweeps):
            ch.sweep()
        confs.append(ch.conf.copy())
    return confs


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--configs", type=int, default=8)
    ap.add_argument("--schemes", default="fp32,tf32x3,bf16x3,bf16x6")
    args = ap.parse_args()
    peps, lat = workload_peps()
    use("fp64")
    t0 = time.time()
    confs = sample_configurations(peps, args.configs)
    ref = [po.observe(peps, c) for c in confs]
    sites = peps.L1 * peps.L2
    w = np.array([r[0] ** 2 for r in ref])
    e_ref = np.array([r[1] for r in ref])
    out = {"lattice": "8x8 U(1) D=6 {-1:2,0:2,+1:2}, Dcut 36", "configs": len(confs),
           "fp64_seconds": time.time() - t0, "schemes": {}}
    for name in args.schemes.split(","):
        use(name)
        t0 = time.time()
        got = [po.observe(peps, c) for c in confs]
        use("fp64")
        ws = np.array([g[0] for g in got])
        el = np.array([g[1] for g in got])
        ws_ref = np.array([r[0] for r in ref])
        # energy per site over the same configurations, each weighted as an exact-sampling estimator
        # would weight it in its own arithmetic: sum E_loc / n (the sampling weights cancel for samples
        # drawn from |psi|^2); both per-configuration E_loc and their mean are compared
        hole_err = max(
            float(np.abs(g[2][a][b] - r[2][a][b]).max() / max(np.abs(r[2][a][b]).max(), 1e-300))
            for g, r in zip(got, ref) for a in range(peps.L1) for b in range(peps.L2))
        out["schemes"][name] = {
            "psi_max_rel_err": float(np.max(np.abs(ws / ws_ref - 1))),
            "eloc_max_abs_err": float(np.max(np.abs(el - e_ref))),
            "eloc_max_rel_err": float(np.max(np.abs(el - e_ref) / np.maximum(np.abs(e_ref), 1e-300))),
            "energy_per_site_err": float(abs(el.mean() - e_ref.mean()) / sites),
            "hole_max_rel_err": hole_err,
            "seconds": time.time() - t0,
        }
        print(name, json.dumps(out["schemes"][name]), flush=True)
    out["eloc_range"] = [float(e_ref.min()), float(e_ref.max())]
    out["weights"] = w.tolist()
    print(json.dumps(out))


if __name__ == "__main__":
    main()
