"""Fermionic t-V lattices on the GPU (tnsp_lattice_fermion: sign-folded slices, prefix parities, E_loc
term signs, odd-prefix hole signs, gradient folding) against the reference's own outputs
(tests/golden/tv_*.npz, made by tests/golden/make_fermi_golden.py from tetraku's t-V plugin,
tetraku/tetraku/models/tV/__init__.py:23-76).

Per case and precision: the sampled configuration of every observed sweep is bit-exact, and the
sampling weight, |ws|, the signed amplitude (in the reference's leg order), E_loc, the energy and
the gradient (converted back to the reference's block storage) agree within the tolerances used for
the bosonic golden cases.  The cases cover an exact cut (3x3), truncating cuts (4x4 cut 2, 3x4 with an
odd particle number cut 3), odd charges on the interior D bonds (4x4 cut 3: the 8x8 workload's
bond layout, the only case where the row family's D-leg signs act) and the 8x8 workload's lattice
itself at cuts 24 and 64."""
import json
import os

import numpy as np
import pytest

from oracle import fermi_peps as fp
from oracle.fermi_tensor import FermiTensor
from test_fermion_host import GOLDEN, _golden, _host
from tnsp_gb300 import fermion as F

pytestmark = pytest.mark.gpu

CASES = ["3x3_D1_T4_dc16", "4x4_D2_T8_dc2", "3x4_D2_T5_dc3", "4x4_D1odd_T8_dc3",
         # the 8x8 fermionic workload's lattice (32 particles, {Q-1:2, Q:4, Q+1:2} flow bonds, {-1:2, 0:4, +1:2}
         # interior D bonds) at cut 24 and at its benchmark cut 64
         "8x8_D242_T32_dc24", "8x8_D242_T32_dc64"]
# float64: the reference's arithmetic up to summation order; double-float: 1e3 times wider (the
# rounding unit is 2^-46 and the truncated SVD amplifies it by the inverse gap at the cut)
TOL = {"fp64": dict(val=1e-10, energy=1e-12, grad=1e-10), "dd": dict(val=1e-7, energy=1e-9, grad=1e-7)}


def _case(name):
    z, meta, sites, mk = _golden(name)
    terms = {tuple(tuple(p) for p in t["positions"]): F.tv_element_table() for t in meta["terms"]}
    host = _host(sites, terms)
    return z, meta, mk, host


def _blocks_error(host, mk, descs, arrays, dense, a, b):
    """max |ours - reference| over the block storage of site (a, b) and the reference's max |element|."""
    mine = FermiTensor(host.names[a][b], host.edges[a][b]).set_storage(host.to_blocks(a, b, dense))
    ref = mk(descs[f"{a},{b}"], arrays)
    return np.abs(mine.transpose(ref.names).storage() - ref.storage()).max(), np.abs(ref.storage()).max()


# every case in both precisions, except the cut-64 lattice (about a minute per sweep of its chain: float64 only)
PARAMS = [(n, p) for n in CASES for p in ("fp64", "dd") if not (n.endswith("dc64") and p == "dd")]


@pytest.mark.parametrize("name,precision", PARAMS)
def test_fermionic_chains_match_reference(name, precision):
    from tnsp_gb300.engine import Sampler, estimators, gradient_from
    tol = TOL[precision]
    z, meta, mk, host = _case(name)
    lat = host.sampling_lattice()
    L1, L2 = meta["L1"], meta["L2"]
    seeds = np.array(meta["chain_seeds"], dtype=np.uint64)
    B, nt, ns = len(seeds), meta["n_therm"], meta["n_samples"]
    confs = z["confs"].reshape(B, ns, L1, L2)
    poss = z["possibility"].reshape(B, ns)
    ws = z["ws"].reshape(B, ns)
    eloc = z["eloc"].reshape(B, ns)
    s = Sampler(lat, meta["cut"])
    s.init_chains(np.array(meta["start"]), seeds, precision=precision)
    s.sweep(nt)
    s.reset_observer()
    canon = fp.canonical_names(L1, L2, fp.ROW)
    for k in range(ns):
        s.sweep(1, observe=True)
        conf, logp = s.read_chains()
        e, logws, _ = s.read_samples(1)
        for b in range(B):
            np.testing.assert_array_equal(conf[b], confs[b, k], err_msg=f"chain {b} sample {k}")
            assert abs(logp[b] - np.log(poss[b, k])) < tol["val"]
            assert abs(logws[0][b] - np.log(abs(ws[b, k]))) < tol["val"]
            assert abs(e[0][b] - eloc[b, k]) < tol["val"] * max(1.0, abs(eloc[b, k]))
        # the signed amplitude of the sampled configurations, in the reference's leg order
        m, x = s.amplitude(conf)
        for b in range(B):
            sign = fp.order_sign_by_count(conf[b], canon, meta["ws_names"][b * ns + k], host.T_charge)
            got = m[b] * np.exp2(float(x[b])) * sign
            assert abs(got / ws[b, k] - 1.0) < tol["val"], (b, k)
    scalars, delta, edelta = s.read_observer()
    assert scalars[0] == B * ns
    energy, err = estimators(scalars, lat.site_number)
    assert abs(energy - z["energy"][0]) < tol["energy"]
    if B * ns > 1:  # one sample's error bar is the square root of a rounding residual (0 here, 4e-9 there)
        assert abs(err - z["energy"][1]) < tol["val"]
    grad = lat.unflatten(host.fold_flat(gradient_from(scalars, delta, edelta)))
    errs, scale = [], 0.0
    for a in range(L1):
        for b in range(L2):
            d, mx = _blocks_error(host, mk, meta["gradient"], z[f"grad_{a}_{b}"], grad[a][b], a, b)
            errs.append(d)
            scale = max(scale, mx)
    assert max(errs) <= tol["grad"] * max(1.0, scale)
    assert s.status() == 0


@pytest.mark.parametrize("precision", ["fp64", "dd"])
def test_fermionic_natural_gradient_matches_reference(precision):
    """The drop-in SweepSampling / Observer on the 4x4 t-V lattice with cut 2: the reference's conjugate-
    gradient natural gradient (fixed step count, and the error-based stop) from the device-kept,
    prefix-signed hole rows, folded into the reference's block storage."""
    from tnsp_gb300.sampling import Observer, SweepSampling
    name = "4x4_D2_T8_dc2"
    z, meta, mk, host = _case(name)
    ng = np.load(os.path.join(GOLDEN, f"tv_{name}_natgrad.npz"))
    ng_meta = json.loads(bytes(ng["meta"]).decode())
    lat = host.sampling_lattice()
    seeds = meta["chain_seeds"]
    chains = len(seeds)
    sampling = SweepSampling(lat, meta["cut"], None, None, chains=chains, seeds=seeds, precision=precision)
    sampling.configuration.import_configuration(np.array(meta["start"])[:, :, None])
    for _ in range(meta["n_therm"] * chains):
        sampling()
    observer = Observer(lat, enable_energy=True, enable_gradient=True, enable_natural_gradient=True)
    with observer:
        for _ in range(meta["n_samples"] * chains):
            possibility, configuration = sampling()
            observer(possibility, configuration)
    assert abs(observer.energy[0] - z["energy"][0]) < TOL[precision]["energy"]
    bound = 1e-8 if precision == "fp64" else 1e-6
    for k, (steps, error) in enumerate(ng["runs"]):
        grad = observer.natural_gradient_by_conjugate_gradient(int(steps), float(error))
        errs, scale = [], 0.0
        for a in range(meta["L1"]):
            for b in range(meta["L2"]):
                d, mx = _blocks_error(host, mk, ng_meta, ng[f"natgrad{k}_{a}_{b}"], grad[a][b], a, b)
                errs.append(d)
                scale = max(scale, mx)
        assert max(errs) <= bound * scale, (k, max(errs), scale)
