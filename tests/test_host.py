"""Host-side logic (no GPU): block-storage import, element tables, the C-ABI export list."""
import os
import re

import numpy as np
import pytest

from golden_cases import CASES, Golden
from tnsp_gb300.lattice import (block_to_dense, element_table, heisenberg_table, random_heisenberg, site_from_blocks)

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("name", CASES)
def test_block_storage_import_matches_reference_dense(name):
    """Symmetry-block indexing: the reference's raw storage, converted by the planner, equals the
    dense tensor the reference's own clear_symmetry produces, bit for bit."""
    g = Golden(name)
    for l1 in range(g.L1):
        for l2 in range(g.L2):
            meta = g.meta["sites"][f"{l1},{l2}"]
            names = [m["name"] for m in meta]
            edges = [[tuple(s) for s in m["segments"]] for m in meta]
            dense = site_from_blocks(g.z[f"site_{l1}_{l2}_storage"], names, edges)
            np.testing.assert_array_equal(dense, g.z[f"site_{l1}_{l2}_dense"])


@pytest.mark.parametrize("name", CASES)
def test_element_tables_match_tensor_element(name):
    g = Golden(name)
    phys = [tuple(s) for s in g.meta["sites"]["0,0"][0]["segments"]]
    ref_terms = g.terms()
    for ti, t in enumerate(g.meta["terms"]):
        names = [e["name"] for e in t["edges"]]
        edges = [[tuple(s) for s in e["segments"]] for e in t["edges"]]
        mine = element_table(g.z[f"term_{ti}_storage"], names, edges, phys)
        ref = ref_terms[ti][1]
        assert list(mine.keys()) == list(ref.keys())
        for k in ref:
            assert [o for o, _ in mine[k]] == [o for o, _ in ref[k]]
            np.testing.assert_allclose([v for _, v in mine[k]], [v for _, v in ref[k]], rtol=0, atol=1e-15)


def test_heisenberg_table_matches_reference_order():
    g = Golden("heis_no_3x3_D3_dc4")
    ref = g.terms()[0][1]
    mine = heisenberg_table(1.0)
    assert list(mine.keys()) == list(ref.keys())
    for k in ref:
        assert [o for o, _ in mine[k]] == [o for o, _ in ref[k]]
        np.testing.assert_allclose([v for _, v in mine[k]], [v for _, v in ref[k]], atol=1e-15)


def test_block_to_dense_rejects_wrong_size():
    with pytest.raises(ValueError):
        block_to_dense(np.zeros(3), [[(0, 2)], [(0, 2)]])


def test_random_u1_lattice_conserves_charge():
    lat = random_heisenberg(4, 4, None, seed=3, sectors=(2, 2, 2))
    # every nonzero element satisfies P + D + R - U - L = 0 (bond charges -1,-1,0,0,+1,+1)
    q = np.array([-1, -1, 0, 0, 1, 1])
    for l1, l2 in lat.sites():
        t = lat[l1, l2]
        nz = np.argwhere(t != 0)
        for p, u, d, l, r in nz:
            pq = 1 if p == 0 else -1
            qu = -q[u] if t.shape[1] > 1 else 0
            qd = q[d] if t.shape[2] > 1 else 0
            ql = -q[l] if t.shape[3] > 1 else 0
            qr = q[r] if t.shape[4] > 1 else 0
            assert pq + qu + qd + ql + qr == 0


def test_header_declares_exactly_the_bound_symbols():
    from tnsp_gb300._lib import SIGNATURES
    header = open(os.path.join(ROOT, "include", "tnsp_gb300.h")).read()
    declared = set(re.findall(r"\b(tnsp_[a-z0-9_]+)\s*\(", header))
    assert declared == set(SIGNATURES)


def test_library_exports_every_declared_symbol():
    from tnsp_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("library not built in this checkout")
    lib = _lib.load()
    for name in _lib.SIGNATURES:
        assert hasattr(lib, name), name


@pytest.mark.parametrize("name", CASES)
def test_site_charges_conserve_on_reference_tensors(name):
    """The charges derived from the reference's edges make every nonzero element conserve charge."""
    from tnsp_gb300.lattice import site_charges
    g = Golden(name)
    for l1 in range(g.L1):
        for l2 in range(g.L2):
            meta = g.meta["sites"][f"{l1},{l2}"]
            legs, phys, flux = site_charges([m["name"] for m in meta], [[tuple(x) for x in m["segments"]] for m in meta])
            t = g.z[f"site_{l1}_{l2}_dense"]
            for p, u, d, l, r in np.argwhere(t != 0):
                assert phys[p] + legs["U"][u] + legs["D"][d] + legs["L"][l] + legs["R"][r] == flux


def test_precision_names_match_the_header():
    """Python precision names map to the header's TNSP_FP64 / TNSP_FP32 / TNSP_DD values."""
    from tnsp_gb300._lib import PRECISIONS
    header = open(os.path.join(ROOT, "include", "tnsp_gb300.h")).read()
    values = {k: int(v) for k, v in re.findall(r"#define (TNSP_(?:FP64|FP32|DD|MIXED)) (\d+)", header)}
    assert PRECISIONS == {"fp64": values["TNSP_FP64"], "fp32": values["TNSP_FP32"], "dd": values["TNSP_DD"],
                          "mixed": values["TNSP_MIXED"]}


def test_sweep_sampling_rejects_unknown_precision_before_the_device():
    from tnsp_gb300.lattice import random_heisenberg
    from tnsp_gb300.sampling import SweepSampling
    lat = random_heisenberg(2, 2, 2, seed=1)
    with pytest.raises(ValueError):
        SweepSampling(lat, 4, precision="fp16")
