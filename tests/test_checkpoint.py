"""Checkpoint files: the reference's lattice pickles and configuration files, read and written by
tnsp_gb300.checkpoint without the reference (fixtures written by the reference itself,
tests/golden/make_golden.py --checkpoint-only)."""
import os
import pickle
import sys

import numpy as np
import pytest

from golden_cases import GOLDEN, Golden

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASES = ["heis_no_3x3_D3_dc4", "heis_u1_4x4_D111_dc5"]


@pytest.mark.parametrize("name", CASES)
def test_reference_lattice_file_loads(name):
    from tnsp_gb300.checkpoint import load_lattice, to_sampling_lattice
    g = Golden(name)
    ref = load_lattice(os.path.join(GOLDEN, f"{name}_lattice.pkl"))
    assert ref.state["L1"] == g.L1 and ref.state["L2"] == g.L2 and ref.state["data_version"] == 6
    lat = to_sampling_lattice(ref)
    for l1 in range(g.L1):
        for l2 in range(g.L2):
            np.testing.assert_array_equal(lat[l1, l2], g.z[f"site_{l1}_{l2}_dense"])
    ref_terms = dict(g.terms())
    assert list(lat._hamiltonians.keys()) == list(ref_terms.keys())
    for pos, table in ref_terms.items():
        mine = lat._hamiltonians[pos]
        assert list(mine.keys()) == list(table.keys())
        for k in table:
            assert [o for o, _ in mine[k]] == [o for o, _ in table[k]]
            np.testing.assert_allclose([v for _, v in mine[k]], [v for _, v in table[k]], rtol=0, atol=1e-15)
    if "_u1_" in name:
        assert lat.charges is not None


@pytest.mark.parametrize("name", CASES)
def test_lattice_file_round_trip(name):
    """load -> new tensors -> save -> load gives the new tensors; the bytes of an unmodified file
    reproduce every tensor dump exactly."""
    import io
    from tnsp_gb300.checkpoint import load_lattice, save_lattice, set_tensors, to_sampling_lattice
    path = os.path.join(GOLDEN, f"{name}_lattice.pkl")
    ref = load_lattice(path)
    lat = to_sampling_lattice(ref)
    new = [[2.0 * lat[l1, l2] for l2 in range(lat.L2)] for l1 in range(lat.L1)]
    for l1 in range(lat.L1):
        for l2 in range(lat.L2):
            lat[l1, l2] = new[l1][l2]
    set_tensors(ref, lat)
    buf = io.BytesIO()
    save_lattice(ref, buf)
    buf.seek(0)
    back = to_sampling_lattice(load_lattice(buf))
    for l1 in range(lat.L1):
        for l2 in range(lat.L2):
            np.testing.assert_array_equal(back[l1, l2], new[l1][l2])


def test_set_tensors_rejects_entries_outside_the_blocks():
    from tnsp_gb300.checkpoint import load_lattice, set_tensors, to_sampling_lattice
    ref = load_lattice(os.path.join(GOLDEN, "heis_u1_4x4_D111_dc5_lattice.pkl"))
    lat = to_sampling_lattice(ref)
    a = lat[1, 1].copy()
    zero = np.argwhere(a == 0)[0]
    a[tuple(zero)] = 1.0
    lat._tensors[1][1] = a
    with pytest.raises(ValueError):
        set_tensors(ref, lat)


def _reference_modules():
    """The reference's TAT / tetragono where this checkout has them: the reference tree named by
    TNSP_REFERENCE_ROOT and its CPU module built by oracle/build_ref.sh."""
    ref_dir = os.environ.get("TNSP_REFERENCE_ROOT", "")
    tat_dir = os.path.join(ROOT, "oracle", "_ref")
    if not (ref_dir and os.path.isdir(os.path.join(ref_dir, "tetragono")) and os.path.isdir(tat_dir)
            and any(f.startswith("TAT") and f.endswith(".so") for f in os.listdir(tat_dir))):
        pytest.skip("the reference is not available in this checkout")
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    saved = sys.argv
    sys.argv = [saved[0]]
    try:
        import make_golden  # noqa: F401  (mpi4py stand-in and paths)
    finally:
        sys.argv = saved
    import TAT
    import tetragono
    return TAT, tetragono


@pytest.mark.parametrize("name", CASES)
def test_saved_lattice_file_is_read_by_the_reference(name):
    import io
    from tnsp_gb300.checkpoint import load_lattice, save_lattice, set_tensors, to_sampling_lattice
    _reference_modules()
    import make_golden
    ref = load_lattice(os.path.join(GOLDEN, f"{name}_lattice.pkl"))
    lat = to_sampling_lattice(ref)
    for l1 in range(lat.L1):
        for l2 in range(lat.L2):
            lat[l1, l2] = -0.5 * lat[l1, l2]
    set_tensors(ref, lat)
    buf = io.BytesIO()
    save_lattice(ref, buf)
    theirs = pickle.loads(buf.getvalue())
    assert type(theirs).__name__ == "SamplingLattice"
    for l1 in range(lat.L1):
        for l2 in range(lat.L2):
            np.testing.assert_array_equal(make_golden.dense_site(theirs[l1, l2]), lat[l1, l2])


def test_configuration_file_round_trip(tmp_path):
    from tnsp_gb300.checkpoint import read_configurations, write_configurations
    rng = np.random.default_rng(3)
    conf = rng.integers(0, 2, size=(5, 3, 4, 1))
    path = str(tmp_path / "conf.dat")
    write_configurations(conf, path)
    raw = np.fromfile(path, dtype=np.int64)
    assert raw[:5].tolist() == [5, 3, 3, 4, 1]  # [blocks, rank, *shape] as utility.py:390-399 writes
    np.testing.assert_array_equal(read_configurations(path), conf)
