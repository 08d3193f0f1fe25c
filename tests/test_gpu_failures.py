"""Failure detection through the C ABI: invalid inputs become error codes on the host, before any
device work; nothing here faults, traps or hangs the GPU."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture()
def lattice():
    from tnsp_gb300.lattice import random_heisenberg
    return random_heisenberg(3, 3, None, seed=5, sectors=(1, 1, 1))


def test_non_finite_tensor_rejected(lattice):
    from tnsp_gb300.engine import Sampler, TnspError
    bad = lattice[1, 1].copy()
    bad.flat[0] = np.nan
    lattice._tensors[1][1] = bad
    with pytest.raises(TnspError, match="non-finite"):
        Sampler(lattice, 4)


def test_charge_violation_rejected(lattice):
    from tnsp_gb300.engine import Sampler, TnspError
    t = lattice[1, 1].copy()
    zero = np.argwhere(t == 0)[0]
    t[tuple(zero)] = 1.0  # an element outside the allowed blocks
    lattice._tensors[1][1] = t
    with pytest.raises(TnspError, match="charge conservation"):
        Sampler(lattice, 4)


def test_configuration_out_of_range_rejected(lattice):
    from tnsp_gb300.engine import Sampler, TnspError
    s = Sampler(lattice, 4)
    conf = np.zeros((3, 3), dtype=np.int32)
    conf[0, 0] = 5
    with pytest.raises(TnspError, match="out of range"):
        s.init_chains(conf, np.array([1], dtype=np.uint64))


def test_calls_out_of_order_rejected():
    from tnsp_gb300 import _lib
    lib = _lib.load()
    ctx = ctypes.c_void_p()
    assert lib.tnsp_ctx_create(ctypes.byref(ctx), 0, None) == 0
    assert lib.tnsp_sweep(ctx, 1, 0) == -3  # TNSP_E_STATE: no chains
    assert b"no chains" in lib.tnsp_last_error(ctx)
    assert lib.tnsp_ctx_destroy(ctx) == 0


def test_non_nearest_neighbour_term_rejected(lattice):
    from tnsp_gb300.engine import Sampler, TnspError
    from tnsp_gb300.lattice import heisenberg_table
    lattice._hamiltonians[((0, 0, 0), (2, 2, 0))] = heisenberg_table()
    with pytest.raises(TnspError, match="nearest-neighbour"):
        Sampler(lattice, 4)


def test_zero_amplitude_is_recorded_not_fatal():
    """A configuration outside the charge sector has psi = 0 exactly: the sampler follows IEEE
    semantics like the reference (p = inf accepts, 0/0 rejects) and records it in the status word."""
    from tnsp_gb300.engine import Sampler
    from tnsp_gb300.lattice import random_heisenberg
    lat = random_heisenberg(2, 2, None, seed=3, sectors=(1, 1, 1))
    s = Sampler(lat, 4)
    conf = np.zeros((2, 2), dtype=np.int32)  # all up: total charge 4, not 0
    s.init_chains(conf, np.array([7], dtype=np.uint64))
    m, e = s.amplitude(conf[None])
    assert m[0] == 0.0
    s.sweep(1)
    assert s.status() & 8  # TNSP_ST_ZERO_WS


def test_double_float_refused_for_uncharged_block_sparse_tensors():
    """Block-sparse tensors passed densely without their charges lose precision in double-float
    (rank-deficient boundaries): the library refuses the combination instead of returning wrong
    values, and accepts the same tensors with the charges declared, or in float64."""
    from golden_cases import Golden
    from test_gpu_parity import make_lattice
    from tnsp_gb300.engine import Sampler, TnspError
    g = Golden("heis_u1_4x4_D111_dc5")
    seeds = np.array(g.meta["chain_seeds"], dtype=np.uint64)
    s = Sampler(make_lattice(g, charged=False), g.cut)
    with pytest.raises(TnspError, match="double-float needs the charges"):
        s.init_chains(g.neel(), seeds, precision="dd")
    s.init_chains(g.neel(), seeds, precision="fp64")
    Sampler(make_lattice(g, charged=True), g.cut).init_chains(g.neel(), seeds, precision="dd")


@pytest.mark.parametrize("precision", ["fp64", "dd"])
def test_jacobi_sweep_limit_reports_a_device_failure(precision):
    """A one-sided Jacobi SVD that does not converge within its sweep limit (here set to 1) sets
    TNSP_ST_SVD_NOCONV, and the sweep returns TNSP_E_DEVICE with the status in its message, as the
    reference raises on a LAPACK failure (TAT/include/TAT/implement/svd.hpp:114-122); the loop ends at
    the limit, the context stays usable and the default limit gives the reference's chains again."""
    from golden_cases import Golden
    from test_gpu_parity import make_lattice
    from tnsp_gb300 import _lib
    from tnsp_gb300.engine import Sampler, TnspError
    g = Golden("heis_no_4x4_D4_dc16")
    seeds = np.array(g.meta["chain_seeds"], dtype=np.uint64)
    s = Sampler(make_lattice(g), g.cut)
    s.set_option(_lib.TNSP_OPT_JACOBI_SWEEPS, 1)
    s.init_chains(g.neel(), seeds, precision=precision)
    with pytest.raises(TnspError, match=r"\(-4\).*device status 0x"):
        s.sweep(1)
    assert s.status() & 1  # TNSP_ST_SVD_NOCONV (read and cleared)
    with pytest.raises(TnspError, match="out of range"):
        s.set_option(_lib.TNSP_OPT_JACOBI_SWEEPS, 0)
    s.set_option(_lib.TNSP_OPT_JACOBI_SWEEPS, 60)
    s.init_chains(g.neel(), seeds, precision=precision)
    s.sweep(1)
    conf, _ = s.read_chains()
    for b in range(len(seeds)):
        np.testing.assert_array_equal(conf[b], g.z["confs"][b][0])
    assert s.status() == 0
