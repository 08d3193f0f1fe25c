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
