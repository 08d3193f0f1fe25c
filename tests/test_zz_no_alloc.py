"""tnsp_amplitude_noalloc: the allocation-free amplitude entry point, for callers that must not
allocate device memory once running (a host whose device memory is all reserved by its own pool or
caching allocator, or a latency-bound host where cudaMalloc may synchronise the device).  Its output is
checked against the regular entry point tnsp_amplitude, on two calls in a row with different
lattices, so the second call also shows that the shared scratch arena is reset between calls.

This file is collected last on purpose: if it fails, every other test has already run.
"""
import ctypes

import numpy as np
import pytest

from golden_cases import Golden

pytestmark = pytest.mark.gpu


def _regular(lat, cut, confs):
    from tnsp_gb300.engine import Sampler
    s = Sampler(lat, cut)
    m, e = s.amplitude(confs)
    s.close()
    return m * np.exp2(e.astype(np.float64))


def _noalloc(lat, cut, confs):
    import torch
    from tnsp_gb300 import _lib
    lib = _lib.load()
    dev = torch.device("cuda:0")
    # the test owns every device buffer; the entry point allocates none
    tensors = torch.from_numpy(lat.flat_tensors()).to(dev)
    conf = torch.from_numpy(np.ascontiguousarray(confs.reshape(confs.shape[0], -1), dtype=np.int32)).to(dev)
    B = conf.shape[0]
    mant = torch.zeros(B, dtype=torch.float64, device=dev)
    expo = torch.zeros(B, dtype=torch.int32, device=dev)
    dims = np.ascontiguousarray(lat.dims())
    stream = torch.cuda.current_stream(dev).cuda_stream
    rc = lib.tnsp_amplitude_noalloc(lat.L1, lat.L2, lat.P, _lib.ptr(dims, ctypes.c_int),
                                    ctypes.c_void_p(tensors.data_ptr()), cut, B, ctypes.c_void_p(conf.data_ptr()),
                                    ctypes.c_void_p(mant.data_ptr()), ctypes.c_void_p(expo.data_ptr()),
                                    ctypes.c_void_p(stream))
    assert rc == 0, f"tnsp_amplitude_noalloc returned {rc}"
    torch.cuda.synchronize(dev)
    return mant.cpu().numpy() * np.exp2(expo.cpu().numpy().astype(np.float64))


def _lattice(name):
    from tnsp_gb300.lattice import SamplingLattice
    g = Golden(name)
    dense = g.dense_sites()
    lat = SamplingLattice(g.L1, g.L2, dense[0][0].shape[0], dense, {pos: t for pos, t in g.terms()})
    return g, lat


def test_noalloc_amplitude_matches_regular_entry_point_twice():
    for name in ("heis_no_4x4_D4_dc16", "heis_u1_4x4_D222_dc8"):
        g, lat = _lattice(name)
        confs = g.z["confs"].reshape(-1, g.L1, g.L2)
        ref = _regular(lat, g.cut, confs)
        got = _noalloc(lat, g.cut, confs)
        np.testing.assert_allclose(got, ref, rtol=1e-10, atol=0)


def _too_large(L1, L2, D, cut):
    """Calls the entry point on a lattice/cut it must refuse before any device work (the device
    pointers are placeholders that a refused call never touches)."""
    from tnsp_gb300 import _lib
    from tnsp_gb300.lattice import random_heisenberg
    lib = _lib.load()
    lat = random_heisenberg(L1, L2, D, seed=1)
    dims = np.ascontiguousarray(lat.dims())
    rc = lib.tnsp_amplitude_noalloc(L1, L2, 2, _lib.ptr(dims, ctypes.c_int), ctypes.c_void_p(16), cut, 1,
                                    ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_void_p(16), None)
    return rc, lib.tnsp_last_error(None).decode()


def test_noalloc_rejects_a_bond_dimension_beyond_its_limit():
    rc, msg = _too_large(12, 12, 8, 256)   # cut * D = 2048 > 1024
    assert rc == -6, msg                   # TNSP_E_TOO_LARGE
    assert "1024" in msg


def test_noalloc_rejects_a_chain_slot_beyond_the_arena():
    rc, msg = _too_large(16, 16, 8, 128)   # cut * D = 1024 is allowed, but one chain slot exceeds 64 MiB
    assert rc == -6, msg
    assert "64 MiB" in msg
