"""Python handle on the C-ABI sampler (include/tnsp_gb300.h)."""
import ctypes

import numpy as np

from . import _lib
from ._lib import PRECISIONS, TNSP_DD, TNSP_FP32, TNSP_FP64, TNSP_MIXED, ptr

LN2 = 0.6931471805599453


class TnspError(RuntimeError):
    pass


class Sampler:
    """B independent sweep-sampling chains of one PEPS on one GPU.

    One chain here is one reference process running ``SweepSampling`` with its own seeded
    ``TAT.random`` engine; all chains advance together on the device.
    """

    def __init__(self, lattice, cut_dimension, device=0, stream=None):
        self.lib = _lib.load()
        self.ctx = ctypes.c_void_p()
        self._check(self.lib.tnsp_ctx_create(ctypes.byref(self.ctx), device, stream), "tnsp_ctx_create")
        self.lattice = lattice
        self.cut = cut_dimension
        self.B = 0
        self.precision = TNSP_FP64
        self._uploaded_version = None
        self._static_uploaded = False
        self.upload()

    def _check(self, code, what):
        if code != 0:
            msg = self.lib.tnsp_last_error(self.ctx).decode() if self.ctx else ""
            raise TnspError(f"{what} failed ({code}): {msg}")

    def close(self):
        if self.ctx:
            self.lib.tnsp_ctx_destroy(self.ctx)
            self.ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---------------------------------------------------------------------------------------
    def upload(self):
        """Uploads the site tensors (and their charges, which the library checks them against); the
        Hamiltonian tables, which a gradient step does not change, only on the first call."""
        lat = self.lattice
        dims = np.ascontiguousarray(lat.dims())
        flat = np.ascontiguousarray(lat.flat_tensors())
        self._check(
            self.lib.tnsp_lattice_upload(self.ctx, lat.L1, lat.L2, lat.P, ptr(dims, ctypes.c_int),
                                         ptr(flat, ctypes.c_double), self.cut), "tnsp_lattice_upload")
        ch = lat.charge_arrays()
        if ch is not None:
            q, qp, fl = ch
            self._check(
                self.lib.tnsp_lattice_charges(self.ctx, ptr(q, ctypes.c_int), ptr(qp, ctypes.c_int),
                                              ptr(fl, ctypes.c_int)), "tnsp_lattice_charges")
        fermion = getattr(lat, "fermion", None)
        if fermion is not None:
            # a fermionic lattice (tnsp_gb300.fermion): the current tensors as sign-folded slices
            slices = np.ascontiguousarray(
                fermion.slices_flat([[lat[l1, l2] for l2 in range(lat.L2)] for l1 in range(lat.L1)]))
            self._check(self.lib.tnsp_lattice_fermion(self.ctx, ptr(slices, ctypes.c_double), fermion.T_charge),
                        "tnsp_lattice_fermion")
        if not self._static_uploaded:
            n, sites, offs, cnts, outs, vals = lat.term_arrays()
            self._check(
                self.lib.tnsp_model_upload(self.ctx, n, ptr(sites, ctypes.c_int), ptr(offs, ctypes.c_int),
                                           ptr(cnts, ctypes.c_int), len(outs), ptr(outs, ctypes.c_int),
                                           ptr(vals, ctypes.c_double)), "tnsp_model_upload")
            self._static_uploaded = True
        self._uploaded_version = lat.version

    def set_option(self, option, value):
        """A context option (``_lib.TNSP_OPT_JACOBI_SWEEPS`` / ``_lib.TNSP_OPT_BLOCKS_PER_SM``)."""
        self._check(self.lib.tnsp_set_option(self.ctx, int(option), int(value)), "tnsp_set_option")

    def set_hopping(self, tables=None, allowed=None):
        """The sweep's proposal tables ({positions: element table}, as the lattice's Hamiltonians;
        None: the energy tables propose) and one 0/1 flag per entry of the proposal tables (None: every
        entry allowed); see tnsp_model_hopping."""
        from .lattice import table_arrays
        flags = None if allowed is None else np.ascontiguousarray(allowed, dtype=np.uint8)
        fptr = ptr(flags, ctypes.c_ubyte)
        if tables is None:
            self._check(self.lib.tnsp_model_hopping(self.ctx, 0, None, None, None, 0, None, fptr), "tnsp_model_hopping")
            return
        n, sites, offs, cnts, outs, _ = table_arrays(self.lattice.P, tables)
        if flags is not None and flags.size != outs.size:
            raise ValueError("one allow flag per proposal-table entry")
        self._check(self.lib.tnsp_model_hopping(self.ctx, n, ptr(sites, ctypes.c_int), ptr(offs, ctypes.c_int),
                                                ptr(cnts, ctypes.c_int), len(outs), ptr(outs, ctypes.c_int), fptr),
                    "tnsp_model_hopping")

    def restrict_energy(self, allowed=None):
        """One 0/1 flag per entry of the energy tables: E_loc terms of disallowed entries are skipped (None:
        all allowed); see tnsp_model_energy_restrict."""
        flags = None if allowed is None else np.ascontiguousarray(allowed, dtype=np.uint8)
        self._check(self.lib.tnsp_model_energy_restrict(self.ctx, ptr(flags, ctypes.c_ubyte)),
                    "tnsp_model_energy_restrict")
        self.energy_restricted = flags is not None

    def resident_chains(self):
        """Chains one launch advances at once (one resident thread block each)."""
        n = ctypes.c_int()
        self._check(self.lib.tnsp_resident_chains(self.ctx, ctypes.byref(n)), "tnsp_resident_chains")
        return n.value

    def init_chains(self, configs, seeds, discard=0, precision=TNSP_FP64):
        """``precision``: TNSP_FP64 / TNSP_FP32 / TNSP_DD / TNSP_MIXED or one of "fp64", "fp32", "dd", "mixed"."""
        if isinstance(precision, str):
            precision = PRECISIONS[precision]
        configs = np.ascontiguousarray(configs, dtype=np.int32)
        seeds = np.ascontiguousarray(seeds, dtype=np.uint64)
        B = seeds.shape[0]
        if configs.ndim == 2:
            configs = np.ascontiguousarray(np.broadcast_to(configs, (B,) + configs.shape))
        configs = configs.reshape(B, -1)
        self._check(
            self.lib.tnsp_chains_init(self.ctx, B, ptr(configs, ctypes.c_int32), ptr(seeds, ctypes.c_uint64), discard,
                                      precision), "tnsp_chains_init")
        self.B = B
        self.precision = precision

    def sweep(self, nsweeps=1, observe=False):
        if self._uploaded_version != self.lattice.version:
            raise TnspError("lattice changed since upload; call upload() and init_chains() again")
        self._check(self.lib.tnsp_sweep(self.ctx, nsweeps, 1 if observe else 0), "tnsp_sweep")

    @staticmethod
    def sweep_batch(samplers, nsweeps=1, observe=False):
        """``sweep`` of several samplers (different lattices; one device) as one CUDA graph launch in
        which their kernels run concurrently."""
        samplers = list(samplers)
        for s in samplers:
            if s._uploaded_version != s.lattice.version:
                raise TnspError("lattice changed since upload; call upload() and init_chains() again")
        arr = (ctypes.c_void_p * len(samplers))(*[s.ctx.value for s in samplers])
        code = samplers[0].lib.tnsp_sweep_batch(arr, len(samplers), nsweeps, 1 if observe else 0)
        samplers[0]._check(code, "tnsp_sweep_batch")

    def reset_observer(self):
        self._check(self.lib.tnsp_observer_reset(self.ctx), "tnsp_observer_reset")

    def read_observer(self, with_gradient=True):
        scalars = np.zeros(8)
        n = sum(self.lattice[l1, l2].size for l1, l2 in self.lattice.sites())
        delta = np.zeros(n) if with_gradient else None
        edelta = np.zeros(n) if with_gradient else None
        self._check(
            self.lib.tnsp_observer_read(self.ctx, ptr(scalars, ctypes.c_double), ptr(delta, ctypes.c_double),
                                        ptr(edelta, ctypes.c_double)), "tnsp_observer_read")
        return scalars, delta, edelta

    def keep_holes(self, enable=True):
        """Keep every observed sample's hole row on the device (for the natural gradient) until the
        next reset_observer; False releases them."""
        self._check(self.lib.tnsp_holes_keep(self.ctx, 1 if enable else 0), "tnsp_holes_keep")

    def holes_count(self):
        n = ctypes.c_int64()
        self._check(self.lib.tnsp_holes_count(self.ctx, ctypes.byref(n)), "tnsp_holes_count")
        return n.value

    def holes_gemv(self, x, transpose=False):
        """H x (x over the parameters) or H^T x (x over the kept samples), H = the kept hole rows."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        n_params = sum(self.lattice[l1, l2].size for l1, l2 in self.lattice.sites())
        y = np.zeros(n_params if transpose else self.holes_count())
        self._check(self.lib.tnsp_holes_gemv(self.ctx, 1 if transpose else 0, ptr(x, ctypes.c_double),
                                             ptr(y, ctypes.c_double)), "tnsp_holes_gemv")
        return y

    def holes_gram(self):
        """H H^T over the kept hole rows (rows x rows), one device product."""
        n = self.holes_count()
        g = np.zeros((n, n))
        self._check(self.lib.tnsp_holes_gram(self.ctx, ptr(g, ctypes.c_double)), "tnsp_holes_gram")
        return g

    def read_samples(self, nsweeps):
        eloc = np.zeros((nsweeps, self.B))
        logws = np.zeros((nsweeps, self.B))
        rw = np.zeros((nsweeps, self.B))
        self._check(
            self.lib.tnsp_samples_read(self.ctx, ptr(eloc, ctypes.c_double), ptr(logws, ctypes.c_double),
                                       ptr(rw, ctypes.c_double)), "tnsp_samples_read")
        return eloc, logws, rw

    def write_chains(self, configs):
        """Replaces every chain's configuration (random-number streams unchanged)."""
        configs = np.ascontiguousarray(configs, dtype=np.int32).reshape(self.B, -1)
        self._check(self.lib.tnsp_chains_write(self.ctx, ptr(configs, ctypes.c_int32)), "tnsp_chains_write")

    def read_chains(self):
        conf = np.zeros((self.B, self.lattice.L1, self.lattice.L2), dtype=np.int32)
        logp = np.zeros(self.B)
        self._check(self.lib.tnsp_chains_read(self.ctx, ptr(conf, ctypes.c_int32), ptr(logp, ctypes.c_double)),
                    "tnsp_chains_read")
        return conf, logp

    def amplitude(self, configs):
        configs = np.ascontiguousarray(configs, dtype=np.int32)
        B = configs.shape[0]
        m = np.zeros(B)
        e = np.zeros(B, dtype=np.int32)
        self._check(
            self.lib.tnsp_amplitude(self.ctx, B, ptr(configs.reshape(B, -1), ctypes.c_int32), ptr(m, ctypes.c_double),
                                    ptr(e, ctypes.c_int32)), "tnsp_amplitude")
        fermion = getattr(self.lattice, "fermion", None)
        if fermion is not None:
            # the graded amplitude in the row-major canonical leg order (T, P_0_0_0, P_0_1_0, ...)
            from .fermion import ROW, configuration_sign
            shape = (B, self.lattice.L1, self.lattice.L2)
            m = m * np.array([configuration_sign(c, fermion.p_T, ROW) for c in configs.reshape(shape)])
        return m, e

    def status(self):
        st = ctypes.c_int32()
        self._check(self.lib.tnsp_device_status(self.ctx, ctypes.byref(st)), "tnsp_device_status")
        return st.value

    PHASES = ("two_line", "sectors", "qr", "r_absorb", "jacobi", "svd_out", "us_absorb", "strip", "-", "observe",
              "-", "-")

    def counters(self, reset=True):
        """[contraction, QR, SVD, strip] flops then 12 phase cycle counters, since the last reset."""
        f = np.zeros(16)
        self._check(self.lib.tnsp_counters_read(self.ctx, ptr(f, ctypes.c_double), 1 if reset else 0),
                    "tnsp_counters_read")
        return f

    def last_timing(self):
        ms = ctypes.c_double()
        n = ctypes.c_int64()
        self._check(self.lib.tnsp_last_timing(self.ctx, ctypes.byref(ms), ctypes.byref(n)), "tnsp_last_timing")
        return ms.value, n.value


def estimators(scalars, site_number):
    """Energy per site and error bar from the reduced accumulators (observer.py:433-469, 528-540)."""
    count, R, RR, logws, ER, ERR, EERR, accepted = scalars
    if ER == 0.0 or R == 0.0:
        return 0.0, 0.0
    expect = ER / R
    variance = (EERR - 2 * ERR * expect + RR * expect**2) / R**2
    dev = variance**0.5 if variance >= 0 else 0.0
    return expect / site_number, dev / site_number


def gradient_from(scalars, delta, edelta):
    """``Observer.gradient`` (observer.py:542-555) for real tensors, flat layout."""
    R = scalars[1]
    energy = scalars[4] / R
    return 2.0 * (edelta / R - energy * delta / R)
