"""The reference's own ``gradient_descent`` driver on the GPU sampler.

``gradient_descent`` (tetragono/tetragono/sampling_lattice/gradient.py:93-445) builds an ``Observer`` and, per
gradient step, a ``SweepSampling`` on a reference ``SamplingLattice`` (TAT tensors), loops over the samples,
takes ``observer.gradient`` (or a natural gradient), applies it with ``state.apply_gradient`` and calls
``observer.normalize_lattice``.  ``run_gradient_descent`` runs that function unchanged with only those two
classes replaced by the adapters below, which keep the reference's interface and hand the work to the
drop-in classes of ``tnsp_gb300.sampling`` (and so to the GPU):

* ``ReferenceObserver`` converts the reference lattice to the dense form of ``tnsp_gb300.lattice`` when its
  context is entered (one conversion per gradient step: the tensors change between steps), and returns
  gradients as lattices of the reference's own tensors with the sites' edges, which ``apply_gradient``
  subtracts; ``normalize_lattice`` rescales the reference tensors;
* ``ReferenceSweepSampling`` samples that dense lattice with ``chains`` chains per launch, seeded from the
  driver's ``SeedDiffer`` (chain b: its seed + b, after the one discarded uniform draw of
  ``SeedDiffer.make_seed_diff``, utility.py:146-150), so one chain reproduces the reference's chain.

Bose U(1) and symmetry-free lattices with one orbit per site; the reference's TAT module must be
importable (this module uses it only to build gradient tensors, never to sample).
"""
import contextlib

import numpy as np

from . import sampling as _drop
from .checkpoint import dense_to_blocks
from .lattice import ORDER, SamplingLattice, element_table, site_charges, site_from_blocks

# chains per launch of the adapted SweepSampling (one reproduces the reference's single chain)
CHAINS = 1

_DENSE = {}  # id(reference lattice) -> the dense lattice of the current gradient step


def _segments(edge):
    return [(int(getattr(s, "u1", 0)), int(d)) for s, d in edge.segments]


def _names_edges(t):
    names = [str(n) for n in t.names]
    return names, [_segments(t.edge_by_name(n)) for n in names]


def dense_lattice(state):
    """The dense ``tnsp_gb300`` lattice (tensors, U(1) charges, Hamiltonian element tables) of a reference
    SamplingLattice."""
    if "Fermi" in type(state[0, 0]).__module__ + type(state[0, 0]).__name__:
        raise NotImplementedError("fermionic lattices: use tnsp_gb300.fermion.from_reference_lattice")
    L1, L2 = state.L1, state.L2
    tensors, legs, flux = [], [], []
    phys = None
    charged = False
    for l1 in range(L1):
        rt, rl, rf = [], [], []
        for l2 in range(L2):
            t = state[l1, l2]
            names, segs = _names_edges(t)
            rt.append(site_from_blocks(np.array(t.storage), names, segs))
            q, phys, f = site_charges(names, segs)
            charged |= any(c != 0 for s in segs for c, _ in s)
            rl.append(q)
            rf.append(f)
        tensors.append(rt)
        legs.append(rl)
        flux.append(rf)
    pseg = _segments(state.physics_edges[0, 0, 0])
    terms = {}
    for positions, H in state._hamiltonians.items():
        names, segs = _names_edges(H)
        terms[positions] = element_table(np.array(H.storage), names, segs, pseg)
    P = sum(d for _, d in pseg)
    return SamplingLattice(L1, L2, P, tensors, terms, (legs, phys, flux) if charged else None)


def reference_lattice_of(state, dense):
    """An (L1, L2) object array of reference tensors with the edges of ``state``'s sites holding the dense
    (P0, U, D, L, R) arrays ``dense[l1][l2]`` (the layout apply_gradient and lattice_dot take)."""
    out = np.empty((state.L1, state.L2), dtype=object)
    for l1 in range(state.L1):
        for l2 in range(state.L2):
            t = state[l1, l2]
            names, segs = _names_edges(t)
            a = np.asarray(dense[l1][l2], dtype=np.float64)
            keep = [n for n in ORDER if n in names]
            extra = [n for n in names if n not in ORDER]
            arr = a.reshape([a.shape[ORDER.index(n)] for n in keep] + [1] * len(extra))
            order = keep + extra
            arr = arr.transpose([order.index(n) for n in names])
            g = t.same_shape()
            np.asarray(g.storage)[:] = dense_to_blocks(arr, segs)
            out[l1, l2] = g
    return out


class ReferenceObserver:
    """``Observer(state, ...)`` for a reference lattice, observing through ``tnsp_gb300.sampling.Observer``."""

    def __init__(self, owner, *, observer_set=None, enable_energy=False, enable_gradient=False,
                 enable_natural_gradient=False, cache_natural_delta=None, cache_configuration=False,
                 restrict_subspace=None, classical_energy=None):
        self.owner = owner
        self._kwargs = dict(observer_set=observer_set, enable_energy=enable_energy, enable_gradient=enable_gradient,
                            enable_natural_gradient=enable_natural_gradient, cache_natural_delta=cache_natural_delta,
                            cache_configuration=cache_configuration, restrict_subspace=restrict_subspace,
                            classical_energy=classical_energy)
        self._inner = None

    def add_observer(self, name, observers):
        raise NotImplementedError("pass diagonal observer sets through observer_set")

    def __enter__(self):
        dense = dense_lattice(self.owner)
        _DENSE[id(self.owner)] = dense
        self._inner = _drop.Observer(dense, **self._kwargs)
        self._inner.__enter__()
        return self

    def __exit__(self, exc_type, exc_val, exc_tb):
        return self._inner.__exit__(exc_type, exc_val, exc_tb)

    def __call__(self, possibility, configuration):
        self._inner(possibility, configuration)

    energy = property(lambda self: self._inner.energy)
    total_energy = property(lambda self: self._inner.total_energy)
    instability = property(lambda self: self._inner.instability)
    result = property(lambda self: self._inner.result)
    whole_result = property(lambda self: self._inner.whole_result)

    @property
    def gradient(self):
        return reference_lattice_of(self.owner, self._inner.gradient)

    def natural_gradient_by_conjugate_gradient(self, step, error):
        return reference_lattice_of(self.owner, self._inner.natural_gradient_by_conjugate_gradient(step, error))

    def natural_gradient_by_direct_pseudo_inverse(self, r_pinv, a_pinv, libraries=None):
        return reference_lattice_of(self.owner,
                                    self._inner.natural_gradient_by_direct_pseudo_inverse(r_pinv, a_pinv, libraries))

    def normalize_lattice(self):
        """``Observer.normalize_lattice`` (observer.py:909-920) on the reference tensors."""
        s = self._inner._read()
        param = np.exp(s[3] / s[0] / (self.owner.L1 * self.owner.L2))
        for l1 in range(self.owner.L1):
            for l2 in range(self.owner.L2):
                self.owner[l1, l2] = self.owner[l1, l2] / param


class ReferenceSweepSampling:
    """``SweepSampling(state, cut, restrict_subspace, hopping_hamiltonians)`` for a reference lattice inside
    a ``ReferenceObserver`` context (or on its own)."""

    def __init__(self, owner, cut_dimension, restrict_subspace, hopping_hamiltonians):
        from tetragono.utility import seed_differ
        dense = _DENSE.get(id(owner)) or dense_lattice(owner)
        hopping = None
        if hopping_hamiltonians is not None:
            hopping = {}
            pseg = _segments(owner.physics_edges[0, 0, 0])
            for positions, H in hopping_hamiltonians.items():
                names, segs = _names_edges(H)
                hopping[positions] = element_table(np.array(H.storage), names, segs, pseg)
        seed = int(seed_differ.seed)
        self._inner = _drop.SweepSampling(dense, cut_dimension, restrict_subspace, hopping, chains=CHAINS,
                                          seeds=np.arange(CHAINS, dtype=np.uint64) + np.uint64(seed), discard=1)
        self.owner = owner

    @property
    def configuration(self):
        return self._inner.configuration

    def __call__(self):
        return self._inner()

    def refresh_all(self):
        self._inner.refresh_all()


@contextlib.contextmanager
def adapted():
    """Within this context tetragono's gradient driver uses the adapters (its module-level names
    SweepSampling and Observer, which it resolves at call time)."""
    from tetragono.sampling_lattice import gradient
    saved = gradient.SweepSampling, gradient.Observer
    gradient.SweepSampling, gradient.Observer = ReferenceSweepSampling, ReferenceObserver
    try:
        yield gradient
    finally:
        gradient.SweepSampling, gradient.Observer = saved


def run_gradient_descent(state, **kwargs):
    """Runs the reference's ``gradient_descent(state, **kwargs)`` unchanged on the GPU sampler
    (``sampling_method="sweep"``); yields what it yields."""
    if kwargs.get("sampling_method", "direct") != "sweep":
        raise NotImplementedError("the GPU sampler provides sweep sampling")
    with adapted() as gradient:
        yield from gradient.gradient_descent(state, **kwargs)
