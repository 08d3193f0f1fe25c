"""Host-side lattice and Hamiltonian description (the planner half of the drop-in boundary).

A site tensor is held densely as ``A[p, u, d, l, r]`` (float64) with extent 1 for bonds that
leave the open lattice.  Bose-symmetric tensors are converted from the reference's block storage
by ``block_to_dense`` (block order of TAT/include/TAT/structure/core.hpp:152-191: every segment
combination whose charges sum to zero, in row-major order of segment indices, each block
row-major), so they keep the reference's symmetry-block indexing bit for bit.

Hamiltonian terms become element tables in the order of ``tensor_element``
(tetragono/tetragono/tensor_element.py:20-108).
"""
import numpy as np

ORDER = ("P0", "U", "D", "L", "R")


def _segment_offsets(segments):
    offs, o = [], 0
    for _, dim in segments:
        offs.append(o)
        o += dim
    return offs, o


def iterate_blocks(edges):
    """Yields (segment index tuple, charges tuple) for every allowed block, in core order.

    ``edges`` is a list of segment lists [(charge, dim), ...]; a block exists iff the charges
    sum to zero (Bose U(1); the no-symmetry case has a single segment of charge 0)."""
    rank = len(edges)
    if rank == 0:
        yield (), ()
        return
    if any(len(e) == 0 for e in edges):
        return
    idx = [0] * rank
    while True:
        charges = tuple(edges[i][idx[i]][0] for i in range(rank))
        if sum(charges) == 0:
            yield tuple(idx), charges
        pos = rank - 1
        idx[pos] += 1
        while idx[pos] == len(edges[pos]):
            if pos == 0:
                return
            idx[pos] = 0
            pos -= 1
            idx[pos] += 1


def block_to_dense(storage, edges):
    """Dense array (segments concatenated in edge order) from block storage in core order."""
    offs = [_segment_offsets(e) for e in edges]
    shape = tuple(o[1] for o in offs)
    dense = np.zeros(shape, dtype=np.float64)
    pos = 0
    for seg_idx, _ in iterate_blocks(edges):
        bshape = tuple(edges[i][seg_idx[i]][1] for i in range(len(edges)))
        n = int(np.prod(bshape)) if bshape else 1
        block = np.asarray(storage[pos:pos + n], dtype=np.float64).reshape(bshape)
        sl = tuple(slice(offs[i][0][seg_idx[i]], offs[i][0][seg_idx[i]] + bshape[i]) for i in range(len(edges)))
        dense[sl] = block
        pos += n
    if pos != len(storage):
        raise ValueError(f"storage size {len(storage)} does not match the block structure ({pos})")
    return dense


def site_from_blocks(storage, names, edges):
    """Site tensor (P0, U, D, L, R) from a reference site tensor's names, edge segments and storage.

    The one-dimensional total-charge leg ``T`` of site (0, 0) is kept in the block structure and
    dropped from the dense shape."""
    dense = block_to_dense(storage, edges)
    names = list(names)
    for n, e in zip(names, edges):
        if n not in ORDER and sum(d for _, d in e) != 1:
            raise ValueError(f"unexpected leg {n}")
    keep = [n for n in ORDER if n in names]
    perm = [names.index(n) for n in keep] + [i for i, n in enumerate(names) if n not in ORDER]
    arr = dense.transpose(perm).reshape(dense.transpose(perm).shape[:len(keep)])
    shape = [arr.shape[keep.index(n)] if n in keep else 1 for n in ORDER]
    return np.ascontiguousarray(arr.reshape(shape))


def expand_charges(segments):
    """Per-index charges of an edge given as [(charge, dim), ...]."""
    return [q for q, d in segments for _ in range(d)]


def site_charges(names, edges):
    """Charges of a reference site tensor: ({"U": [...], "D": [...], "L": [...], "R": [...]},
    physical charges, flux).  Absent legs get [0]; the one-dimensional total-charge leg T moves to
    the flux (every block of the reference satisfies sum of charges == 0, T included)."""
    names = list(names)
    legs = {}
    flux = 0
    phys = None
    for n, e in zip(names, edges):
        q = expand_charges(e)
        if n == "P0":
            phys = q
        elif n in ("U", "D", "L", "R"):
            legs[n] = q
        else:
            flux -= sum(q)  # a single index
    for n in ("U", "D", "L", "R"):
        legs.setdefault(n, [0])
    return legs, phys, flux


def physics_index(phys_segments, charge, index):
    """``Edge.index_by_point((charge, index))`` on the physical edge."""
    offs, _ = _segment_offsets(phys_segments)
    for k, (q, _) in enumerate(phys_segments):
        if q == charge:
            return offs[k] + index
    raise KeyError((charge, index))


def element_table(storage, names, edges, phys_segments):
    """``calculate_element`` of a Hamiltonian tensor with legs I0.., O0..

    Returns {input tuple: [(output tuple, value), ...]} with physical indices, iterating blocks in
    core order and elements row-major (loop_nonzero_tensor, tensor_element.py:51-88); the input
    point is the conjugate of the I-leg point (tensor_element.py:87-104)."""
    names = list(names)
    body = len(names) // 2
    table = {}
    pos = 0
    for seg_idx, charges in iterate_blocks(edges):
        bshape = tuple(edges[i][seg_idx[i]][1] for i in range(len(edges)))
        n = int(np.prod(bshape))
        block = np.asarray(storage[pos:pos + n]).reshape(bshape)
        pos += n
        for flat in range(n):
            value = block.flat[flat]
            if value == 0:
                continue
            elem = np.unravel_index(flat, bshape)
            points = {names[i]: (charges[i], int(elem[i])) for i in range(len(names))}
            s_in = tuple(physics_index(phys_segments, -points[f"I{i}"][0], points[f"I{i}"][1]) for i in range(body))
            s_out = tuple(physics_index(phys_segments, points[f"O{i}"][0], points[f"O{i}"][1]) for i in range(body))
            table.setdefault(s_in, []).append((s_out, float(value)))
    return table


class SamplingLattice:
    """Site tensors and Hamiltonian of a square-lattice PEPS (the state the sampler reads).

    Mirrors the parts of ``SamplingLattice`` (tetragono/tetragono/sampling_lattice/lattice.py:699-998)
    that the sweep / E_loc / gradient path reads: ``L1``, ``L2``, ``site_number``, ``[l1, l2]``
    get/set of site tensors, ``_hamiltonians`` (ordered), ``apply_gradient`` and ``lattice_dot``.
    """

    def __init__(self, L1, L2, P, tensors, hamiltonians, charges=None):
        """``charges``: optional (legs, phys, flux) with legs[l1][l2] = {"U": [...], "D": [...],
        "L": [...], "R": [...]} per-index charges, phys the physical charges and flux[l1][l2] the
        conserved sum of every nonzero element; enables per-sector factorisation on the device."""
        self.L1 = L1
        self.L2 = L2
        self.P = P
        self.charges = charges
        self._tensors = [[np.ascontiguousarray(tensors[l1][l2], dtype=np.float64) for l2 in range(L2)]
                         for l1 in range(L1)]
        self._hamiltonians = dict(hamiltonians)  # positions -> element table, reference dict order
        self.version = 0
        self._check()

    def _check(self):
        for l1 in range(self.L1):
            for l2 in range(self.L2):
                t = self._tensors[l1][l2]
                if t.ndim != 5 or t.shape[0] != self.P:
                    raise ValueError(f"site {(l1, l2)} must be (P, U, D, L, R)")
                U, D, L, R = t.shape[1:]
                if (l1 == 0 and U != 1) or (l1 == self.L1 - 1 and D != 1) or (l2 == 0 and L != 1) or \
                        (l2 == self.L2 - 1 and R != 1):
                    raise ValueError(f"site {(l1, l2)}: bonds leaving the lattice must have extent 1")
                if l2 + 1 < self.L2 and R != self._tensors[l1][l2 + 1].shape[3]:
                    raise ValueError("mismatched horizontal bond")
                if l1 + 1 < self.L1 and D != self._tensors[l1 + 1][l2].shape[1]:
                    raise ValueError("mismatched vertical bond")

    @property
    def site_number(self):
        return self.L1 * self.L2

    def sites(self):
        for l1 in range(self.L1):
            for l2 in range(self.L2):
                yield l1, l2

    def __getitem__(self, l1l2):
        l1, l2 = l1l2
        return self._tensors[l1][l2]

    def __setitem__(self, l1l2, tensor):
        l1, l2 = l1l2
        tensor = np.ascontiguousarray(tensor, dtype=np.float64)
        if tensor.shape != self._tensors[l1][l2].shape:
            raise ValueError("site tensor shape change is not supported")
        self._tensors[l1][l2] = tensor
        self.version += 1

    def dims(self):
        return np.array([[t.shape[1], t.shape[2], t.shape[3], t.shape[4]] for row in self._tensors for t in row],
                        dtype=np.int32)

    def charge_arrays(self):
        """(leg_charges, phys_charges, site_flux) in the layout of tnsp_lattice_charges, or None."""
        if self.charges is None:
            return None
        legs, phys, flux = self.charges
        Dmax = int(self.dims().max())
        q = np.zeros((self.L1, self.L2, 4, Dmax), dtype=np.int32)
        for l1, l2 in self.sites():
            for k, n in enumerate(("U", "D", "L", "R")):
                v = legs[l1][l2][n]
                q[l1, l2, k, :len(v)] = v
        return (np.ascontiguousarray(q.reshape(-1)), np.ascontiguousarray(np.asarray(phys, dtype=np.int32)),
                np.ascontiguousarray(np.asarray(flux, dtype=np.int32).reshape(-1)))

    def flat_tensors(self):
        return np.concatenate([t.reshape(-1) for row in self._tensors for t in row])

    def unflatten(self, flat):
        out, pos = [], 0
        for l1 in range(self.L1):
            row = []
            for l2 in range(self.L2):
                t = self._tensors[l1][l2]
                row.append(np.asarray(flat[pos:pos + t.size]).reshape(t.shape))
                pos += t.size
            out.append(row)
        return out

    def apply_gradient(self, gradient, step_size):
        """``SamplingLattice.apply_gradient`` (lattice.py:936-948) for real tensors; ``gradient`` is
        indexed [l1][l2] (or [l1, l2] for a numpy object array)."""
        for l1, l2 in self.sites():
            g = gradient[l1, l2] if isinstance(gradient, np.ndarray) else gradient[l1][l2]
            self[l1, l2] = self._tensors[l1][l2] - step_size * g

    def bcast_lattice(self, root=0):
        """One process owns every chain: nothing to broadcast (lattice.py:950-954)."""

    def lattice_dot(self, a=None, b=None):
        a = self._tensors if a is None else a
        b = a if b is None else b
        return float(sum(np.vdot(a[l1][l2], b[l1][l2]) for l1, l2 in self.sites()))

    def term_arrays(self):
        """Flattened Hamiltonian tables in the layout of tnsp_model_upload."""
        return table_arrays(self.P, self._hamiltonians)


def table_arrays(P, tables):
    """Flattened element tables {positions: {input tuple: [(output tuple, value), ...]}} in the layout
    of tnsp_model_upload / tnsp_model_hopping: (n_terms, sites, offsets, counts, out_index, values); the
    entries follow the dictionary order of the terms, inputs row-major, outputs in table order."""
    terms = list(tables.items())
    sites, offsets, counts, outs, vals = [], [], [], [], []
    for positions, table in terms:
        if len(positions) != 2:
            raise NotImplementedError("only two-site terms are supported")
        (a1, a2, ao), (b1, b2, bo) = positions
        if ao != 0 or bo != 0:
            raise NotImplementedError("only orbit 0 is supported")
        sites += [a1, a2, b1, b2]
        for s0 in range(P):
            for s1 in range(P):
                entries = table.get((s0, s1))
                if entries is None:
                    offsets.append(0)
                    counts.append(-1)
                    continue
                offsets.append(len(outs))
                counts.append(len(entries))
                for (o0, o1), v in entries:
                    outs.append(o0 * P + o1)
                    vals.append(v)
    return (len(terms), np.array(sites, dtype=np.int32), np.array(offsets, dtype=np.int32),
            np.array(counts, dtype=np.int32), np.array(outs, dtype=np.int32), np.array(vals, dtype=np.float64))


# --------------------------------------------------------------------------------------------
# model builders for synthetic, seeded states
# --------------------------------------------------------------------------------------------
def heisenberg_table(J=1.0):
    """H = J S.S on two spin-1/2 sites, physical index 0 = up, 1 = down.  Element order is the
    one tensor_element gives for the reference's SS tensors: inputs row-major, and for each input
    the outputs row-major."""
    table = {}
    for s0 in range(2):
        for s1 in range(2):
            sz = 0.25 if s0 == s1 else -0.25
            entries = [((s0, s1), J * sz)]
            if s0 != s1:
                entries.append(((s1, s0), J * 0.5))
            table[(s0, s1)] = sorted(entries)
    return table


def nearest_neighbour_terms(L1, L2, table):
    """Vertical bonds then horizontal bonds, as AbstractState's "vertical_bond" / "horizontal_bond"
    setters insert them (tetragono/tetragono/abstract_state.py, hamiltonians setter)."""
    terms = {}
    for l1 in range(L1 - 1):
        for l2 in range(L2):
            terms[((l1, l2, 0), (l1 + 1, l2, 0))] = table
    for l1 in range(L1):
        for l2 in range(L2 - 1):
            terms[((l1, l2, 0), (l1, l2 + 1, 0))] = table
    return terms


def u1_allowed_mask(P_charges, bond_charges_u, bond_charges_d, bond_charges_l, bond_charges_r, total=0):
    """Mask of allowed elements for a U(1) site tensor with legs (P, U, D, L, R) whose charges sum
    to ``total``; each argument lists the charge of every index of that leg."""
    q = (np.asarray(P_charges)[:, None, None, None, None] + np.asarray(bond_charges_u)[None, :, None, None, None] +
         np.asarray(bond_charges_d)[None, None, :, None, None] + np.asarray(bond_charges_l)[None, None, None, :, None] +
         np.asarray(bond_charges_r)[None, None, None, None, :])
    return q == total


def random_heisenberg(L1, L2, D, seed, scale=True, sectors=None, J=1.0):
    """Seeded random Heisenberg PEPS.

    ``sectors=None``: no symmetry, bond dimension D, elements N(0,1), optionally scaled by
    1/sqrt(2 D^z).  ``sectors=(n_m1, n_0, n_p1)``: Bose U(1) with physical charges (+1, -1) and
    virtual bonds {-1: n_m1, 0: n_0, +1: n_p1}; allowed blocks N(0,1).  The U/L legs carry the
    conjugated (negated) charges of the neighbour's D/R legs, so allowed blocks satisfy
    P + D + R - U - L = 0.
    """
    rng = np.random.default_rng(seed)
    tensors = []
    legs_q = []
    if sectors is None:
        Dv = D
        bond_q = None
    else:
        bond_q = np.concatenate([np.full(n, q) for q, n in zip((-1, 0, 1), sectors)])
        Dv = len(bond_q)
    for l1 in range(L1):
        row = []
        qrow = []
        for l2 in range(L2):
            U = Dv if l1 > 0 else 1
            Dd = Dv if l1 < L1 - 1 else 1
            L = Dv if l2 > 0 else 1
            R = Dv if l2 < L2 - 1 else 1
            t = rng.standard_normal((2, U, Dd, L, R))
            z = (l1 > 0) + (l1 < L1 - 1) + (l2 > 0) + (l2 < L2 - 1)
            if bond_q is not None:

                def qs(n, sign):
                    return sign * bond_q if n > 1 else np.zeros(1)

                mask = u1_allowed_mask([1, -1], qs(U, -1), qs(Dd, 1), qs(L, -1), qs(R, 1))
                t = t * mask
                qrow.append({"U": [int(x) for x in qs(U, -1)], "D": [int(x) for x in qs(Dd, 1)],
                             "L": [int(x) for x in qs(L, -1)], "R": [int(x) for x in qs(R, 1)]})
            if scale:
                t = t / np.sqrt(2.0 * Dv**z)
            row.append(t)
        tensors.append(row)
        legs_q.append(qrow)
    charges = None
    if bond_q is not None:
        charges = (legs_q, [1, -1], [[0] * L2 for _ in range(L1)])
    return SamplingLattice(L1, L2, 2, tensors, nearest_neighbour_terms(L1, L2, heisenberg_table(J)), charges)


def neel(L1, L2):
    return np.fromfunction(lambda a, b: (a + b) % 2, (L1, L2)).astype(np.int32)
