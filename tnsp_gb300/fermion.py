"""Host side of fermionic (Fermi U(1)) lattices: the spinless t-V state of tetraku
(tetraku/tetraku/models/tV/__init__.py:23-76), the reference's fermionic lattice files in dense
form, and the tables with which a dense (bosonic) boundary-MPS sampler evaluates them exactly as the
reference's graded contraction does.

Why a dense sampler can evaluate a fermionic PEPS.  TAT contracts Z2-graded tensors: transposing two
odd legs gives -1, reversing an arrow-False leg during a contraction gives (-1)^parity, and merges
carry ((n_odd & 2) != 0) (TAT/include/TAT/implement/edge_operator.hpp:497-612,
contract.hpp:381-580).  Contracting a whole network in a fixed linear order of its legs then equals
the plain sum over bond indices times, per index assignment, (-1)^p for every bond whose first leg
is arrow False, (-1)^(p_e p_f) for every pair of bonds whose ends interleave, and
(-1)^(p_e * parity of the open legs between e's ends).  tetragono's projected sites have their legs
in the order (T, U, D, L, R, P) with the open dimension-one leg ``P_{l1}_{l2}_0`` last
(tetragono/tetragono/sampling_lattice/lattice.py:291-339), every projected site is even, and charge
conservation across every prefix of sites turns the non-local terms into a sign of the configuration
alone plus one parity operator per site raised to a particle count of its own row (or column).
Per site, on the stored slice of occupation n (the shrinker contraction itself gives (-1)^n):

* row-major (up / down boundaries, row strips):
  (-1)^( n + p_R (1 + n) + p_L p_D + p_D M_row ),  M_row = particles left of the site in its row;
* column-major (left / right boundaries, column strips):
  (-1)^( n + p_D (1 + n) + p_D p_L + p_D p_R + p_L p_U + p_R M_col ),  M_col = particles above it;

with p_X the parity of the charge of the index on leg X.  The amplitude in the reference's canonical
leg order is the bosonic value times ``configuration_sign``; E_loc takes ``hop_sign`` per term, and a
vertical pair evaluated on column strips also the column / row configuration signs and
``order_inversions``; the gradient is the bosonic one (each sample's hole multiplied by the same
(-1)^(p_D M_row) as its slice) times ``gradient_sign`` per element.  The truncated boundary-MPS
compression is unchanged: on every cut of a boundary line these signs are per-leg signs times a
function of the two sides' total parities, so the singular values and the kept subspaces are the
graded ones.  Every rule here is pinned to the reference's own amplitudes, local energies, holes and
gradients with the truncation active (tests/test_fermion_host.py, tests/test_fermi_peps.py).

``sign_folded_slices`` stores, per site, the eight slices [family][n][M parity] a sampler reads
instead of the two physical slices.
"""
import numpy as np

from .lattice import element_table, iterate_blocks, site_charges, site_from_blocks

ROW, COL = 0, 1
LEGS = ("U", "D", "L", "R")
PHYSICS = [(0, 1), (1, 1)]   # spinless fermion: empty (charge 0), occupied (charge 1); arrow False


def _parity(charges):
    return (np.asarray(charges, dtype=np.int64) & 1).astype(np.int64)


class FermionLattice:
    """Dense site tensors ``A[p, u, d, l, r]`` in TAT's block layout (segments concatenated in edge
    order; the one-dimensional T leg of site (0, 0) dropped), the U(1) charges of every leg index,
    the charge of the T leg, and the Hamiltonian's element tables."""

    def __init__(self, L1, L2, tensors, legs, T_charge, terms, edges=None, names=None):
        self.L1, self.L2 = L1, L2
        self.tensors = tensors
        self.legs = legs                 # legs[l1][l2][X] = per-index charges (TAT's edge charges)
        self.T_charge = int(T_charge)    # charge of the T leg of site (0, 0): minus the particle number
        self.terms = terms               # {positions: {input tuple: [(output tuple, value)]}}
        self.edges = edges               # per site: TAT segment lists and arrows, in ``names`` order
        self.names = names

    @property
    def particles(self):
        return -self.T_charge

    @property
    def p_T(self):
        return self.T_charge & 1

    def parities(self, l1, l2):
        return [_parity(self.legs[l1][l2][x]) for x in LEGS]

    def flux(self):
        """Per-site flux of the sector rule: sum of leg charges + physical charge == flux."""
        return [[(-self.T_charge if (a, b) == (0, 0) else 0) for b in range(self.L2)] for a in range(self.L1)]

    def charges(self):
        """(legs, physical charges, flux) as ``tnsp_gb300.lattice.SamplingLattice`` takes them."""
        return self.legs, [q for q, d in PHYSICS for _ in range(d)], self.flux()

    def _grid(self, l1, l2):
        par = self.parities(l1, l2)
        return np.ix_(*par), tuple(len(p) for p in par)

    def static_signs(self, l1, l2, family, n):
        """+-1 array (u, d, l, r): the configuration-independent part of the site's sign."""
        (U, D, L, R), shape = self._grid(l1, l2)
        if family == ROW:
            e = n + R * (1 + n) + L * D
        else:
            e = n + D * (1 + n) + D * L + D * R + L * U
        return np.where(np.broadcast_to(e & 1, shape).astype(bool), -1.0, 1.0)

    def prefix_sign(self, l1, l2, family):
        """The +-1 array (u, d, l, r) of the prefix parity operator: -1 on odd D (row) or R (column)
        indices, applied when the site's prefix count is odd."""
        (U, D, L, R), shape = self._grid(l1, l2)
        return np.where(np.broadcast_to(D if family == ROW else R, shape).astype(bool), -1.0, 1.0)

    def sign_folded_slices(self, l1, l2, tensor=None):
        """float64 [2 families][2 occupations][2 prefix parities][u][d][l][r] of the site's tensor (or of
        ``tensor``, the same site after a gradient step)."""
        a = self.tensors[l1][l2] if tensor is None else np.asarray(tensor)
        out = np.empty((2, 2, 2) + a.shape[1:])
        for family in (ROW, COL):
            prefix = self.prefix_sign(l1, l2, family)
            for n in (0, 1):
                s = a[n] * self.static_signs(l1, l2, family, n)
                out[family, n, 0] = s
                out[family, n, 1] = s * prefix
        return out

    def gradient_sign(self, l1, l2, n):
        """(-1)^(n + p_R (1 + n) + p_L p_D): the bosonic gradient's sign per element."""
        return self.static_signs(l1, l2, ROW, n)

    def fold_gradient(self, l1, l2, dense):
        """Gradient of site (l1, l2) in the dense layout of its tensor from the bosonic one
        (n, u, d, l, r), whose holes already carry the prefix parity."""
        out = np.array(dense, dtype=np.float64, copy=True)
        for n in (0, 1):
            out[n] *= self.gradient_sign(l1, l2, n)
        return out

    def slices_flat(self, tensors=None):
        """Every site's eight slices, in site order: the array ``tnsp_lattice_fermion`` takes."""
        return np.concatenate([self.sign_folded_slices(l1, l2, None if tensors is None else tensors[l1][l2]).ravel()
                               for l1 in range(self.L1) for l2 in range(self.L2)])

    def fold_flat(self, flat):
        """``fold_gradient`` over the flat (site-ordered, (n, u, d, l, r) per site) parameter vector."""
        out, pos = [], 0
        for l1 in range(self.L1):
            for l2 in range(self.L2):
                n = self.tensors[l1][l2].size
                out.append(self.fold_gradient(l1, l2, np.asarray(flat[pos:pos + n]).reshape(self.tensors[l1][l2].shape))
                           .ravel())
                pos += n
        return np.concatenate(out)

    def sampling_lattice(self):
        """The lattice the sampler takes: dense tensors, the Fermi U(1) charges as U(1) charges, the
        element tables, and this object as its ``fermion`` attribute, which makes ``engine.Sampler``
        upload the sign-folded slices and the drop-in Observer fold its gradients."""
        from .lattice import SamplingLattice
        lat = SamplingLattice(self.L1, self.L2, 2, [[t.copy() for t in row] for row in self.tensors], dict(self.terms),
                              self.charges())
        lat.fermion = self
        return lat

    def to_blocks(self, l1, l2, dense):
        """Block storage (TAT core order, the site's own leg order) of a dense (p, u, d, l, r) array."""
        from .checkpoint import dense_to_blocks
        names, edges = self.names[l1][l2], [segs for segs, _ in self.edges[l1][l2]]
        order = ["P0"] + list(LEGS)
        keep = [x for x in order if x in names]
        arr = np.asarray(dense).reshape([np.asarray(dense).shape[order.index(x)] for x in keep] +
                                        [1] * (len(names) - len(keep)))
        full = keep + [x for x in names if x not in order]
        arr = arr.transpose([full.index(x) for x in names])
        return dense_to_blocks(arr, edges)


def set_reference_tensors(ref, tensors):
    """Writes dense site tensors ``tensors[l1][l2]`` (p, u, d, l, r, the layout of FermionLattice) into
    the block storage of a fermionic lattice file read by ``tnsp_gb300.checkpoint.load_lattice`` (edges
    and arrows unchanged), so that ``save_lattice`` writes a file the reference loads; entries outside
    the charge blocks must be zero."""
    lat = from_reference_lattice(ref)
    st = ref.state
    for l1 in range(lat.L1):
        for l2 in range(lat.L2):
            storage = lat.to_blocks(l1, l2, tensors[l1][l2])
            back = site_from_blocks(storage, lat.names[l1][l2], [segs for segs, _ in lat.edges[l1][l2]])
            if not np.array_equal(back, np.asarray(tensors[l1][l2])):
                raise ValueError(f"site ({l1}, {l2}) has nonzero entries outside its symmetry blocks")
            st["_lattice"][l1][l2].storage = storage


def configuration_sign(conf, p_T, family):
    """prod over cuts k of (-1)^((N_<k + p_T)(N_<=k + p_T)), N counting the particles of the rows
    (row-major) or columns (column-major) before / up to k."""
    conf = np.asarray(conf)
    counts = conf.sum(axis=1) if family == ROW else conf.sum(axis=0)
    s, before = 0, int(p_T) & 1
    for k in range(len(counts) - 1):
        upto = (before + int(counts[k])) & 1
        s ^= before & upto
        before = upto
    return -1.0 if s else 1.0


def hop_sign(conf, positions, new):
    """Sign of one Hamiltonian element in E_loc with both amplitudes in row-major canonical order:
    1 for a diagonal element; for a particle moved between sites i < j (row-major),
    (-1)^(particles strictly between them), times -1 when it moves from i to j."""
    conf = np.asarray(conf)
    L2 = conf.shape[1]
    idx = [a * L2 + b for a, b in positions]
    flat = conf.reshape(-1)
    if all(flat[i] == s for i, s in zip(idx, new)):
        return 1.0
    i, j = sorted(idx)
    between = int(flat[i + 1:j].sum()) & 1
    target = dict(zip(idx, new))
    forward = flat[i] == 1 and target[i] == 0
    return (-1.0 if between else 1.0) * (-1.0 if forward else 1.0)


def order_inversions(conf):
    """Parity of the pairs of occupied sites with one strictly left of and below the other (the
    reordering of odd legs between column-major and row-major orders)."""
    conf = np.asarray(conf, dtype=np.int64)
    L1, L2 = conf.shape
    total = 0
    for a in range(1, L1):
        right = np.cumsum(conf[:a].sum(axis=0)[::-1])[::-1]   # particles in rows < a, columns >= b
        for b in range(L2 - 1):
            if conf[a, b]:
                total += int(right[b + 1])
    return total & 1


def vertical_pair_sign(conf, after, p_T):
    """Extra sign of a vertical pair evaluated on column strips against the row-strip amplitude of
    ``conf``: G_col(after) G_row(conf) (-1)^inversions(after)."""
    return configuration_sign(after, p_T, COL) * configuration_sign(conf, p_T, ROW) * \
        (-1.0)**order_inversions(after)


def tv_element_table(t=1.0, V=1.0):
    """Element table of H = -t CC + V N N on a bond (tetraku/tetraku/models/tV/__init__.py:36-41) as
    tensor_element reads it from TAT's blocks: input (n0, n1) -> [(output, value)], in the order the
    reference lists it.  The two hopping directions carry opposite values (the element of C0+ C1 and
    of C1+ C0 in TAT's graded convention, tetragono/tetragono/common_tensor/Fermi.py:24-36)."""
    return {(1, 0): [((0, 1), t)], (0, 1): [((1, 0), -t)], (1, 1): [((1, 1), V)]}


def from_reference_lattice(ref):
    """A FermionLattice from a reference lattice file read by ``tnsp_gb300.checkpoint.load_lattice``."""
    st = ref.state
    L1, L2 = st["L1"], st["L2"]
    grid = st["_lattice"]
    if getattr(type(grid[0][0]), "symmetry", "No") != "FermiU1":
        raise ValueError("not a Fermi U(1) lattice")
    phys = st["_physics_edges"][0][0][0].segments
    if [tuple(s) for s in phys] != PHYSICS:
        raise NotImplementedError("spinless fermions (physical edge [(0, 1), (1, 1)]) only")
    tensors = [[None] * L2 for _ in range(L1)]
    legs = [[None] * L2 for _ in range(L1)]
    edges = [[None] * L2 for _ in range(L1)]
    names = [[None] * L2 for _ in range(L1)]
    T_charge = 0
    for l1 in range(L1):
        for l2 in range(L2):
            t = grid[l1][l2]
            nm, eg = list(t.names), [list(e) for e in t.edges]
            if [n for n in nm if n.startswith("P")] != ["P0"]:
                raise NotImplementedError("one orbit (physical leg P0) per site only")
            tensors[l1][l2] = site_from_blocks(t.storage, nm, eg)
            legs[l1][l2], _, flux = site_charges(nm, eg)
            if "T" in nm:
                T_charge = eg[nm.index("T")][0][0]
            edges[l1][l2] = [(segs, arrow) for segs, arrow in zip(eg, t.arrows)]
            names[l1][l2] = nm
    terms = {}
    for positions, H in st["_hamiltonians"].items():
        terms[tuple(tuple(p) for p in positions)] = element_table(H.storage, list(H.names),
                                                                  [list(e) for e in H.edges], phys)
    return FermionLattice(L1, L2, tensors, legs, T_charge, terms, edges, names)


def random_tv(L1, L2, D, particles, seed, interior=None, t=1.0, V=1.0, scale=True):
    """A t-V lattice with tetraku's bond layout (tV/__init__.py:52-76): R bonds and the column-0 D
    bonds carry sectors {Q-1, Q, Q+1} with the charge flow Q of those lines and dimensions ``D`` (an
    int for all three, or a (d_-, d_0, d_+) triple), interior D bonds ``interior`` (default tetraku's
    [(0, D)]); blocks i.i.d. N(0, 1) from numpy's generator, scaled by 1/sqrt(2 D_bond^z) when
    ``scale``.  The 8x8 fermionic workload is ``random_tv(8, 8, (2, 4, 2), 32, seed,
    interior=[(-1, 2), (0, 4), (1, 2)])``."""
    rng = np.random.default_rng(seed)
    T = particles
    dims = (D, D, D) if np.isscalar(D) else tuple(D)
    bonds_d = {}
    for l1 in range(L1 - 1):
        Q = int(T * (L1 - l1 - 1) / L1)
        bonds_d[l1, 0] = [(Q - 1, dims[0]), (Q, dims[1]), (Q + 1, dims[2])]
        for l2 in range(1, L2):
            bonds_d[l1, l2] = list(interior) if interior is not None else [(0, dims[1])]
    bonds_r = {}
    tt = T / L1
    for l1 in range(L1):
        for l2 in range(L2 - 1):
            Q = int(tt * (L2 - l2 - 1) / L2)
            bonds_r[l1, l2] = [(Q - 1, dims[0]), (Q, dims[1]), (Q + 1, dims[2])]
    tensors = [[None] * L2 for _ in range(L1)]
    legs = [[None] * L2 for _ in range(L1)]
    edges = [[None] * L2 for _ in range(L1)]
    names = [[None] * L2 for _ in range(L1)]
    for l1 in range(L1):
        for l2 in range(L2):
            nm, eg = ["P0"], [(list(PHYSICS), False)]
            if (l1, l2) == (0, 0):
                nm.append("T")
                eg.append(([(-T, 1)], False))
            if l1 > 0:
                nm.append("U")
                eg.append(([(-q, d) for q, d in bonds_d[l1 - 1, l2]], True))
            if l1 < L1 - 1:
                nm.append("D")
                eg.append((bonds_d[l1, l2], False))
            if l2 > 0:
                nm.append("L")
                eg.append(([(-q, d) for q, d in bonds_r[l1, l2 - 1]], True))
            if l2 < L2 - 1:
                nm.append("R")
                eg.append((bonds_r[l1, l2], False))
            segs = [s for s, _ in eg]
            size = _block_storage_size(segs)
            storage = rng.standard_normal(size)
            if scale:
                z = sum(1 for n in nm if n in LEGS)
                bond = sum(d for _, d in bonds_r[0, 0]) if L2 > 1 else 1
                storage /= np.sqrt(2.0 * bond**z)
            tensors[l1][l2] = site_from_blocks(storage, nm, segs)
            legs[l1][l2], _, _ = site_charges(nm, segs)
            edges[l1][l2] = eg
            names[l1][l2] = nm
    table = tv_element_table(t, V)
    terms = {}   # the reference's order: every vertical bond, then every horizontal bond
    for l1 in range(L1 - 1):
        for l2 in range(L2):
            terms[((l1, l2, 0), (l1 + 1, l2, 0))] = table
    for l1 in range(L1):
        for l2 in range(L2 - 1):
            terms[((l1, l2, 0), (l1, l2 + 1, 0))] = table
    return FermionLattice(L1, L2, tensors, legs, -T, terms, edges, names)


def _block_storage_size(edges):
    return sum(int(np.prod([edges[i][k][1] for i, k in enumerate(idx)])) for idx, _ in iterate_blocks(edges))


__all__ = ["FermionLattice", "configuration_sign", "hop_sign", "order_inversions", "vertical_pair_sign",
           "tv_element_table", "from_reference_lattice", "set_reference_tensors", "random_tv"]
