"""CPU (numpy, FP64) restatement of tetragono's sampling-lattice hot path over a PEPS.

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports this module: it is the oracle that
tests/, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use as the checker.
It is pinned against golden vectors produced by the reference itself (tests/golden/).

The state is held densely: a site tensor is an array ``A[p, u, d, l, r]`` (physical index, then
the up/down/left/right virtual bonds; a missing bond at the lattice edge has extent 1).  A
Bose-symmetric (U(1), Z2) tensor is the same array with zeros outside its allowed blocks; every
quantity below is then identical to the block-sparse result of the reference, because block
structure only permutes rows/columns of each matrix that is factorised and the truncated SVD
keeps the same singular subspace (up to exact ties at the cut).

What is restated, with the reference lines it follows:

* boundary MPS compression ``_two_line_to_one_line``
  (tetragono/tetragono/auxiliaries/single_layer_auxiliaries.py:462-498): contract a boundary
  line with the next row (or column), QR sweep towards the far end, then SVD sweep back,
  truncating every bond to ``cut``; ``normalize=False`` on this path
  (tetragono/tetragono/sampling_lattice/lattice.py:69);
* the four boundary families ``_up_to_down`` / ``_down_to_up`` / ``_left_to_right`` /
  ``_right_to_left`` (single_layer_auxiliaries.py:430-456);
* three-line strips and the amplitude ``hole(())`` = ``_inline_right_to_left[0, 0]``
  (single_layer_auxiliaries.py:254-280, 710-720);
* two-site replacements for horizontal and vertical pairs (single_layer_auxiliaries.py:568-692);
* one-site holes ``hole(((l1, l2),))`` with the horizontal hint (single_layer_auxiliaries.py:721-729)
  and ``Configuration.holes`` (tetragono/tetragono/sampling_lattice/lattice.py:362-416);
* ``SweepSampling._single_term`` / ``__call__`` / ``_get_proper_position_order``
  (tetragono/tetragono/sampling_lattice/sampling.py:117-190);
* ``Observer.__call__`` and the estimators (tetragono/tetragono/sampling_lattice/observer.py:313-415,
  433-469, 528-555);
* ``DirectSampling.__call__`` with exact cuts (tetragono/tetragono/sampling_lattice/sampling.py:276-371),
  its marginals by enumeration (``DirectSamplerExact``, small lattices).

With charges (Bose U(1)) every QR and SVD of the compression is done per charge sector, with the
truncation keeping the largest singular values over all sectors, as TAT's block-sparse qr / svd
do (TAT/include/TAT/implement/qr.hpp:310-510, svd.hpp:259-532); the boundaries are cached and
invalidated like the reference's lazy DAG (only the lines containing a changed site are dropped),
so the oracle's cost per sample follows the reference's.
"""

import numpy as np

from .rng import MT19937_64, uniform_int, uniform_real01

# Every tensor contraction of the boundary-MPS path goes through these three functions (float64 by
# default).  oracle/precision_study.py replaces them to measure what lower-precision products (float32,
# split TF32/BF16 products with float32 accumulation) do to amplitudes and E_loc, with the QR and SVD
# kept in float64.
contract = np.tensordot
matmul = np.matmul


def full_dot(a, b):
    """sum of a * b over all (three) legs"""
    return np.einsum("arb,arb->", a, b)



# ----------------------------------------------------------------------------------------------
# boundary MPS
# ----------------------------------------------------------------------------------------------
def ones_line(n):
    """The boundary beyond the lattice edge: scalar ones (``_one_l1``/``_one_l2``)."""
    return [np.ones((1, 1, 1)) for _ in range(n)]


def ones_charges(n):
    return [(np.zeros(1, int), np.zeros(1, int), 0) for _ in range(n)]


def _sectors(qrow, qcol, F):
    """[(r, rows, cols)] for the block structure qrow + qcol == F, row charges ascending."""
    out = []
    for r in sorted(set(qrow.tolist())):
        rows = np.nonzero(qrow == r)[0]
        cols = np.nonzero(qcol == F - r)[0]
        if len(rows) and len(cols):
            out.append((r, rows, cols))
    return out


def compress(line, sites, cut, line_q=None, site_q=None):
    """``_two_line_to_one_line`` on dense tensors.

    ``line[i]`` has shape (a, p, b): left bond, open leg towards ``sites``, right bond.
    ``sites[i]`` has shape (u, d, l, r) with ``u`` contracted against ``line``'s ``p``.
    ``line_q[i]`` = (qa, qb, flux) and ``site_q[i]`` = (qu, qd, ql, qr, flux) are index charges
    (None: no symmetry).  Returns the new line, tensors (a', d, b'), and its charges.
    """
    n = len(line)
    T, qA, qD, qB, F = [], [], [], [], []
    for i in range(n):
        a, p, b = line[i].shape
        u, d, l, r = sites[i].shape
        assert p == u
        t = contract(line[i], sites[i], axes=([1], [0]))  # (a, b, d, l, r)
        T.append(t.transpose(0, 3, 2, 1, 4).reshape(a * l, d, b * r))
        la, lb, lf = line_q[i] if line_q is not None else (np.zeros(a, int), np.zeros(b, int), 0)
        _, sd, sl, sr, sf = site_q[i] if site_q is not None else (None, np.zeros(d, int), np.zeros(l, int),
                                                                    np.zeros(r, int), 0)
        qA.append((np.asarray(la)[:, None] + np.asarray(sl)[None, :]).reshape(-1))
        qD.append(np.asarray(sd))
        qB.append((np.asarray(lb)[:, None] + np.asarray(sr)[None, :]).reshape(-1))
        F.append(lf + sf)
    # QR sweep, per sector (single_layer_auxiliaries.py:484-488)
    for i in range(n - 1):
        A, d, B = T[i].shape
        M = T[i].reshape(A * d, B)
        qrow = (qA[i][:, None] + qD[i][None, :]).reshape(-1)
        secs = _sectors(qrow, qB[i], F[i])
        ktot = sum(min(len(rows), len(cols)) for _, rows, cols in secs)
        Q = np.zeros((A * d, ktot))
        R = np.zeros((ktot, B))
        qk = np.zeros(ktot, int)
        k0 = 0
        for r, rows, cols in secs:
            q, rr = np.linalg.qr(M[np.ix_(rows, cols)])
            k = q.shape[1]
            Q[rows, k0:k0 + k] = q
            R[k0:k0 + k][:, cols] = rr
            qk[k0:k0 + k] = r
            k0 += k
        T[i] = Q.reshape(A, d, ktot)
        b_, d_, c_ = T[i + 1].shape
        T[i + 1] = matmul(R, T[i + 1].reshape(b_, d_ * c_)).reshape(ktot, d_, c_)
        qB[i] = -qk
        qA[i + 1] = qk
        F[i + 1] += F[i]
        F[i] = 0
    # SVD sweep with truncation over all sectors (single_layer_auxiliaries.py:490-496, svd.hpp:429-470)
    for i in reversed(range(1, n)):
        A, d, B = T[i].shape
        M = T[i].reshape(A, d * B)
        qcol = (qD[i][:, None] + qB[i][None, :]).reshape(-1)
        secs = _sectors(qA[i], qcol, F[i])
        found = []
        for si, (r, rows, cols) in enumerate(secs):
            U, S, Vh = np.linalg.svd(M[np.ix_(rows, cols)], full_matrices=False)
            for j in range(len(S)):
                found.append((-S[j], si, j, U[:, j] * S[j], Vh[j]))
        found.sort(key=lambda x: (x[0], x[1], x[2]))
        kept = found[:min(cut, len(found))]
        c = len(kept)
        Vnew = np.zeros((c, d * B))
        US = np.zeros((A, c))
        qk = np.zeros(c, int)
        for t, (_, si, _, us, vh) in enumerate(kept):
            r, rows, cols = secs[si]
            Vnew[t, cols] = vh
            US[rows, t] = us
            qk[t] = r
        T[i] = Vnew.reshape(c, d, B)
        a_, d_, b_ = T[i - 1].shape
        T[i - 1] = matmul(T[i - 1].reshape(a_ * d_, b_), US).reshape(a_, d_, c)
        qA[i] = qk
        qB[i - 1] = -qk
    return T, [(qA[i], qB[i], F[i]) for i in range(n)]


# ----------------------------------------------------------------------------------------------
# strips: the exact contraction of (up line, row of sites, down line)
# ----------------------------------------------------------------------------------------------
def strip_step_left(E, up, site, down):
    """E (x, y, z) -> E' (a, r, b): absorb one column of a three-line strip from the left."""
    t1 = contract(E, up, axes=([0], [0]))  # (y, z, u, a)
    t2 = contract(t1, site, axes=([0, 2], [2, 0]))  # (z, a, d, r)
    return contract(t2, down, axes=([0, 2], [0, 1]))  # (a, r, b)


def strip_step_right(F, up, site, down):
    """F (a, r, b) -> F' (x, l, z): absorb one column of a three-line strip from the right."""
    s1 = contract(up, F, axes=([2], [0]))  # (x, u, r, b)
    s2 = contract(s1, site, axes=([1, 2], [0, 3]))  # (x, b, d, l)
    return contract(s2, down, axes=([1, 2], [2, 1])).transpose(0, 1, 2)  # (x, l, z)


def strip_envs(up, sites, down):
    n = len(sites)
    E = [None] * (n + 1)  # E[c+1] = contraction of columns 0..c
    F = [None] * (n + 1)  # F[c] = contraction of columns c..n-1
    E[0] = np.ones((1, 1, 1))
    F[n] = np.ones((1, 1, 1))
    for c in range(n):
        E[c + 1] = strip_step_left(E[c], up[c], sites[c], down[c])
    for c in reversed(range(n)):
        F[c] = strip_step_right(F[c + 1], up[c], sites[c], down[c])
    return E, F


def strip_value(up, sites, down):
    F = np.ones((1, 1, 1))
    for c in reversed(range(len(sites))):
        F = strip_step_right(F, up[c], sites[c], down[c])
    return float(F.reshape(-1)[0])


def strip_hole(E_left, up, down, F_right):
    """d value / d site, shape (u, d, l, r)."""
    h1 = contract(E_left, up, axes=([0], [0]))  # (l, z, u, a)
    h2 = contract(h1, down, axes=([1], [0]))  # (l, u, a, d, b)
    h = contract(h2, F_right, axes=([2, 4], [0, 2]))  # (l, u, d, r)
    return h.transpose(1, 2, 0, 3)


# ----------------------------------------------------------------------------------------------
# the lattice and its configuration
# ----------------------------------------------------------------------------------------------
class DensePEPS:
    """Site tensors ``A[l1][l2]`` of shape (P, U, D, L, R) plus the Hamiltonian element tables.

    ``terms`` is the ordered Hamiltonian: a list of ``(positions, table)`` where ``positions`` is
    a tuple of (l1, l2, orbit) and ``table`` maps an input tuple of physical indices to the
    ordered list of ``(output tuple, value)``, exactly as ``tensor_element`` orders it
    (tetragono/tetragono/tensor_element.py:91-108).  Only orbit 0 is supported.
    """

    def __init__(self, tensors, terms, cut, charges=None):
        """``charges``: optional (legs, phys, flux) as in tnsp_gb300.lattice.SamplingLattice."""
        self.A = tensors
        self.L1 = len(tensors)
        self.L2 = len(tensors[0])
        self.terms = terms
        self.cut = cut
        self.site_number = self.L1 * self.L2
        self.charges = charges

    def site_q(self, l1, l2, s, orient):
        """Index charges (qu, qd, ql, qr, flux) of the projected site in one of the orientations
        used by row_sites / col_sites: 0 row, 1 row flipped, 2 column, 3 column flipped."""
        if self.charges is None:
            return None
        legs, phys, flux = self.charges
        q = {k: np.asarray(v, int) for k, v in legs[l1][l2].items()}
        f = flux[l1][l2] - phys[s]
        U, D, L, R = q["U"], q["D"], q["L"], q["R"]
        return [(U, D, L, R, f), (D, U, L, R, f), (L, R, U, D, f), (R, L, U, D, f)][orient]

    # projected sites in the four orientations -------------------------------------------
    def site(self, l1, l2, s):
        return self.A[l1][l2][s]  # (u, d, l, r)

    def row_sites(self, conf, l1, flip=False):
        """Row l1 in (u, d, l, r) orientation; ``flip`` swaps up/down (for down_to_up)."""
        out = []
        for l2 in range(self.L2):
            t = self.site(l1, l2, conf[l1, l2])
            out.append(t.transpose(1, 0, 2, 3) if flip else t)
        return out

    def row_q(self, conf, l1, flip=False):
        if self.charges is None:
            return None
        return [self.site_q(l1, l2, conf[l1, l2], 1 if flip else 0) for l2 in range(self.L2)]

    def col_sites(self, conf, l2, flip=False):
        """Column l2 as a "row": (l, r, u, d) orientation; ``flip`` -> (r, l, u, d)."""
        out = []
        for l1 in range(self.L1):
            t = self.site(l1, l2, conf[l1, l2])
            out.append(t.transpose(3, 2, 0, 1) if flip else t.transpose(2, 3, 0, 1))
        return out

    def col_q(self, conf, l2, flip=False):
        if self.charges is None:
            return None
        return [self.site_q(l1, l2, conf[l1, l2], 3 if flip else 2) for l1 in range(self.L1)]


class Environment:
    """All boundaries and strips of one configuration (what the lazy DAG would hold).

    ``update`` changes sites and drops exactly the cached boundaries that contain them, as an
    accepted hop resets the reference's lazy nodes (lazy_graph/lazy/__init__.py ``Node.reset``)."""

    def __init__(self, peps, conf):
        self.peps = peps
        self.conf = np.array(conf)
        self._up = {}
        self._down = {}
        self._left = {}
        self._right = {}
        self._row_envs = {}
        self._col_envs = {}

    def update(self, changes):
        for l1, l2, s in changes:
            self.conf[l1, l2] = s
            for k in [k for k in self._up if k >= l1]:
                del self._up[k]
            for k in [k for k in self._down if k <= l1]:
                del self._down[k]
            for k in [k for k in self._left if k >= l2]:
                del self._left[k]
            for k in [k for k in self._right if k <= l2]:
                del self._right[k]
        self._row_envs = {}
        self._col_envs = {}

    def _line(self, cache, k, edge, n, prev, sites, sq):
        if k == edge:
            return ones_line(n), ones_charges(n)
        if k not in cache:
            line, lq = prev()
            cache[k] = compress(line, sites(), self.peps.cut, lq if self.peps.charges is not None else None, sq())
        return cache[k]

    # boundary families (single_layer_auxiliaries.py:430-456) ------------------------------
    def up_q(self, l1):
        """``_up_to_down[l1]``: rows 0..l1 compressed from the top; open legs point down."""
        p = self.peps
        return self._line(self._up, l1, -1, p.L2, lambda: self.up_q(l1 - 1), lambda: p.row_sites(self.conf, l1),
                          lambda: p.row_q(self.conf, l1))

    def down_q(self, l1):
        """``_down_to_up[l1]``: rows l1..L1-1 compressed from the bottom; open legs point up."""
        p = self.peps
        return self._line(self._down, l1, p.L1, p.L2, lambda: self.down_q(l1 + 1),
                          lambda: p.row_sites(self.conf, l1, flip=True), lambda: p.row_q(self.conf, l1, flip=True))

    def left_q(self, l2):
        p = self.peps
        return self._line(self._left, l2, -1, p.L1, lambda: self.left_q(l2 - 1), lambda: p.col_sites(self.conf, l2),
                          lambda: p.col_q(self.conf, l2))

    def right_q(self, l2):
        p = self.peps
        return self._line(self._right, l2, p.L2, p.L1, lambda: self.right_q(l2 + 1),
                          lambda: p.col_sites(self.conf, l2, flip=True), lambda: p.col_q(self.conf, l2, flip=True))

    def up(self, l1):
        return self.up_q(l1)[0]

    def down(self, l1):
        return self.down_q(l1)[0]

    def left(self, l2):
        return self.left_q(l2)[0]

    def right(self, l2):
        return self.right_q(l2)[0]

    # strips -------------------------------------------------------------------------------
    def row_envs(self, l1):
        if l1 not in self._row_envs:
            self._row_envs[l1] = strip_envs(self.up(l1 - 1), self.peps.row_sites(self.conf, l1), self.down(l1 + 1))
        return self._row_envs[l1]

    def col_envs(self, l2):
        if l2 not in self._col_envs:
            self._col_envs[l2] = strip_envs(self.left(l2 - 1), self.peps.col_sites(self.conf, l2), self.right(l2 + 1))
        return self._col_envs[l2]

    def amplitude(self):
        """``hole(())`` = ``_inline_right_to_left[0, 0]``: the row-0 strip."""
        E, F = self.row_envs(0)
        return float(F[0].reshape(-1)[0])

    def replace_horizontal(self, l1, l2, s0, s1):
        """psi with sites (l1,l2),(l1,l2+1) set to s0,s1 (single_layer_auxiliaries.py:674-680)."""
        p = self.peps
        E, F = self.row_envs(l1)
        up, down = self.up(l1 - 1), self.down(l1 + 1)
        e = strip_step_left(E[l2], up[l2], p.site(l1, l2, s0), down[l2])
        e = strip_step_left(e, up[l2 + 1], p.site(l1, l2 + 1, s1), down[l2 + 1])
        return float(full_dot(e, F[l2 + 2]))

    def replace_vertical(self, l1, l2, s0, s1):
        """psi with sites (l1,l2),(l1+1,l2) set to s0,s1 (single_layer_auxiliaries.py:686-692)."""
        p = self.peps
        E, F = self.col_envs(l2)
        lf, rt = self.left(l2 - 1), self.right(l2 + 1)
        e = strip_step_left(E[l1], lf[l1], p.site(l1, l2, s0).transpose(2, 3, 0, 1), rt[l1])
        e = strip_step_left(e, lf[l1 + 1], p.site(l1 + 1, l2, s1).transpose(2, 3, 0, 1), rt[l1 + 1])
        return float(full_dot(e, F[l1 + 2]))

    def site_hole(self, l1, l2):
        """d psi / d A[l1,l2][s] from the row strip, shape (u, d, l, r)."""
        E, F = self.row_envs(l1)
        return strip_hole(E[l2], self.up(l1 - 1)[l2], self.down(l1 + 1)[l2], F[l2 + 1])


def replace_amplitude(env, positions, s_new):
    """``Configuration.replace`` for a term's replacement (lattice.py:231-267 grouping)."""
    changed = [(pos, s) for pos, s in zip(positions, s_new) if env.conf[pos[0], pos[1]] != s]
    if len(changed) == 0:
        return env.amplitude()
    if len(changed) != 2:
        raise NotImplementedError("only two-site changes are restated")
    (p0, s0), (p1, s1) = changed
    if p0[0] == p1[0]:
        if p1[1] < p0[1]:
            p0, s0, p1, s1 = p1, s1, p0, s0
        assert p1[1] == p0[1] + 1
        return env.replace_horizontal(p0[0], p0[1], s0, s1)
    if p0[1] == p1[1]:
        if p1[0] < p0[0]:
            p0, s0, p1, s1 = p1, s1, p0, s0
        assert p1[0] == p0[0] + 1
        return env.replace_vertical(p0[0], p0[1], s0, s1)
    raise NotImplementedError("only nearest-neighbour pairs are restated")


# ----------------------------------------------------------------------------------------------
# sweep sampling
# ----------------------------------------------------------------------------------------------
def sweep_order(peps):
    """``_get_proper_position_order`` for nearest-neighbour two-site terms (sampling.py:156-190):
    horizontal pairs row-major, then vertical pairs column-major."""
    keys = [tuple(pos) for pos, _ in peps.terms]
    index = {k: i for i, k in enumerate(keys)}
    remaining = set(keys)
    result = []
    for l1 in range(peps.L1):
        for l2 in range(peps.L2):
            hit = [k for k in remaining if all((p[0], p[1]) in ((l1, l2), (l1, l2 + 1)) for p in k)]
            if len(hit) > 1:
                raise NotImplementedError("several terms on one pair")
            result += hit
            remaining -= set(hit)
    for l2 in range(peps.L2):
        for l1 in range(peps.L1):
            hit = [k for k in remaining if all((p[0], p[1]) in ((l1, l2), (l1 + 1, l2)) for p in k)]
            if len(hit) > 1:
                raise NotImplementedError("several terms on one pair")
            result += hit
            remaining -= set(hit)
    if remaining:
        raise NotImplementedError("Not implemented hamiltonian")
    return [index[k] for k in result]


class SweepChain:
    """One Markov chain of ``SweepSampling`` with its own engine (a reference process)."""

    def __init__(self, peps, conf, seed, discard=0):
        self.peps = peps
        self.conf = np.array(conf, dtype=np.int64)
        self.engine = MT19937_64(seed)
        for _ in range(discard):
            uniform_real01(self.engine)
        self.order = sweep_order(peps)
        self.accepts = 0
        self.proposals = 0
        self.env = None

    def sweep(self):
        """``SweepSampling.__call__``: returns (possibility, configuration copy)."""
        peps = self.peps
        if self.env is None:
            self.env = Environment(peps, self.conf)
        env = self.env
        ws = env.amplitude()
        for ti in self.order:
            positions, table = peps.terms[ti]
            s = tuple(int(self.conf[p[0], p[1]]) for p in positions)
            if s not in table:
                continue
            hops = table[s]
            if not hops:
                continue
            n = len(hops)
            s_new = hops[uniform_int(self.engine, 0, n - 1)][0]
            n_new = len(table[s_new])
            wss = replace_amplitude(env, positions, s_new)
            p = abs(wss / ws)**2 * n / n_new
            self.proposals += 1
            if uniform_real01(self.engine) < p:
                ws = wss
                if s_new != s:
                    self.accepts += 1
                    for pos, v in zip(positions, s_new):
                        self.conf[pos[0], pos[1]] = v
                    env.update([(pos[0], pos[1], v) for pos, v in zip(positions, s_new)])
        return abs(ws)**2, self.conf.copy()


# ----------------------------------------------------------------------------------------------
# observer
# ----------------------------------------------------------------------------------------------
def observe(peps, conf, env=None):
    """Per-sample quantities of ``Observer.__call__`` (observer.py:313-415).

    Returns (ws, eloc, holes) with ``holes[l1][l2]`` of shape (u, d, l, r) already divided by
    ws (the sampled physical slice of ``Configuration.holes``).  ``env``: the sampler's cached
    environment of the same configuration, if any."""
    if env is None or not np.array_equal(env.conf, conf):
        env = Environment(peps, np.asarray(conf))
    ws = env.amplitude()
    eloc = 0.0
    for positions, table in peps.terms:
        s = tuple(int(conf[p[0], p[1]]) for p in positions)
        if s not in table:
            continue
        total = 0.0
        for s_new, value in table[s]:
            wss = replace_amplitude(env, positions, s_new)
            if wss == 0.0:
                continue
            total += (ws / (ws * ws)) * value * wss
        eloc += total
    holes = [[env.site_hole(l1, l2) / ws for l2 in range(peps.L2)] for l1 in range(peps.L1)]
    return ws, eloc, holes


class ObserverAccumulator:
    """The energy/gradient accumulators of ``Observer`` (observer.py:41-126, 313-415)."""

    def __init__(self, peps, natural=False):
        self.peps = peps
        # per-sample (reweight, E_loc, dense hole row) kept for the natural gradient (observer.py:403-409)
        self.samples = [] if natural else None
        self.count = 0
        self.total_weight = 0.0
        self.total_weight_square = 0.0
        self.total_log_ws = 0.0
        self.er = 0.0
        self.err = 0.0
        self.eerr = 0.0
        self.Delta = [[np.zeros_like(peps.A[l1][l2]) for l2 in range(peps.L2)] for l1 in range(peps.L1)]
        self.EDelta = [[np.zeros_like(peps.A[l1][l2]) for l2 in range(peps.L2)] for l1 in range(peps.L1)]

    def add(self, possibility, conf, env=None):
        self.count += 1
        ws, eloc, holes = observe(self.peps, conf, env)
        if ws == 0.0:
            return ws, None, holes
        reweight = ws * ws / possibility
        self.total_weight += reweight
        self.total_weight_square += reweight * reweight
        self.total_log_ws += np.log(abs(ws))
        self.er += eloc * reweight
        self.err += eloc * reweight**2
        self.eerr += eloc**2 * reweight**2
        for l1 in range(self.peps.L1):
            for l2 in range(self.peps.L2):
                h = holes[l1][l2] * reweight
                s = conf[l1, l2]
                self.Delta[l1][l2][s] += h
                self.EDelta[l1][l2][s] += eloc * h
        if self.samples is not None:
            row = []
            for l1 in range(self.peps.L1):
                for l2 in range(self.peps.L2):
                    full = np.zeros_like(self.peps.A[l1][l2])
                    full[conf[l1, l2]] = holes[l1][l2]
                    row.append(full.ravel())
            self.samples.append((reweight, eloc, np.concatenate(row)))
        return ws, eloc, holes

    def total_energy(self):
        """``_expect_and_deviation`` (observer.py:433-469)."""
        if self.er == 0.0 or self.total_weight == 0.0:
            return 0.0, 0.0
        R, ER, RR, ERR, EERR = self.total_weight, self.er, self.total_weight_square, self.err, self.eerr
        expect = ER / R
        variance = (EERR - 2 * ERR * expect + RR * expect**2) / R**2
        return expect, (variance**0.5 if variance >= 0 else 0.0)

    def energy(self):
        e, d = self.total_energy()
        return e / self.peps.site_number, d / self.peps.site_number

    def natural_gradient(self, step, error):
        """``Observer.natural_gradient_by_conjugate_gradient`` (observer.py:576-675) for real tensors:
        conjugate gradient on D^T D x = D^T E with D_s = (delta_s - <delta>) sqrt(w_s / W) and
        E_s = (E_loc,s - <E>) sqrt(w_s / W), stopped after `step` steps or when |r|^2 / |b|^2 < error^2;
        returns 2 x per site.  Rows are dense (P, U, D, L, R) per site, concatenated in site order."""
        W = self.total_weight
        energy = self.er / W
        delta = np.concatenate([d.ravel() for row in self.Delta for d in row]) / W
        param = np.array([(r / W)**0.5 for r, _, _ in self.samples])
        Dm = np.array([(h - delta) * c for (_, _, h), c in zip(self.samples, param)])
        En = np.array([(e - energy) * c for (_, e, _), c in zip(self.samples, param)])

        def D(v):
            return Dm @ v

        def DT(v):
            return Dm.T @ v

        b = DT(En)
        b_square = np.dot(b, b)
        x = np.zeros_like(b)
        r = b - DT(D(x))
        p = r
        r_square = np.dot(r, r)
        t = 0
        while True:
            if t == step:
                break
            if error != 0.0 and error**2 > r_square / b_square:
                break
            Dp = D(p)
            alpha = r_square / np.dot(Dp, Dp)
            x = x + alpha * p
            r = r - alpha * DT(Dp)
            new_r_square = np.dot(r, r)
            beta = new_r_square / r_square
            r_square = new_r_square
            p = r + beta * p
            t += 1
        x = 2 * x
        out, o = [], 0
        for l1 in range(self.peps.L1):
            row = []
            for l2 in range(self.peps.L2):
                n = self.peps.A[l1][l2].size
                row.append(x[o:o + n].reshape(self.peps.A[l1][l2].shape))
                o += n
            out.append(row)
        return out, t

    def natural_gradient_pinv(self, r_pinv, a_pinv):
        """``natural_gradient_by_direct_pseudo_inverse`` (observer.py:697-907) by its single-process
        equation (observer.py:902-907): T = D D^T with unweighted rows D_s = delta_s - <delta>,
        L^+ = 1 / (L (1 + ((r max L + a) / L)^6)) on L > 0, NG = D^T U L^+ U^T (E - <E>); returns 2 NG
        per site."""
        if self.samples is None:
            raise RuntimeError("natural gradient not enabled")
        W = self.total_weight
        delta = np.concatenate([d.ravel() for row in self.Delta for d in row]) / W
        D = np.array([h - delta for _, _, h in self.samples])
        E = np.array([e for _, e, _ in self.samples]) - self.er / W
        L, U = np.linalg.eigh(D @ D.T)
        num = r_pinv * L.max() + a_pinv
        Linv = np.array([0.0 if l <= 0 else 1.0 / (l * (1 + (num / l)**6)) for l in L])
        x = 2 * (D.T @ (U @ (Linv * (U.T @ E))))
        out, o = [], 0
        for l1 in range(self.peps.L1):
            row = []
            for l2 in range(self.peps.L2):
                n = self.peps.A[l1][l2].size
                row.append(x[o:o + n].reshape(self.peps.A[l1][l2].shape))
                o += n
            out.append(row)
        return out

    def gradient(self):
        """``Observer.gradient`` (observer.py:542-555) for real tensors."""
        energy = self.er / self.total_weight
        return [[2 * (self.EDelta[l1][l2] / self.total_weight - energy * self.Delta[l1][l2] / self.total_weight)
                 for l2 in range(self.peps.L2)] for l1 in range(self.peps.L1)]


# ----------------------------------------------------------------------------------------------
# direct sampling, exact (small lattices)
# ----------------------------------------------------------------------------------------------
class DirectSamplerExact:
    """``DirectSampling.__call__`` (tetragono/tetragono/sampling_lattice/sampling.py:276-371) when its
    single- and double-layer cuts make every contraction exact: site by site in row-major order, one
    ``uniform_real(0, 1)`` draw per site chooses the physical index from the conditional marginal
    rho(x) ~ (sum over the unsampled sites of |psi|^2)^alpha, normalised, by the cumulative rule of
    ``_choice`` (:362-371); the returned possibility is the product of the chosen rho.  The marginals
    come from enumerating every configuration (P^(L1 L2) amplitudes; small lattices only)."""

    def __init__(self, peps, engine, alpha=1.0):
        import itertools
        self.peps, self.engine, self.alpha = peps, engine, alpha
        P = peps.A[0][0].shape[0]
        n = peps.L1 * peps.L2
        self.P, self.n = P, n
        w = np.zeros((P,) * n)
        for idx in itertools.product(range(P), repeat=n):
            conf = np.array(idx).reshape(peps.L1, peps.L2)
            w[idx] = Environment(peps, conf).amplitude()**2
        self.w = w

    def __call__(self):
        chosen = []
        possibility = 1.0
        for k in range(self.n):
            marg = self.w[tuple(chosen)]
            rho = marg.reshape(self.P, -1).sum(axis=1)
            rho = np.maximum(rho, 0.0)
            if rho.sum() == 0:
                raise NotImplementedError("zero marginal: the reference redraws the whole sample")
            rho = rho**self.alpha
            rho = rho / rho.sum()
            p = uniform_real01(self.engine)
            choice = len(rho) - 1
            for i, r in enumerate(rho):
                p -= r
                if p < 0:
                    choice = i
                    break
            possibility *= rho[choice]
            chosen.append(choice)
        return possibility, np.array(chosen).reshape(self.peps.L1, self.peps.L2)
