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
  433-469, 528-555).
"""

import numpy as np

from .rng import MT19937_64, uniform_int, uniform_real01


# ----------------------------------------------------------------------------------------------
# boundary MPS
# ----------------------------------------------------------------------------------------------
def ones_line(n):
    """The boundary beyond the lattice edge: scalar ones (``_one_l1``/``_one_l2``)."""
    return [np.ones((1, 1, 1)) for _ in range(n)]


def compress(line, sites, cut):
    """``_two_line_to_one_line`` on dense tensors.

    ``line[i]`` has shape (a, p, b): left bond, open leg towards ``sites``, right bond.
    ``sites[i]`` has shape (u, d, l, r) with ``u`` contracted against ``line``'s ``p``.
    Returns the new line, tensors (a', d, b').
    """
    n = len(line)
    T = []
    for i in range(n):
        a, p, b = line[i].shape
        u, d, l, r = sites[i].shape
        assert p == u
        t = np.einsum("apb,pdlr->aldbr", line[i], sites[i]).reshape(a * l, d, b * r)
        T.append(t)
    # QR sweep (single_layer_auxiliaries.py:484-488)
    for i in range(n - 1):
        a, d, b = T[i].shape
        q, r = np.linalg.qr(T[i].reshape(a * d, b))
        k = q.shape[1]
        T[i] = q.reshape(a, d, k)
        T[i + 1] = np.einsum("kb,bdc->kdc", r, T[i + 1])
    # SVD sweep with truncation (single_layer_auxiliaries.py:490-496)
    for i in reversed(range(1, n)):
        a, d, b = T[i].shape
        U, S, Vh = np.linalg.svd(T[i].reshape(a, d * b), full_matrices=False)
        c = min(cut, S.shape[0])
        T[i] = Vh[:c].reshape(c, d, b)
        T[i - 1] = np.einsum("adb,bc->adc", T[i - 1], U[:, :c] * S[None, :c])
    return T


# ----------------------------------------------------------------------------------------------
# strips: the exact contraction of (up line, row of sites, down line)
# ----------------------------------------------------------------------------------------------
def strip_step_left(E, up, site, down):
    """E (x, y, z) -> E' (a, r, b): absorb one column of a three-line strip from the left."""
    return np.einsum("xyz,xua,udyr,zdb->arb", E, up, site, down, optimize=True)


def strip_step_right(F, up, site, down):
    """F (a, r, b) -> F' (x, l, z): absorb one column of a three-line strip from the right."""
    return np.einsum("arb,xua,udlr,zdb->xlz", F, up, site, down, optimize=True)


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
    return np.einsum("xlz,xua,zdb,arb->udlr", E_left, up, down, F_right, optimize=True)


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

    def __init__(self, tensors, terms, cut):
        self.A = tensors
        self.L1 = len(tensors)
        self.L2 = len(tensors[0])
        self.terms = terms
        self.cut = cut
        self.site_number = self.L1 * self.L2

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

    def col_sites(self, conf, l2, flip=False):
        """Column l2 as a "row": (l, r, u, d) orientation; ``flip`` -> (r, l, u, d)."""
        out = []
        for l1 in range(self.L1):
            t = self.site(l1, l2, conf[l1, l2])
            out.append(t.transpose(3, 2, 0, 1) if flip else t.transpose(2, 3, 0, 1))
        return out


class Environment:
    """All boundaries and strips of one configuration (what the lazy DAG would hold)."""

    def __init__(self, peps, conf):
        self.peps = peps
        self.conf = conf
        self._up = {}
        self._down = {}
        self._left = {}
        self._right = {}
        self._row_envs = {}
        self._col_envs = {}

    # boundary families (single_layer_auxiliaries.py:430-456) ------------------------------
    def up(self, l1):
        """``_up_to_down[l1]``: rows 0..l1 compressed from the top; open legs point down."""
        p = self.peps
        if l1 == -1:
            return ones_line(p.L2)
        if l1 not in self._up:
            self._up[l1] = compress(self.up(l1 - 1), p.row_sites(self.conf, l1), p.cut)
        return self._up[l1]

    def down(self, l1):
        """``_down_to_up[l1]``: rows l1..L1-1 compressed from the bottom; open legs point up."""
        p = self.peps
        if l1 == p.L1:
            return ones_line(p.L2)
        if l1 not in self._down:
            self._down[l1] = compress(self.down(l1 + 1), p.row_sites(self.conf, l1, flip=True), p.cut)
        return self._down[l1]

    def left(self, l2):
        p = self.peps
        if l2 == -1:
            return ones_line(p.L1)
        if l2 not in self._left:
            self._left[l2] = compress(self.left(l2 - 1), p.col_sites(self.conf, l2), p.cut)
        return self._left[l2]

    def right(self, l2):
        p = self.peps
        if l2 == p.L2:
            return ones_line(p.L1)
        if l2 not in self._right:
            self._right[l2] = compress(self.right(l2 + 1), p.col_sites(self.conf, l2, flip=True), p.cut)
        return self._right[l2]

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
        return float(np.einsum("arb,arb->", e, F[l2 + 2]))

    def replace_vertical(self, l1, l2, s0, s1):
        """psi with sites (l1,l2),(l1+1,l2) set to s0,s1 (single_layer_auxiliaries.py:686-692)."""
        p = self.peps
        E, F = self.col_envs(l2)
        lf, rt = self.left(l2 - 1), self.right(l2 + 1)
        e = strip_step_left(E[l1], lf[l1], p.site(l1, l2, s0).transpose(2, 3, 0, 1), rt[l1])
        e = strip_step_left(e, lf[l1 + 1], p.site(l1 + 1, l2, s1).transpose(2, 3, 0, 1), rt[l1 + 1])
        return float(np.einsum("arb,arb->", e, F[l1 + 2]))

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

    def sweep(self):
        """``SweepSampling.__call__``: returns (possibility, configuration copy)."""
        peps = self.peps
        env = Environment(peps, self.conf)
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
                    env = Environment(peps, self.conf)
        return abs(ws)**2, self.conf.copy()


# ----------------------------------------------------------------------------------------------
# observer
# ----------------------------------------------------------------------------------------------
def observe(peps, conf):
    """Per-sample quantities of ``Observer.__call__`` (observer.py:313-415).

    Returns (ws, eloc, holes) with ``holes[l1][l2]`` of shape (u, d, l, r) already divided by
    ws (the sampled physical slice of ``Configuration.holes``)."""
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

    def __init__(self, peps):
        self.peps = peps
        self.count = 0
        self.total_weight = 0.0
        self.total_weight_square = 0.0
        self.total_log_ws = 0.0
        self.er = 0.0
        self.err = 0.0
        self.eerr = 0.0
        self.Delta = [[np.zeros_like(peps.A[l1][l2]) for l2 in range(peps.L2)] for l1 in range(peps.L1)]
        self.EDelta = [[np.zeros_like(peps.A[l1][l2]) for l2 in range(peps.L2)] for l1 in range(peps.L1)]

    def add(self, possibility, conf):
        self.count += 1
        ws, eloc, holes = observe(self.peps, conf)
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

    def gradient(self):
        """``Observer.gradient`` (observer.py:542-555) for real tensors."""
        energy = self.er / self.total_weight
        return [[2 * (self.EDelta[l1][l2] / self.total_weight - energy * self.Delta[l1][l2] / self.total_weight)
                 for l2 in range(self.peps.L2)] for l1 in range(self.peps.L1)]
