"""CPU restatement of tetragono's amplitudes and local energies for a fermionic PEPS, by exact graded
contraction (test infrastructure only; the checker for fermionic lattices, never the product).

* projection on the configuration: ``Configuration._get_shrinker`` / ``_shrink_configuration``
  (tetragono/tetragono/sampling_lattice/lattice.py:291-339): the site tensor contracted over ``P0``
  with a shrinker (legs ``P`` = [(s, 1)], ``Q`` = the conjugated physical edge, one element 1 at
  Q = (-s, index), P = (s, 0)); the dimension-one leg ``P_{l1}_{l2}_0`` stays open and carries the
  charge;
* the amplitude ``<s|psi>`` = ``hole(())``: here the whole network of projected tensors contracted
  exactly, row-major, with the graded contraction of ``oracle.fermi_tensor`` (which is independent
  of the order in which a network is contracted, so that with a cut large enough for the reference's
  boundary MPS to be exact the two agree up to the order of the open legs);
* ``tensor_element`` (tetragono/tetragono/tensor_element.py:20-108): every nonzero element of a
  Hamiltonian term as a one-element tensor with the term's names and arrows, keyed by the
  conjugated input points and the output points;
* E_loc (tetragono/tetragono/sampling_lattice/observer.py:344-392): per term and per output
  configuration s', ``(ws / |ws|^2) . H(s', s) . conj(wss)`` contracted over ``T`` and every ``P``
  leg, summed.
"""
import itertools

import numpy as np

from .fermi_tensor import FermiTensor

PHYSICS = (((0, 1), (1, 1)), False)   # spinless fermion site: empty (charge 0), occupied (charge 1)


def point(index):
    """Edge point (symmetry, index in segment) of physical index 0 / 1 on [(0, 1), (1, 1)]."""
    return (int(index), 0)


def shrink(site, l1, l2, index):
    """lattice.py:306-339 for the single orbit 0."""
    sym, k = point(index)
    conj = (tuple((-s, d) for s, d in PHYSICS[0]), not PHYSICS[1])
    shrinker = FermiTensor(["P", "Q"], [(((sym, 1),), False), conj])
    shrinker[{"Q": (-sym, k), "P": (sym, 0)}] = 1.0
    return site.contract(shrinker.edge_rename({"P": f"P_{l1}_{l2}_0"}), {("P0", "Q")})


def _bond_names(l1, l2):
    return {"R": f"H{l1}.{l2}", "L": f"H{l1}.{l2 - 1}", "D": f"V{l1}.{l2}", "U": f"V{l1 - 1}.{l2}"}


def amplitude(sites, conf):
    """The amplitude tensor (legs T and every P_{l1}_{l2}_0) of configuration ``conf[l1][l2]``."""
    L1, L2 = len(sites), len(sites[0])
    acc = None
    for l1, l2 in itertools.product(range(L1), range(L2)):
        t = shrink(sites[l1][l2], l1, l2, conf[l1][l2]).edge_rename(_bond_names(l1, l2))
        if acc is None:
            acc = t
            continue
        shared = {(n, n) for n in t.names if n in acc.names}
        acc = acc.contract(t, shared)
    return acc


def value(ws, names):
    """The element of amplitude tensor ``ws`` with its legs in the order ``names``."""
    return float(ws.transpose(list(names)).scalar())


def element_table(H):
    """tensor_element.py:72-108 for a term whose legs all have one-dimensional segments."""
    body = len(H.names) // 2
    table = {}
    for combo, sl in H._blocks():
        block = H.data[sl]
        for idx in itertools.product(*[range(n) for n in block.shape]):
            v = block[idx]
            if v == 0:
                continue
            points = [(H.edges[i][0][combo[i]][0], idx[i]) for i in range(len(H.names))]
            edges = [(((points[i][0], 1),), H.edges[i][1]) for i in range(len(H.names))]
            elem = FermiTensor(H.names, edges, H.group, np.full((1,) * len(H.names), v))
            key_in = tuple((-points[H.names.index(f"I{i}")][0], points[H.names.index(f"I{i}")][1]) for i in range(body))
            key_out = tuple(points[H.names.index(f"O{i}")] for i in range(body))
            table.setdefault(key_in, {})[key_out] = elem
    return table


def local_energy(sites, terms, conf):
    """E_loc of configuration ``conf`` (observer.py:344-392); ``terms`` = [(positions, H)], positions
    ((l1, l2, 0), ...)."""
    L1, L2 = len(sites), len(sites[0])
    ws = amplitude(sites, conf)
    if ws.norm_max() == 0:
        return None
    inv = ws / ws.norm_2()**2
    all_names = {(n, n) for n in ws.names}
    total = 0.0
    for positions, H in terms:
        table = element_table(H)
        here = tuple(point(conf[l1][l2]) for l1, l2, _ in positions)
        if here not in table:
            continue
        pnames = [f"P_{l1}_{l2}_{o}" for l1, l2, o in positions]
        for out, elem in table[here].items():
            new = [list(r) for r in conf]
            for (l1, l2, _), (sym, _k) in zip(positions, out):
                new[l1][l2] = sym
            wss = amplitude(sites, new)
            if wss.norm_max() == 0:
                continue
            v = inv.contract(elem, {(pnames[i], f"I{i}") for i in range(len(positions))})
            v = v.edge_rename({f"O{i}": pnames[i] for i in range(len(positions))})
            total += float(v.contract(wss.conjugate(), all_names).scalar())
    return total


# ----------------------------------------------------------------------------------------------
# the same amplitudes as a bosonic network (what a dense boundary-MPS contraction evaluates)
# ----------------------------------------------------------------------------------------------
# A graded network contracted in a linear order of its legs equals the plain (bosonic) sum over
# bond indices times, per index assignment, the product of: (-1)^p for every bond whose first leg
# in that order has arrow False; (-1)^(p_e p_f) for every pair of bonds whose ends interleave; and
# (-1)^(p_e * parity of the open legs between e's ends).  With the projected site legs in the
# order (T, U, D, L, R, P) and the sites taken row-major, charge conservation of every prefix of
# sites turns the non-local part into (a) a sign of the configuration alone and (b) a parity
# operator on each site's D leg raised to the number of particles to its left in its row; the
# rest is local to each site.  Taken column-major the same holds with the roles of the legs
# exchanged.  Per site, on the projected slice (which is (-1)^n times the stored slice of the
# occupation n, from the reversal of P0 when it is contracted with the shrinker):
#
#   row-major:    (-1)^( p_R (1 + n) + p_L p_D + p_D M_row )    M_row = particles left of the site
#   column-major: (-1)^( p_D (1 + n) + p_D p_L + p_D p_R + p_L p_U + p_R M_col )
#                                                               M_col = particles above the site
#
# and the configuration sign is prod over cuts k of (-1)^((N_<k + p_T)(N_<=k + p_T)), N counting
# the particles of the rows (columns) before / up to k, p_T the parity of the T leg.  Boundary-MPS
# truncation commutes with these signs: on every cut of a boundary line they are per-leg signs
# times a function of the two sides' total parities, so singular values and kept subspaces are
# those of the graded boundary state.

ROW, COL = 0, 1
_LEGS = ["U", "D", "L", "R"]


def _leg_parities(site):
    out = []
    for x in _LEGS:
        if x in site.names:
            e = site.edge_by_name(x)
            out.append(np.concatenate([np.full(d, (s & 1) == 1) for s, d in e[0]]).astype(np.int64))
        else:
            out.append(np.zeros(1, np.int64))
    return out


def leg_charges(site):
    """Per-index U(1) charges of the U, D, L, R legs (1 entry 0 for a missing leg)."""
    out = {}
    for x in _LEGS:
        if x in site.names:
            out[x] = [s for s, d in site.edge_by_name(x)[0] for _ in range(d)]
        else:
            out[x] = [0]
    return out


def projected_dense(site, l1, l2, n):
    """The graded projected tensor as a dense (u, d, l, r) array."""
    t = shrink(site, l1, l2, n)
    names = [x for x in ["T"] + _LEGS if x in t.names] + [f"P_{l1}_{l2}_0"]
    t = t.transpose(names)
    dims = [len(p) for p in _leg_parities(site)]
    return t.data.reshape(dims)


def bosonized_site(site, l1, l2, n, M, family):
    d = projected_dense(site, l1, l2, n)
    U, D, L, R = np.ix_(*_leg_parities(site))
    if family == ROW:
        e = (R * (1 - n)) ^ (L * D) ^ (D * (M & 1))
    else:
        e = (D * (1 - n)) ^ (D * L) ^ (D * R) ^ (L * U) ^ (R * (M & 1))
    return np.where(e.astype(bool), -d, d)


def prefix_counts(conf, family):
    conf = np.asarray(conf)
    if family == ROW:
        return np.cumsum(conf, axis=1) - conf
    return np.cumsum(conf, axis=0) - conf


def configuration_sign(conf, p_T, family):
    conf = np.asarray(conf)
    N = conf.sum(axis=1) if family == ROW else conf.sum(axis=0)
    s, before = 0, int(p_T)
    for k in range(len(N) - 1):
        upto = (before + int(N[k])) & 1
        s ^= before & upto
        before = upto
    return -1.0 if s else 1.0


def canonical_names(L1, L2, family):
    sites = [(a, b) for a in range(L1) for b in range(L2)] if family == ROW else \
            [(a, b) for b in range(L2) for a in range(L1)]
    return ["T"] + [f"P_{a}_{b}_0" for a, b in sites]


def amplitude_tensor(conf, value, T_symmetry, family):
    """A one-element amplitude tensor with the open legs in the family's canonical order."""
    conf = np.asarray(conf)
    L1, L2 = conf.shape
    names = canonical_names(L1, L2, family)
    edges = [(((T_symmetry, 1),), False)] + [(((int(conf[int(n.split("_")[1]), int(n.split("_")[2])]), 1),), False)
                                             for n in names[1:]]
    return FermiTensor(names, edges, data=np.full((1,) * len(names), value))


class BosonizedLattice:
    """A fermionic lattice evaluated through the dense (bosonic) boundary-MPS oracle: per
    configuration the projected slices carry the signs above, row-major for the row boundaries
    (amplitude, horizontal replacements) and column-major for the column boundaries (vertical
    replacements)."""

    def __init__(self, sites, cut):
        from .peps_oracle import DensePEPS
        self.sites = sites
        self.L1, self.L2 = len(sites), len(sites[0])
        self.cut = cut
        self.T_symmetry = sites[0][0].edge_by_name("T")[0][0][0]
        self.p_T = self.T_symmetry & 1
        legs = [[leg_charges(sites[a][b]) for b in range(self.L2)] for a in range(self.L1)]
        flux = [[(-self.T_symmetry if (a, b) == (0, 0) else 0) for b in range(self.L2)] for a in range(self.L1)]
        self.charges = (legs, [0, 1], flux)
        self._DensePEPS = DensePEPS

    def _peps(self, conf, family):
        conf = np.asarray(conf)
        M = prefix_counts(conf, family)
        A = []
        for a in range(self.L1):
            row = []
            for b in range(self.L2):
                n = int(conf[a, b])
                t = bosonized_site(self.sites[a][b], a, b, n, int(M[a, b]), family)
                full = np.zeros((2,) + t.shape)
                full[n] = t
                row.append(full)
            A.append(row)
        return self._DensePEPS(A, [], self.cut, charges=self.charges)

    def environments(self, conf):
        from .peps_oracle import Environment
        conf = np.asarray(conf)
        return {f: Environment(self._peps(conf, f), conf) for f in (ROW, COL)}

    def amplitude(self, envs):
        conf = envs[ROW].conf
        value = envs[ROW].amplitude() * configuration_sign(conf, self.p_T, ROW)
        return amplitude_tensor(conf, value, self.T_symmetry, ROW)

    def replace(self, envs, positions, new):
        """``Configuration.replace`` of a nearest-neighbour pair as the reference dispatches it
        (single_layer_auxiliaries.py:568-692): a row strip for a horizontal pair, a column strip for a
        vertical one."""
        conf = envs[ROW].conf
        changed = [(p, s) for p, s in zip(positions, new) if conf[p[0], p[1]] != s]
        if not changed:
            return self.amplitude(envs)
        (p0, s0), (p1, s1) = sorted(changed)
        after = conf.copy()
        after[p0[0], p0[1]], after[p1[0], p1[1]] = s0, s1
        family = ROW if p0[0] == p1[0] else COL
        env = envs[family]
        M = prefix_counts(after, family)
        for (a, b), s in ((p0[:2], s0), (p1[:2], s1)):
            env.peps.A[a][b][s] = bosonized_site(self.sites[a][b], a, b, s, int(M[a, b]), family)
        if family == ROW:
            value = env.replace_horizontal(p0[0], p0[1], s0, s1)
        else:
            value = env.replace_vertical(p0[0], p0[1], s0, s1)
        value *= configuration_sign(after, self.p_T, family)
        return amplitude_tensor(after, value, self.T_symmetry, family)

    def local_energy(self, terms, conf):
        """E_loc through the bosonic environments, with the graded pairing of observer.py:378-383."""
        conf = np.asarray(conf)
        envs = self.environments(conf)
        ws = self.amplitude(envs)
        if ws.norm_max() == 0:
            return None
        return _pair_energy(ws, terms, conf, lambda positions, new: self.replace(envs, positions, new))


def _pair_energy(ws, terms, conf, replaced):
    inv = ws / ws.norm_2()**2
    all_names = {(n, n) for n in ws.names}
    total = 0.0
    for positions, H in terms:
        table = element_table(H)
        here = tuple(point(conf[l1][l2]) for l1, l2, _ in positions)
        if here not in table:
            continue
        pnames = [f"P_{l1}_{l2}_{o}" for l1, l2, o in positions]
        for out, elem in table[here].items():
            wss = replaced([p[:2] for p in positions], [sym for sym, _ in out])
            if wss.norm_max() == 0:
                continue
            v = inv.contract(elem, {(pnames[i], f"I{i}") for i in range(len(positions))})
            v = v.edge_rename({f"O{i}": pnames[i] for i in range(len(positions))})
            total += float(v.contract(wss.conjugate(), all_names).scalar())
    return total


def hop_sign(conf, positions, new):
    """The graded pairing of observer.py:378-383 for one term, in closed form, with both amplitudes
    in the row-major canonical order: 1 for a diagonal element; for a particle moved between sites
    i < j (row-major), (-1)^(particles strictly between them), times -1 when it moves from i to j."""
    conf = np.asarray(conf)
    L2 = conf.shape[1]
    idx = [a * L2 + b for a, b in positions]
    flat = conf.reshape(-1)
    if all(flat[i] == s for i, s in zip(idx, new)):
        return 1.0
    i, j = sorted(idx)
    between = int(flat[i + 1:j].sum()) & 1
    forward = flat[i] == 1 and dict(zip(idx, new))[i] == 0
    return (-1.0 if between else 1.0) * (-1.0 if forward else 1.0)


def order_sign(conf, names_from, names_to, T_symmetry):
    """Sign of reordering the one-element amplitude tensor's legs (only odd legs exchange)."""
    conf = np.asarray(conf)
    edges = [(((T_symmetry, 1),), False) if n == "T" else
             (((int(conf[int(n.split("_")[1]), int(n.split("_")[2])]), 1),), False) for n in names_from]
    t = FermiTensor(list(names_from), edges, data=np.ones((1,) * len(edges)))
    return float(t.transpose(list(names_to)).scalar())


def order_sign_by_count(conf, names_from, names_to, T_symmetry):
    """``order_sign`` without building the tensor (any number of legs): a reordering of dimension-1
    legs exchanges pairs of legs, and only pairs whose legs are both odd contribute a sign
    (TAT/include/TAT/implement/edge_operator.hpp:521-555), so the sign is (-1)^(inversions among the
    odd legs)."""
    conf = np.asarray(conf)

    def parity(n):
        if n == "T":
            return int(T_symmetry) & 1
        return int(conf[int(n.split("_")[1]), int(n.split("_")[2])]) & 1

    odd = [n for n in names_from if parity(n)]
    pos = {n: i for i, n in enumerate(names_to)}
    seq = [pos[n] for n in odd]
    inv = sum(1 for i in range(len(seq)) for j in range(i + 1, len(seq)) if seq[i] > seq[j])
    return -1.0 if inv & 1 else 1.0


def hole_network(sites, conf, l1, l2):
    """``hole(((l1, l2),))`` exactly (single_layer_auxiliaries.py:721-736): every projected tensor but
    the one at (l1, l2), contracted; the bonds to (l1, l2) stay open, named as the reference names
    them (``R0`` the left neighbour's R leg, ``L0`` the right neighbour's L leg, ``U0`` the lower
    neighbour's U leg, ``D0`` the upper neighbour's D leg)."""
    L1, L2 = len(sites), len(sites[0])
    acc = None
    for a, b in itertools.product(range(L1), range(L2)):
        if (a, b) == (l1, l2):
            continue
        t = shrink(sites[a][b], a, b, conf[a][b]).edge_rename(_bond_names(a, b))
        acc = t if acc is None else acc.contract(t, {(n, n) for n in t.names if n in acc.names})
    return acc.edge_rename({f"H{l1}.{l2 - 1}": "R0", f"H{l1}.{l2}": "L0", f"V{l1 - 1}.{l2}": "D0", f"V{l1}.{l2}": "U0"})


def holes(sites, conf):
    """``Configuration.holes`` (lattice.py:362-416): <psi|s|d psi / d A[l1,l2]> / <psi|s|psi> as tensors
    with the site's names and conjugated edges, expanded to the full physical leg by the shrinker."""
    L1, L2 = len(sites), len(sites[0])
    ws = amplitude(sites, conf)
    inv_ws = (ws / ws.norm_2()**2).conjugate()
    out = [[None] * L2 for _ in range(L1)]
    for l1, l2 in itertools.product(range(L1), range(L2)):
        h = hole_network(sites, conf, l1, l2)
        own = f"P_{l1}_{l2}_0"
        names = {(n, n) for n in ws.names if n != own and n in h.names}
        h = h.contract(inv_ws, names)
        h = h.edge_rename({"L0": "R", "R0": "L", "U0": "D", "D0": "U", own: "P0"})
        sym, k = point(conf[l1][l2])
        conj = (tuple((-s, d) for s, d in PHYSICS[0]), not PHYSICS[1])
        shrinker = FermiTensor(["P", "Q"], [(((sym, 1),), False), conj])
        shrinker[{"Q": (-sym, k), "P": (sym, 0)}] = 1.0
        out[l1][l2] = h.contract(shrinker, {("P0", "P")}).edge_rename({"Q": "P0"})
    return out


# ----------------------------------------------------------------------------------------------
# gradient through the bosonic holes
# ----------------------------------------------------------------------------------------------
# A hole H satisfies A . H = psi(A) / psi(A0), so in the site's leg order H[e] = kappa(e) *
# (d psi / d A[e]) / psi, kappa the sign of TAT's full contraction of A with H:
# (-1)^(n + p_T + p_D + p_R + [n_odd = 2 mod 4]) (the reversal of A's arrow-False legs and the merge
# sign of its common group, contract.hpp:381-402, 487-500).  The gradient is conjugate(True) of a sum
# of holes (observer.py:542-555, utility.py:230-231); on a tensor with the hole's arrows that
# conjugation multiplies each block by the same kappa, so the two cancel: in the site's own leg order
#
#   gradient[n, e] = (-1)^(n + p_R (1 + n) + p_L p_D) * 2 (E Delta_B / W - E Delta_B / W)[n, e]
#
# where Delta_B accumulates the row-strip bosonic holes d psi_B / d B / psi_B, each multiplied by the
# sample's own prefix parity (-1)^(p_D M_row) before it is added.


def gradient_sign(site, n):
    """(-1)^(n + p_R (1 + n) + p_L p_D) as a (u, d, l, r) array."""
    U, D, L, R = np.ix_(*_leg_parities(site))
    e = (n + R * (1 + n) + L * D) & 1
    return np.where(e.astype(bool), -1.0, 1.0) * np.ones([len(p) for p in _leg_parities(site)])


def signed_hole(lattice, envs, l1, l2):
    """The row-strip bosonic hole of (l1, l2) divided by psi_B, with the prefix parity applied."""
    env = envs[ROW]
    h = env.site_hole(l1, l2) / env.amplitude()
    M = int(prefix_counts(env.conf, ROW)[l1, l2])
    pD = _leg_parities(lattice.sites[l1][l2])[1]
    return np.where((pD[None, :, None, None] * (M & 1)).astype(bool), -h, h)


def site_gradients(lattice, samples):
    """Gradient tensors (dense (n, u, d, l, r) in the site's leg order) from samples of
    (configuration, reweight, E_loc), as Observer.gradient forms them."""
    L1, L2 = lattice.L1, lattice.L2
    W = sum(rw for _, rw, _ in samples)
    E = sum(rw * e for _, rw, e in samples) / W
    out = []
    for l1 in range(L1):
        row = []
        for l2 in range(L2):
            shape = (2,) + tuple(len(p) for p in _leg_parities(lattice.sites[l1][l2]))
            d, ed = np.zeros(shape), np.zeros(shape)
            for conf, rw, e in samples:
                envs = lattice.environments(conf)
                h = signed_hole(lattice, envs, l1, l2)
                n = int(np.asarray(conf)[l1, l2])
                d[n] += rw * h
                ed[n] += rw * e * h
            g = 2 * (ed / W - E * d / W)
            for n in (0, 1):
                g[n] *= gradient_sign(lattice.sites[l1][l2], n)
            row.append(g)
        out.append(row)
    return out


# ----------------------------------------------------------------------------------------------
# E_loc from bosonic strip values and integer signs only
# ----------------------------------------------------------------------------------------------
def order_inversions(conf):
    """Parity of the pairs of occupied sites that column-major and row-major orders put in opposite
    order (a site strictly left of and below another): the sign of reordering the amplitude's odd
    P legs from the column-major to the row-major canonical order."""
    conf = np.asarray(conf)
    L1, L2 = conf.shape
    count = 0
    for a, b in itertools.product(range(L1), range(L2)):
        if conf[a, b]:
            count += int(conf[:a, b + 1:].sum())
    return count & 1


def local_energy_signs(lattice, terms, conf):
    """E_loc = sum over terms and outputs of h * hop_sign * sigma * psi_B(s') / psi_B(s), with psi_B(s)
    the row-strip value, psi_B(s') the row-strip (horizontal pair) or column-strip (vertical pair)
    replacement, and sigma = 1 for a horizontal pair, G_col(s') G_row(s) (-1)^inversions(s') for a
    vertical one."""
    conf = np.asarray(conf)
    envs = lattice.environments(conf)
    psi = envs[ROW].amplitude()
    if psi == 0:
        return None
    g_row = configuration_sign(conf, lattice.p_T, ROW)
    total = 0.0
    for positions, H in terms:
        table = element_table(H)
        here = tuple(point(conf[a][b]) for a, b, _ in positions)
        for out, elem in table.get(here, {}).items():
            new = [sym for sym, _ in out]
            pos = [p[:2] for p in positions]
            h = float(elem.data.reshape(-1)[0])
            changed = [(p, s) for p, s in zip(pos, new) if conf[p] != s]
            if not changed:
                total += h
                continue
            (p0, s0), (p1, s1) = sorted(changed)
            after = conf.copy()
            after[p0], after[p1] = s0, s1
            family = ROW if p0[0] == p1[0] else COL
            env = envs[family]
            M = prefix_counts(after, family)
            for (a, b), s in ((p0, s0), (p1, s1)):
                env.peps.A[a][b][s] = bosonized_site(lattice.sites[a][b], a, b, s, int(M[a, b]), family)
            if family == ROW:
                wss = env.replace_horizontal(p0[0], p0[1], s0, s1)
                sigma = 1.0
            else:
                wss = env.replace_vertical(p0[0], p0[1], s0, s1)
                sigma = configuration_sign(after, lattice.p_T, COL) * g_row * (-1.0)**order_inversions(after)
            if wss == 0.0:
                continue
            total += h * hop_sign(conf, pos, new) * sigma * wss / psi
    return total


def natural_gradient(lattice, samples, step, error):
    """``natural_gradient_by_conjugate_gradient`` (observer.py:576-675) on the bosonic rows: each
    sample's row is its prefix-signed row-strip holes laid out per site as (n, u, d, l, r); the
    reference's rows are the same numbers up to one fixed sign and order per element, under which the
    conjugate-gradient iteration is covariant, and its final ``conjugate(True)`` of the solution is
    the same per-element fold as the gradient's."""
    L1, L2 = lattice.L1, lattice.L2
    shapes = [[(2,) + tuple(len(p) for p in _leg_parities(lattice.sites[a][b])) for b in range(L2)] for a in range(L1)]
    sizes = [int(np.prod(shapes[a][b])) for a in range(L1) for b in range(L2)]
    rows, W, EW = [], 0.0, 0.0
    for conf, rw, e in samples:
        envs = lattice.environments(conf)
        parts = []
        for a in range(L1):
            for b in range(L2):
                full = np.zeros(shapes[a][b])
                full[int(np.asarray(conf)[a, b])] = signed_hole(lattice, envs, a, b)
                parts.append(full.ravel())
        rows.append(np.concatenate(parts))
        W += rw
        EW += rw * e
    E = EW / W
    rows = np.array(rows)
    rw = np.array([s[1] for s in samples])
    es = np.array([s[2] for s in samples])
    delta = (rw[:, None] * rows).sum(axis=0) / W
    param = np.sqrt(rw / W)
    Delta = (rows - delta) * param[:, None]
    Energy = (es - E) * param

    def A(v):
        return Delta.T @ (Delta @ v)

    b = Delta.T @ Energy
    b_square = float(b @ b)
    x = np.zeros_like(b)
    r = b - A(x)
    p = r
    r_square = float(r @ r)
    t = 0
    while t != step and not (error != 0.0 and error**2 > r_square / b_square):
        Dp = Delta @ p
        alpha = r_square / float(Dp @ Dp)
        x = x + alpha * p
        r = r - alpha * (Delta.T @ Dp)
        new = float(r @ r)
        p = r + (new / r_square) * p
        r_square = new
        t += 1
    x = 2 * x
    out, k = [], 0
    for a in range(L1):
        row = []
        for b in range(L2):
            g = x[k:k + sizes[a * L2 + b]].reshape(shapes[a][b]).copy()
            k += sizes[a * L2 + b]
            for n in (0, 1):
                g[n] *= gradient_sign(lattice.sites[a][b], n)
            row.append(g)
        out.append(row)
    return out


class FermionSweepChain:
    """One chain of ``SweepSampling`` (sampling.py:117-154) on a fermionic lattice: the reference's
    proposal order, RNG draws and acceptance |psi(s')/psi(s)|^2 n/n', with amplitudes from the
    bosonized row / column strips (a boundary depends only on the rows or columns it covers, so
    fresh environments after an accepted hop equal the reference's lazily kept ones)."""

    def __init__(self, lattice, terms, conf, seed):
        from .peps_oracle import sweep_order
        from .rng import MT19937_64
        self.lattice = lattice
        self.conf = np.array(conf, dtype=np.int64)
        self.engine = MT19937_64(seed)
        self.terms = []
        for positions, H in terms:
            table = {}
            for key_in, outs in element_table(H).items():
                table[tuple(s for s, _ in key_in)] = [(tuple(s for s, _ in key_out), float(e.data.reshape(-1)[0]))
                                                      for key_out, e in outs.items()]
            self.terms.append((positions, table))

        class _Order:
            pass
        shape = _Order()
        shape.terms, shape.L1, shape.L2 = self.terms, lattice.L1, lattice.L2
        self.order = sweep_order(shape)

    def sweep(self):
        from .rng import uniform_int, uniform_real01
        lat = self.lattice
        envs = lat.environments(self.conf)
        ws = float(lat.amplitude(envs).data.reshape(-1)[0])
        for ti in self.order:
            positions, table = self.terms[ti]
            s = tuple(int(self.conf[p[0], p[1]]) for p in positions)
            if s not in table or not table[s]:
                continue
            hops = table[s]
            n = len(hops)
            s_new = hops[uniform_int(self.engine, 0, n - 1)][0]
            n_new = len(table[s_new])
            wss = float(lat.replace(envs, [p[:2] for p in positions], list(s_new)).data.reshape(-1)[0])
            p = abs(wss / ws)**2 * n / n_new
            if uniform_real01(self.engine) < p:
                ws = wss
                if s_new != s:
                    for pos, v in zip(positions, s_new):
                        self.conf[pos[0], pos[1]] = v
                    envs = lat.environments(self.conf)
        return abs(ws)**2, self.conf.copy()
