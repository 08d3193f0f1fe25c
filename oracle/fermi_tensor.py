"""CPU restatement of TAT's fermionic (Z2-graded) block tensors.

TEST INFRASTRUCTURE ONLY: the checker for fermionic tensors, imported by tests and never by the
product.  A tensor is held densely (every block of the block-sparse layout laid out at its segment
offsets, zeros elsewhere) together with TAT's edge description, so that every operation is the
bosonic index operation times a sign that depends only on the parities of the indices' segments.
The signs follow TAT, file by file:

* ``edge_operator`` (TAT/include/TAT/implement/edge_operator.hpp:33-692): split, reverse, transpose,
  reverse-before-merge and merge in one pass.  Per block at the transposition stage the sign is the
  XOR of

  - a reversed edge of odd parity, where the reversal is marked (edge_operator.hpp:497-520); a
    reversal before the transposition and one before the merge cancel on the same edge;
  - every pair of odd edges whose order the transposition exchanges (:521-555), always applied;
  - every merged group of more than one edge whose count of odd edges has bit 1 set,
    ``(count & 2) != 0`` (:591), where the merge is marked;
  - the same for every split group (:612);

  marks are "apply" unless the edge is named in the exclusion set when ``apply_parity`` is true,
  and "do not apply" unless it is named there when it is false (:455-483).  A merged edge takes the
  arrow of its first member; members with the other arrow are reversed (:331-349).  The merged
  edge's segments appear in the order in which their symmetries are first met while running over
  the members' segments in row-major order, and each combination of member segments occupies the
  next slice of its merged segment (:352-390); a split inverts that layout (:140-188).
* ``transpose`` / ``reverse_edge`` / ``merge_edge`` / ``split_edge``
  (TAT/include/TAT/structure/tensor.hpp:791-835, TAT/include/TAT/implement/split_and_merge.hpp:27-109):
  the merged edge is put where the last member of its group stood.
* ``conjugate`` (TAT/include/TAT/implement/conjugate.hpp:30-122): symmetries negated, arrows flipped,
  block sign ``((n_odd & 2) != 0) ^ XOR(odd and arrow and trivial_metric)``.
* ``contract`` (TAT/include/TAT/implement/contract.hpp:306-620): free edges reversed to arrow False
  and common edges of the first tensor to True (sign only on that first tensor's common edges),
  both tensors merged into (free, common) matrices with the merge sign on the first tensor's common
  group, one product per sector with factor -1 on odd sectors when the two common groups sit on
  the same side (``put_common_1_right ^ !put_common_2_right``, :571-580), then split and reversed
  back without sign.  The side on which each common group is put follows the reference's choice
  (:405-473).
* ``__getitem__`` / ``storage`` / ``range_``: TAT's block order, blocks of zero total symmetry in
  row-major order of segment positions, each block row-major
  (TAT/include/TAT/structure/core.hpp:152-191).

The symmetry groups are Fermi U(1) (integer charge, odd charges are odd) and Fermi Z2 (0/1).
"""

import itertools

import numpy as np

C1 = "\x00contract_1"
C2 = "\x00contract_2"


class _U1:
    name = "U1"
    zero = 0

    @staticmethod
    def add(a, b):
        return a + b

    @staticmethod
    def neg(a):
        return -a

    @staticmethod
    def parity(a):
        return (int(a) & 1) == 1


class _Z2:
    name = "Z2"
    zero = 0

    @staticmethod
    def add(a, b):
        return int(a) ^ int(b)

    @staticmethod
    def neg(a):
        return int(a)

    @staticmethod
    def parity(a):
        return bool(a)


GROUPS = {"U1": _U1, "Z2": _Z2}


def _norm_symmetry(group, s):
    return int(s) if group is _U1 else int(bool(s))


def make_edge(group, spec):
    """``spec`` as PyTAT takes it: a segment list, or ``(segments, arrow)``; a segment is
    ``(symmetry, dimension)`` or a bare symmetry of dimension 1."""
    if isinstance(spec, tuple) and len(spec) == 2 and isinstance(spec[1], (bool, np.bool_)):
        segs, arrow = spec
    else:
        segs, arrow = spec, False
    out = []
    for s in segs:
        if isinstance(s, tuple):
            out.append((_norm_symmetry(group, s[0]), int(s[1])))
        else:
            out.append((_norm_symmetry(group, s), 1))
    return (tuple(out), bool(arrow))


def _dim(edge):
    return sum(d for _, d in edge[0])


def _starts(edge):
    st, acc = [], 0
    for _, d in edge[0]:
        st.append(acc)
        acc += d
    return st


def _index_symmetry(edge):
    return np.concatenate([np.full(d, s, dtype=np.int64) for s, d in edge[0]] or [np.zeros(0, np.int64)])


def _index_parity(group, edge):
    return np.concatenate([np.full(d, group.parity(s), dtype=bool) for s, d in edge[0]] or [np.zeros(0, bool)])


def _position(edge, symmetry):
    for j, (s, _) in enumerate(edge[0]):
        if s == symmetry:
            return j
    return None


def _bcast(v, axis, rank):
    shape = [1] * rank
    shape[axis] = len(v)
    return v.reshape(shape)


def _combination_layout(group, member_edges, target_edge=None):
    """Row-major run over the members' segment combinations (edge_operator.hpp:156-188, 352-390).

    Returns (segments of the fused edge, index map): the index map has the members' dense shape and
    gives each members' multi-index its dense index on the fused edge (-1 where a split's source
    edge has no segment of that symmetry).  With ``target_edge`` (a split) the fused edge is the
    given one; otherwise (a merge) it is built in order of first appearance."""
    seg_lists = [e[0] for e in member_edges]
    merged = [] if target_edge is None else [list(sd) for sd in target_edge[0]]
    bank = [0] * len(merged)
    combos = []
    for combo in itertools.product(*[range(len(sl)) for sl in seg_lists]):
        sym = group.zero
        size = 1
        for m, j in enumerate(combo):
            sym = group.add(sym, seg_lists[m][j][0])
            size *= seg_lists[m][j][1]
        if target_edge is None:
            pos = next((k for k, (s, _) in enumerate(merged) if s == sym), None)
            if pos is None:
                merged.append([sym, 0])
                bank.append(0)
                pos = len(merged) - 1
            offset = merged[pos][1]
            merged[pos][1] += size
        else:
            pos = _position(target_edge, sym)
            if pos is None:
                combos.append((combo, None, 0))
                continue
            offset = bank[pos]
            bank[pos] += size
        combos.append((combo, pos, offset))
    fused = (tuple((s, d) for s, d in merged), None)
    fstarts = _starts(fused)
    mstarts = [_starts(e) for e in member_edges]
    index = np.full(tuple(_dim(e) for e in member_edges), -1, dtype=np.int64)
    for combo, pos, offset in combos:
        if pos is None:
            continue
        dims = [seg_lists[m][j][1] for m, j in enumerate(combo)]
        local = np.arange(int(np.prod(dims))).reshape(dims) if dims else np.zeros((), np.int64)
        sl = tuple(slice(mstarts[m][j], mstarts[m][j] + seg_lists[m][j][1]) for m, j in enumerate(combo))
        index[sl] = fstarts[pos] + offset + local
    return fused[0], index


class FermiTensor:
    """Dense image of a TAT fermionic tensor: ``names``, ``edges`` ((segments, arrow) per edge)
    and ``data`` (float64 or complex128, zeros outside the blocks of zero total symmetry)."""

    def __init__(self, names, edges, group="U1", data=None, dtype=np.float64):
        self.group = GROUPS[group] if isinstance(group, str) else group
        self.names = list(names)
        self.edges = [make_edge(self.group, e) for e in edges]
        shape = tuple(_dim(e) for e in self.edges)
        self.data = np.zeros(shape, dtype=dtype) if data is None else np.asarray(data).reshape(shape)

    # ---- layout ------------------------------------------------------------------------------
    def parities(self):
        return [_index_parity(self.group, e) for e in self.edges]

    def allowed(self):
        """Mask of the elements inside blocks of zero total symmetry."""
        r = len(self.edges)
        tot = np.zeros(self.data.shape, dtype=np.int64)
        for i, e in enumerate(self.edges):
            v = _bcast(_index_symmetry(e), i, r)
            tot = (tot + v) if self.group is _U1 else (tot ^ v)
        return tot == 0

    def _blocks(self):
        starts = [_starts(e) for e in self.edges]
        for combo in itertools.product(*[range(len(e[0])) for e in self.edges]):
            sym = self.group.zero
            for i, j in enumerate(combo):
                sym = self.group.add(sym, self.edges[i][0][j][0])
            if sym != self.group.zero:
                continue
            yield combo, tuple(slice(starts[i][j], starts[i][j] + self.edges[i][0][j][1]) for i, j in enumerate(combo))

    def storage(self):
        if not self.edges:
            return self.data.reshape(1).copy()
        parts = [self.data[sl].ravel() for _, sl in self._blocks()]
        return np.concatenate(parts) if parts else np.zeros(0, self.data.dtype)

    def set_storage(self, storage):
        storage = np.asarray(storage)
        if not self.edges:
            self.data = storage.reshape(()).astype(self.data.dtype)
            return self
        self.data[...] = 0
        k = 0
        for _, sl in self._blocks():
            n = int(np.prod([s.stop - s.start for s in sl]))
            self.data[sl] = storage[k:k + n].reshape([s.stop - s.start for s in sl])
            k += n
        if k != storage.size:
            raise ValueError("storage size does not match the blocks")
        return self

    def range_(self, first=0, step=1):
        n = self.storage().size
        return self.set_storage(first + step * np.arange(n, dtype=self.data.dtype))

    def copy(self):
        return FermiTensor(self.names, self.edges, self.group, self.data.copy())

    def __getitem__(self, where):
        idx = []
        for n, e in zip(self.names, self.edges):
            sym, k = where[n]
            j = _position(e, _norm_symmetry(self.group, sym))
            idx.append(_starts(e)[j] + k)
        return self.data[tuple(idx)]

    def __setitem__(self, where, value):
        idx = []
        for n, e in zip(self.names, self.edges):
            sym, k = where[n]
            j = _position(e, _norm_symmetry(self.group, sym))
            idx.append(_starts(e)[j] + k)
        self.data[tuple(idx)] = value

    def scalar(self):
        """``Tensor::operator scalar_t`` (TAT/include/TAT/structure/tensor.hpp:394-401): the first stored
        element, 0 when there is none."""
        s = self.storage()
        return s[0] if s.size else 0.0

    def norm_max(self):
        return float(np.abs(self.data).max()) if self.data.size else 0.0

    def norm_2(self):
        return float(np.sqrt((np.abs(self.data)**2).sum()))

    def edge_by_name(self, name):
        return self.edges[self.names.index(name)]

    # ---- edge operations ---------------------------------------------------------------------
    def edge_rename(self, mapping):
        return FermiTensor([mapping.get(n, n) for n in self.names], self.edges, self.group, self.data)

    def edge_operator(self, split_map, reversed_names, merge_map, new_names, apply_parity=False,
                      exclude_split=(), exclude_reversed_before=(), exclude_reversed_after=(), exclude_merge=()):
        """edge_operator.hpp:33-692 with no cut."""
        g = self.group

        def mark(name, excluded):
            return (name not in excluded) if apply_parity else (name in excluded)

        # split (top-down)
        data = self.data
        names_s, edges_s, split_groups = [], [], []   # split_groups: (old name, [after-split indices])
        axis = 0
        for i, (n, e) in enumerate(zip(self.names, self.edges)):
            if n in split_map:
                parts = split_map[n]
                members = [make_edge(g, (list(segs), e[1])) for _, segs in parts]
                _, index = _combination_layout(g, members, target_edge=e)
                flat = index.ravel()
                taken = np.take(data, np.where(flat < 0, 0, flat), axis=axis)
                if (flat < 0).any():
                    mask = _bcast(flat >= 0, axis, taken.ndim)
                    taken = np.where(mask, taken, 0)
                data = taken.reshape(data.shape[:axis] + index.shape + data.shape[axis + 1:])
                first = len(names_s)
                for (nn, _), me in zip(parts, members):
                    names_s.append(nn)
                    edges_s.append(me)
                split_groups.append((n, list(range(first, len(names_s)))))
                axis += len(members)
            else:
                names_s.append(n)
                edges_s.append(e)
                split_groups.append((n, [len(names_s) - 1]))
                axis += 1
        rank_t = len(names_s)

        # reverse before transposition
        rev_before = [n in reversed_names for n in names_s]
        edges_bt = [(e[0], (not e[1]) if r else e[1]) for e, r in zip(edges_s, rev_before)]

        # names before merge (bottom-up) and the transposition plan
        names_bm, merge_groups = [], []
        for n in new_names:
            if n in merge_map:
                group = list(merge_map[n])
            else:
                group = [n]
            merge_groups.append((n, list(range(len(names_bm), len(names_bm) + len(group)))))
            names_bm.extend(group)
        if sorted(names_bm) != sorted(names_s):
            raise ValueError("edge operator with incompatible name lists")
        d2s = [names_s.index(n) for n in names_bm]
        data = np.transpose(data, d2s) if rank_t else data
        edges_bm = [edges_bt[s] for s in d2s]

        # reverse before merge: a group takes the arrow of its first member
        rev_after = [False] * rank_t
        for n, members in merge_groups:
            if not members:
                continue
            arrow = edges_bm[members[0]][1]
            for m in members:
                if edges_bm[m][1] != arrow:
                    edges_bm[m] = (edges_bm[m][0], arrow)
                    rev_after[m] = True

        # signs
        par = [_index_parity(g, e) for e in edges_bm]
        sign = np.zeros(data.shape, dtype=bool)
        for i in range(rank_t):
            flag = (rev_after[i] and mark(names_bm[i], exclude_reversed_after)) ^ \
                   (rev_before[d2s[i]] and mark(names_s[d2s[i]], exclude_reversed_before))
            if flag:
                sign ^= _bcast(par[i], i, rank_t)
        for i in range(rank_t):
            for j in range(i + 1, rank_t):
                if d2s[i] > d2s[j]:
                    sign ^= _bcast(par[i], i, rank_t) & _bcast(par[j], j, rank_t)
        s2d = {s: d for d, s in enumerate(d2s)}
        for n, members in merge_groups:
            if len(members) != 1 and mark(n, exclude_merge):
                cnt = sum((_bcast(par[m].astype(np.int64), m, rank_t) for m in members), np.zeros((), np.int64))
                sign ^= (cnt & 2) != 0
        for n, members in split_groups:
            if len(members) != 1 and mark(n, exclude_split):
                cnt = sum((_bcast(par[s2d[m]].astype(np.int64), s2d[m], rank_t) for m in members),
                          np.zeros((), np.int64))
                sign ^= (cnt & 2) != 0
        data = np.where(sign, -data, data)

        # merge
        out_edges = []
        axis = 0
        for n, members in merge_groups:
            if len(members) == 1:
                out_edges.append(edges_bm[members[0]])
                axis += 1
                continue
            if not members:
                data = np.expand_dims(data, axis)
                out_edges.append((((g.zero, 1),), False))
                axis += 1
                continue
            member_edges = [edges_bm[m] for m in members]
            segs, index = _combination_layout(g, member_edges)
            k = len(members)
            sh = data.shape
            flat = data.reshape(sh[:axis] + (int(np.prod(sh[axis:axis + k])),) + sh[axis + k:])
            merged_dim = sum(d for _, d in segs)
            out = np.zeros(sh[:axis] + (merged_dim,) + sh[axis + k:], dtype=data.dtype)
            sel = [slice(None)] * out.ndim
            sel[axis] = index.ravel()
            out[tuple(sel)] = flat
            data = out
            out_edges.append((segs, member_edges[0][1]))
            axis += 1
        return FermiTensor(new_names, out_edges, g, data)

    def transpose(self, names):
        if list(names) == self.names:
            return self
        return self.edge_operator({}, set(), {}, list(names))

    def reverse_edge(self, names, apply_parity=False, exclude=()):
        return self.edge_operator({}, set(names), {}, self.names, apply_parity, exclude_reversed_before=set(exclude))

    def merge_edge(self, merge, apply_parity=False, exclude_merge=(), exclude_reverse=()):
        target = []
        for n in reversed(self.names):
            found = False
            for new, group in merge.items():
                if n in group:
                    if n == group[-1]:
                        target.append(new)
                    found = True
                    break
            if not found:
                target.append(n)
        for new, group in merge.items():
            if not group:
                target.append(new)
        target.reverse()
        return self.edge_operator({}, set(), merge, target, apply_parity, exclude_reversed_after=set(exclude_reverse),
                                  exclude_merge=set(exclude_merge))

    def split_edge(self, split, apply_parity=False, exclude_split=()):
        target = []
        for n in self.names:
            if n in split:
                target.extend(nn for nn, _ in split[n])
            else:
                target.append(n)
        return self.edge_operator(split, set(), {}, target, apply_parity, exclude_split=set(exclude_split))

    def conjugate(self, trivial_metric=False):
        g = self.group
        r = len(self.edges)
        cnt = np.zeros(self.data.shape, dtype=np.int64)
        flip = np.zeros(self.data.shape, dtype=bool)
        for i, e in enumerate(self.edges):
            p = _bcast(_index_parity(g, e), i, r)
            cnt = cnt + p.astype(np.int64)
            if e[1] and trivial_metric:
                flip = flip ^ p
        sign = flip ^ ((cnt & 2) != 0)
        data = np.conj(self.data) if np.iscomplexobj(self.data) else self.data.copy()
        data = np.where(sign, -data, data)
        edges = [(tuple((g.neg(s), d) for s, d in e[0]), not e[1]) for e in self.edges]
        return FermiTensor(self.names, edges, g, data)

    def storage_size(self):
        return int(self.allowed().sum()) if self.edges else 1

    def contract(self, other, pairs):
        return contract(self, other, pairs)

    def __mul__(self, x):
        return FermiTensor(self.names, self.edges, self.group, self.data * x)

    __rmul__ = __mul__

    def __truediv__(self, x):
        return FermiTensor(self.names, self.edges, self.group, self.data / x)

    def __add__(self, other):
        other = other.transpose(self.names)
        return FermiTensor(self.names, self.edges, self.group, self.data + other.data)

    def __sub__(self, other):
        other = other.transpose(self.names)
        return FermiTensor(self.names, self.edges, self.group, self.data - other.data)


def contract(t1, t2, pairs):
    """contract_without_fuse, TAT/include/TAT/implement/contract.hpp:306-620."""
    g = t1.group
    m12 = {a: b for a, b in pairs}
    m21 = {b: a for a, b in pairs}
    free1 = [n for n in t1.names if n not in m12]
    free2 = [n for n in t2.names if n not in m21]
    rev1 = {n for n, e in zip(t1.names, t1.edges) if (n not in m12 and e[1]) or (n in m12 and not e[1])}
    common_rev1 = {n for n, e in zip(t1.names, t1.edges) if n in m12 and not e[1]}
    rev2 = {n for n, e in zip(t2.names, t2.edges) if e[1]}
    rev_result = {n for n, e in zip(t1.names, t1.edges) if n not in m12 and e[1]} | \
                 {n for n, e in zip(t2.names, t2.edges) if n not in m21 and e[1]}
    for a, b in pairs:
        ea, eb = t1.edge_by_name(a), t2.edge_by_name(b)
        if tuple((g.neg(s), d) for s, d in ea[0]) != eb[0] or ea[1] == eb[1]:
            raise ValueError("Incompatible edge segments in contract")

    def fit1():
        c1 = [n for n in t1.names if n in m12]
        return c1, [m12[n] for n in c1]

    def fit2():
        c2 = [n for n in t2.names if n in m21]
        return [m21[n] for n in c2], c2

    larger1 = t1.storage_size() > t2.storage_size()
    if not free1:
        put1 = True
        c1, c2 = fit2()
        put2 = (not c2) or c2[-1] == t2.names[-1]
    elif not free2:
        put2 = True
        c1, c2 = fit1()
        put1 = (not c1) or c1[-1] == t1.names[-1]
    elif larger1:
        if free1[-1] != t1.names[-1]:
            put1 = True
            c1, c2 = fit1()
            put2 = (not c2) or c2[-1] == t2.names[-1]
        elif free2[-1] != t2.names[-1]:
            put2 = True
            c1, c2 = fit2()
            put1 = (not c1) or c1[-1] == t1.names[-1]
        else:
            put1 = put2 = False
            c1, c2 = fit1()
    else:
        if free2[-1] != t2.names[-1]:
            put2 = True
            c1, c2 = fit2()
            put1 = (not c1) or c1[-1] == t1.names[-1]
        elif free1[-1] != t1.names[-1]:
            put1 = True
            c1, c2 = fit1()
            put2 = (not c2) or c2[-1] == t2.names[-1]
        else:
            put1 = put2 = False
            c1, c2 = fit2()

    a = t1.edge_operator({}, rev1, {C1: free1, C2: c1}, [C1, C2] if put1 else [C2, C1], False,
                         exclude_reversed_before=common_rev1, exclude_merge={C2})
    b = t2.edge_operator({}, rev2, {C2: free2, C1: c2}, [C2, C1] if put2 else [C1, C2], False)
    A = a.data if put1 else a.data.T          # (free1, common)
    B = b.data if put2 else b.data.T          # (free2, common)
    e0 = a.edges[0 if put1 else 1]
    e1 = b.edges[0 if put2 else 1]
    C = A @ B.T
    if put1 ^ (not put2):
        C = np.where(_index_parity(g, e0)[:, None], -C, C)
    product = FermiTensor([C1, C2], [e0, e1], g, C)
    split = {C1: [(n, t1.edge_by_name(n)[0]) for n in free1], C2: [(n, t2.edge_by_name(n)[0]) for n in free2]}
    return product.edge_operator(split, rev_result, {}, free1 + free2, False)
