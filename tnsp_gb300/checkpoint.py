"""The reference's checkpoint files, read and written without the reference installed.

Lattice files are pickles of tetragono's ``SamplingLattice``
(tetragono/tetragono/sampling_lattice/lattice.py:706-744, ``gm_save`` / ``gm_load``) whose TAT
tensors, edges and symmetries pickle their binary dump as state (PyTAT/PyTAT.hpp:170-182, 290-305,
757-771; format TAT/include/TAT/miscellaneous/io.hpp:199-345, 455-473, 687-781):

* tensor: ``b"TAT"``, u16 version (1), names, edges, storage;
* names: u64 count, then per name a u64 length and its bytes;
* edge: a u8 arrow for fermionic symmetries, then u64 count and ``count`` (symmetry, u64 dimension)
  pairs of 16 bytes each (no symmetry: 8 bytes of padding; Bose or Fermi U(1): i32 charge and 4 bytes
  of padding);
* storage: u64 count and ``count`` float64 values in TAT's block order.

``load_lattice`` reads such a file into stand-in objects (``RefSamplingLattice`` with ``RefTensor``
/ ``RefEdge`` / ``RefSymmetry`` members), ``to_sampling_lattice`` turns it into this package's
``SamplingLattice``, ``set_tensors`` writes dense site tensors back into the block storage, and
``save_lattice`` pickles the stand-ins under the reference's own class paths, so the reference loads
the file unchanged.  Supported: real (float64) tensors without symmetry, with Bose U(1) or with
Fermi U(1) (edges then carry their arrows; ``tnsp_gb300.fermion`` turns such a lattice into its
dense form).

Configuration files are the int64 files of ``write_configurations`` / ``read_configurations``
(tetragono/tetragono/utility.py:390-418): a header [number of blocks, rank, *shape] followed by one
configuration array per MPI rank; here one block per chain.
"""
import io
import pickle
import struct

import numpy as np

from .lattice import ORDER, SamplingLattice, block_to_dense, element_table, iterate_blocks, _segment_offsets, \
    site_charges

_SYMMETRIES = {"No": 0, "BoseU1": 4, "FermiU1": 4}  # bytes of the symmetry value in a 16-byte segment pair
_CHARGED = ("BoseU1", "FermiU1")
_FERMI = ("FermiU1",)


def _u64(buf, pos):
    return struct.unpack_from("<Q", buf, pos)[0], pos + 8


class RefSymmetry:
    """A TAT symmetry value (the U(1) charge, or None without symmetry)."""
    _ref_module = None
    _ref_name = "Symmetry"
    symmetry = "No"

    def __init__(self, charge=None):
        self.charge = charge

    def __setstate__(self, state):
        self.charge = struct.unpack_from("<i", state, 0)[0] if self.symmetry in _CHARGED else None

    def dumps(self):
        return struct.pack("<i", self.charge) if self.symmetry in _CHARGED else b"\x00"

    def __reduce_ex__(self, protocol):
        return _newobj, (type(self),), self.dumps()


class RefEdge:
    """A TAT edge: segments [(charge, dimension), ...] (charge 0 without symmetry) and, for a
    fermionic symmetry, its arrow."""
    _ref_module = None
    _ref_name = "Edge"
    symmetry = "No"

    def __init__(self, segments=(), arrow=False):
        self.segments = [tuple(s) for s in segments]
        self.arrow = bool(arrow)

    @classmethod
    def _parse(cls, buf, pos, symmetry):
        arrow = False
        if symmetry in _FERMI:
            arrow = buf[pos] != 0
            pos += 1
        count, pos = _u64(buf, pos)
        segments = []
        for _ in range(count):
            charge = struct.unpack_from("<i", buf, pos)[0] if symmetry in _CHARGED else 0
            dim = struct.unpack_from("<Q", buf, pos + 8)[0]
            segments.append((int(charge), int(dim)))
            pos += 16
        return segments, arrow, pos

    @staticmethod
    def _pack(segments, symmetry, arrow=False):
        out = [bytes([1 if arrow else 0])] if symmetry in _FERMI else []
        out.append(struct.pack("<Q", len(segments)))
        for charge, dim in segments:
            head = struct.pack("<i", charge) + b"\x00" * 4 if symmetry in _CHARGED else b"\x00" * 8
            out.append(head + struct.pack("<Q", dim))
        return b"".join(out)

    def __setstate__(self, state):
        self.segments, self.arrow, _ = RefEdge._parse(state, 0, self.symmetry)

    def dumps(self):
        return RefEdge._pack(self.segments, self.symmetry, self.arrow)

    def __reduce_ex__(self, protocol):
        return _newobj, (type(self),), self.dumps()


class RefTensor:
    """A TAT tensor: leg names, edges (segment lists) and block storage (float64)."""
    _ref_module = None
    _ref_name = "Tensor"
    symmetry = "No"

    def __init__(self, names=(), edges=(), storage=(), arrows=None):
        self.names = list(names)
        self.edges = [list(e) for e in edges]
        self.arrows = list(arrows) if arrows is not None else [False] * len(self.edges)
        self.storage = np.asarray(storage, dtype=np.float64)

    def __setstate__(self, state):
        buf = bytes(state)
        if buf[:3] != b"TAT":
            raise NotImplementedError("tensor dumps of TAT's version 0 layout are not supported")
        version = struct.unpack_from("<H", buf, 3)[0]
        if version != 1:
            raise NotImplementedError(f"tensor dump version {version}")
        pos = 5
        count, pos = _u64(buf, pos)
        names = []
        for _ in range(count):
            n, pos = _u64(buf, pos)
            names.append(buf[pos:pos + n].decode())
            pos += n
        count, pos = _u64(buf, pos)
        edges, arrows = [], []
        for _ in range(count):
            segments, arrow, pos = RefEdge._parse(buf, pos, self.symmetry)
            edges.append(segments)
            arrows.append(arrow)
        count, pos = _u64(buf, pos)
        self.names, self.edges, self.arrows = names, edges, arrows
        self.storage = np.frombuffer(buf, dtype="<f8", count=count, offset=pos).copy()

    def dumps(self):
        out = [b"TAT", struct.pack("<H", 1), struct.pack("<Q", len(self.names))]
        for n in self.names:
            b = n.encode()
            out.append(struct.pack("<Q", len(b)) + b)
        out.append(struct.pack("<Q", len(self.edges)))
        for e, a in zip(self.edges, self.arrows):
            out.append(RefEdge._pack(e, self.symmetry, a))
        out.append(struct.pack("<Q", self.storage.size))
        out.append(np.ascontiguousarray(self.storage, dtype="<f8").tobytes())
        return b"".join(out)

    def dense(self):
        return block_to_dense(self.storage, self.edges)

    def __reduce_ex__(self, protocol):
        return _newobj, (type(self),), self.dumps()


class RefSamplingLattice:
    """tetragono's SamplingLattice as stored: the ``__getstate__`` dict (lattice.py:741-744)."""
    _ref_module = "tetragono.sampling_lattice.lattice"
    _ref_name = "SamplingLattice"

    def __init__(self, state=None):
        self.state = dict(state or {})

    def __setstate__(self, state):
        if isinstance(state, tuple):  # files written before the reference's data_version field
            state = state[1]
        self.state = dict(state)

    def __reduce_ex__(self, protocol):
        return _newobj, (type(self),), self.state


def _newobj(cls):
    return cls.__new__(cls)


_CLASSES = {}


def _ref_class(module, name):
    """The stand-in class for the reference class ``module.name`` (one per class path)."""
    key = (module, name)
    if key in _CLASSES:
        return _CLASSES[key]
    parts = module.split(".")
    if module == RefSamplingLattice._ref_module and name == "SamplingLattice":
        cls = RefSamplingLattice
    elif parts[0] == "TAT" and len(parts) >= 2 and parts[1] in _SYMMETRIES:
        base = {"Tensor": RefTensor, "Edge": RefEdge, "Symmetry": RefSymmetry}.get(name)
        if base is None or (name == "Tensor" and parts[2:] != ["D"]) or (name != "Tensor" and len(parts) != 2):
            raise NotImplementedError(f"{module}.{name}: only float64 tensors without symmetry, Bose or Fermi U(1)")
        cls = type(f"{parts[1]}{name}", (base,), {"_ref_module": module, "_ref_name": name, "symmetry": parts[1]})
    elif parts[0] in ("TAT", "tetragono"):
        raise NotImplementedError(f"{module}.{name} is not supported (no symmetry, Bose or Fermi U(1), float64 only)")
    else:
        return None
    _CLASSES[key] = cls
    return cls


class _Unpickler(pickle.Unpickler):

    def find_class(self, module, name):
        cls = _ref_class(module, name)
        return cls if cls is not None else super().find_class(module, name)


class _Pickler(pickle._Pickler):
    """Pickles the stand-in classes under the reference's module and class names."""

    def save_global(self, obj, name=None):
        module = getattr(obj, "_ref_module", None) if isinstance(obj, type) else None
        if module is None:
            return super().save_global(obj, name)
        self.save(module)
        self.save(obj._ref_name)
        self.write(pickle.STACK_GLOBAL)
        self.memoize(obj)

    def save_reduce(self, func, args, state=None, listitems=None, dictitems=None, state_setter=None, *, obj=None):
        if func is _newobj:  # the reference's own objects are rebuilt with cls.__new__ + __setstate__
            self.save(args[0])
            self.save(())
            self.write(pickle.NEWOBJ)
            if obj is not None:
                self.memoize(obj)
            self.save(state)
            self.write(pickle.BUILD)
            return
        return super().save_reduce(func, args, state, listitems, dictitems, state_setter, obj=obj)


def load_lattice(path_or_file):
    """Reads a reference lattice file (``gm_save``) into a RefSamplingLattice."""
    if hasattr(path_or_file, "read"):
        obj = _Unpickler(path_or_file).load()
    else:
        with open(path_or_file, "rb") as f:
            obj = _Unpickler(f).load()
    if not isinstance(obj, RefSamplingLattice):
        raise ValueError(f"not a sampling lattice file ({type(obj).__name__})")
    return obj


def save_lattice(ref, path_or_file):
    """Writes a RefSamplingLattice so that the reference's ``gm_load`` (pickle.load) reads it."""
    buf = io.BytesIO()
    _Pickler(buf, protocol=4).dump(ref)
    data = buf.getvalue()
    if hasattr(path_or_file, "write"):
        path_or_file.write(data)
    else:
        with open(path_or_file, "wb") as f:
            f.write(data)


def _site_names_edges(t):
    return list(t.names), [list(e) for e in t.edges]


def to_sampling_lattice(ref):
    """The package's SamplingLattice (dense tensors, U(1) charges, element tables) of a stored one."""
    st = ref.state
    L1, L2 = st["L1"], st["L2"]
    grid = st["_lattice"]
    if getattr(type(grid[0][0]), "symmetry", "No") in _FERMI:
        raise NotImplementedError("a fermionic lattice: use tnsp_gb300.fermion.from_reference_lattice")
    phys = st["_physics_edges"][0][0][0].segments
    P = sum(d for _, d in phys)
    tensors = [[None] * L2 for _ in range(L1)]
    charged = getattr(type(grid[0][0]), "symmetry", "No") != "No"
    legs = [[None] * L2 for _ in range(L1)]
    flux = [[0] * L2 for _ in range(L1)]
    phys_q = None
    for l1 in range(L1):
        for l2 in range(L2):
            t = grid[l1][l2]
            names, edges = _site_names_edges(t)
            if [n for n in names if n.startswith("P")] != ["P0"]:
                raise NotImplementedError("one orbit (physical leg P0) per site only")
            tensors[l1][l2] = _site_dense(t)
            if charged:
                legs[l1][l2], phys_q, flux[l1][l2] = site_charges(names, edges)
    terms = {}
    for positions, H in st["_hamiltonians"].items():
        names, edges = _site_names_edges(H)
        terms[tuple(tuple(p) for p in positions)] = element_table(H.storage, names, edges, phys)
    charges = (legs, phys_q, flux) if charged else None
    return SamplingLattice(L1, L2, P, tensors, terms, charges)


def _site_dense(t):
    names, edges = _site_names_edges(t)
    dense = block_to_dense(t.storage, edges)
    keep = [n for n in ORDER if n in names]
    perm = [names.index(n) for n in keep] + [i for i, n in enumerate(names) if n not in ORDER]
    arr = dense.transpose(perm)
    arr = arr.reshape(arr.shape[:len(keep)])
    shape = [arr.shape[keep.index(n)] if n in keep else 1 for n in ORDER]
    return np.ascontiguousarray(arr.reshape(shape))


def dense_to_blocks(dense, edges):
    """Block storage (core order) of a dense array laid out like ``block_to_dense``'s output."""
    offs = [_segment_offsets(e) for e in edges]
    out = []
    for seg_idx, _ in iterate_blocks(edges):
        sl = tuple(slice(offs[i][0][seg_idx[i]], offs[i][0][seg_idx[i]] + edges[i][seg_idx[i]][1])
                   for i in range(len(edges)))
        out.append(np.asarray(dense[sl], dtype=np.float64).ravel())
    return np.concatenate(out) if out else np.zeros(0)


def set_tensors(ref, lattice):
    """Writes the dense site tensors of ``lattice`` (e.g. after gradient steps on the GPU) into the
    block storage of the stored lattice ``ref``; entries outside the blocks must be zero."""
    st = ref.state
    for l1 in range(st["L1"]):
        for l2 in range(st["L2"]):
            t = st["_lattice"][l1][l2]
            names, edges = _site_names_edges(t)
            a = np.asarray(lattice[l1, l2], dtype=np.float64)
            keep = [n for n in ORDER if n in names]
            extra = [n for n in names if n not in ORDER]
            arr = a.reshape([a.shape[ORDER.index(n)] for n in keep] + [1] * len(extra))
            order = keep + extra
            arr = arr.transpose([order.index(n) for n in names])
            storage = dense_to_blocks(arr, edges)
            back = block_to_dense(storage, edges)
            if not np.array_equal(back, arr):
                raise ValueError(f"site ({l1}, {l2}) has nonzero entries outside its symmetry blocks")
            t.storage = storage


def write_configurations(configs, path):
    """``write_configurations`` (utility.py:390-399) for a batch of chains: one block per chain,
    configs int64 [chains, L1, L2, orbits]."""
    configs = np.asarray(configs, dtype=np.int64)
    if configs.ndim == 3:
        configs = configs[..., None]
    head = np.array([configs.shape[0], configs.ndim - 1, *configs.shape[1:]], dtype=np.int64)
    with open(path, "wb") as f:
        f.write(head.tobytes())
        f.write(np.ascontiguousarray(configs).tobytes())


def read_configurations(path):
    """All blocks of a ``write_configurations`` file (utility.py:402-418): int64 [blocks, *shape]."""
    raw = np.fromfile(path, dtype=np.int64)
    size, rank = int(raw[0]), int(raw[1])
    shape = tuple(int(x) for x in raw[2:2 + rank])
    n = int(np.prod(shape))
    body = raw[2 + rank:2 + rank + size * n]
    if body.size != size * n:
        raise ValueError("configuration file shorter than its header")
    return body.reshape((size,) + shape)
