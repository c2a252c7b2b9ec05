"""Python access to the C oracle (``torque_oracle.c``) plus numpy dense checks.

TEST INFRASTRUCTURE ONLY.  This module is the oracle the CUDA path is checked
against; only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline legs import it.  The product package never does.

Each entry restates the reference (Walter-Feng/Torque) algorithm; the C file
cites the file:line it follows.  A block-sparse tensor is passed as a
``HostBS`` (numpy arrays, the reference's column-major metadata layout).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "liboracle.so")
_SRC = os.path.join(_HERE, "torque_oracle.c")


def build(force: bool = False) -> str:
    """Compile the C oracle with gcc (x86_64 or aarch64; no flags that differ)."""
    if force or not os.path.exists(_SO) or os.path.getmtime(_SO) < os.path.getmtime(_SRC):
        cmd = ["gcc", "-O2", "-std=c99", "-fopenmp", "-fPIC", "-shared", "-o", _SO, _SRC]
        subprocess.check_call(cmd)
    return _SO


class _OrcBS(ctypes.Structure):
    _fields_ = [
        ("rank", ctypes.c_int32),
        ("dimension", ctypes.POINTER(ctypes.c_int64)),
        ("n_blocks", ctypes.c_int64),
        ("begin", ctypes.POINTER(ctypes.c_int64)),
        ("end", ctypes.POINTER(ctypes.c_int64)),
        ("strides", ctypes.POINTER(ctypes.c_int64)),
        ("offsets", ctypes.POINTER(ctypes.c_int64)),
        ("data", ctypes.POINTER(ctypes.c_double)),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        P64 = ctypes.POINTER(ctypes.c_int64)
        PD = ctypes.POINTER(ctypes.c_double)
        PB = ctypes.POINTER(_OrcBS)
        _lib.orc_match.restype = ctypes.c_int64
        _lib.orc_match.argtypes = [PB, PB, ctypes.c_int32, P64, P64, P64, P64, ctypes.c_int64]
        _lib.orc_pair_boxes.restype = None
        _lib.orc_pair_boxes.argtypes = [PB, PB, ctypes.c_int32, P64, P64, ctypes.c_int64,
                                        ctypes.c_int64] + [P64] * 8
        _lib.orc_pair_values.restype = ctypes.c_int32
        _lib.orc_pair_values.argtypes = [PB, PB, ctypes.c_int32, P64, P64, ctypes.c_int64,
                                         ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, PD]
        _lib.orc_contract_size.restype = ctypes.c_int64
        _lib.orc_contract_size.argtypes = [PB, PB, ctypes.c_int32, P64, P64]
        _lib.orc_contract.restype = ctypes.c_int32
        _lib.orc_contract.argtypes = [PB, PB, ctypes.c_int32, P64, P64, ctypes.c_int32,
                                      P64, P64, P64, PD]
        _lib.orc_query.restype = ctypes.c_double
        _lib.orc_query.argtypes = [PB, P64]
        _lib.orc_densify.restype = None
        _lib.orc_densify.argtypes = [PB, PD]
        _lib.orc_hard_transpose.restype = None
        _lib.orc_hard_transpose.argtypes = [PB, P64, PD]
        _lib.orc_pairs_baseline.restype = ctypes.c_int32
        _lib.orc_pairs_baseline.argtypes = [PB, PB, ctypes.c_int32, P64, P64, ctypes.c_int64,
                                            P64, P64, P64, PD]
    return _lib


def pairs_baseline(A: HostBS, B: HostBS, pairs, pa, pb):
    """The reference CPU path's per-pair work (gather + dense multiply) for the
    given pairs, OpenMP-parallel over pairs.  Returns (blocks, threads used)."""
    al, bl, nc = _legs(pairs)
    pa = np.ascontiguousarray(pa, dtype=np.int64)
    pb = np.ascontiguousarray(pb, dtype=np.int64)
    fa = [l for l in range(A.rank) if l not in set(al.tolist())]
    fb = [l for l in range(B.rank) if l not in set(bl.tolist())]
    m = np.prod(A.block_dims[pa][:, fa], axis=1) if fa else np.ones(pa.size, np.int64)
    n = np.prod(B.block_dims[pb][:, fb], axis=1) if fb else np.ones(pb.size, np.int64)
    sizes = (m * n).astype(np.int64)
    offs = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
    out = np.zeros(max(int(sizes.sum()), 1), np.float64)
    ca, cb = A.c(), B.c()
    threads = lib().orc_pairs_baseline(ctypes.byref(ca), ctypes.byref(cb), nc, _p64(al), _p64(bl),
                                       pa.size, _p64(pa), _p64(pb), _p64(offs), _pd(out))
    return out, offs, threads


def _p64(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))


def _pd(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


@dataclass
class HostBS:
    """Host block-sparse tensor in the reference's layout (float64 values)."""
    dimension: np.ndarray                 # [rank]
    begin: np.ndarray                     # [n_blocks, rank]
    end: np.ndarray                       # [n_blocks, rank]
    data: np.ndarray                      # [n_elem] float64
    strides: np.ndarray = None            # [n_blocks, rank]; default column-major
    offsets: np.ndarray = None            # [n_blocks]; default exclusive scan
    _keep: list = field(default_factory=list, repr=False)

    def __post_init__(self):
        self.dimension = np.ascontiguousarray(self.dimension, dtype=np.int64)
        r = self.dimension.size
        nb = np.asarray(self.begin).size // r if r else 0
        self.begin = np.ascontiguousarray(np.asarray(self.begin, dtype=np.int64).reshape(nb, r))
        self.end = np.ascontiguousarray(np.asarray(self.end, dtype=np.int64).reshape(nb, r))
        dims = self.end - self.begin + 1
        if self.strides is None:
            st = np.ones_like(dims)
            if r > 1:
                st[:, 1:] = np.cumprod(dims[:, :-1], axis=1)
            self.strides = st
        self.strides = np.ascontiguousarray(np.asarray(self.strides, dtype=np.int64).reshape(nb, r))
        n_elem = np.prod(dims, axis=1) if r else np.zeros(0, np.int64)
        if self.offsets is None:
            self.offsets = np.concatenate([[0], np.cumsum(n_elem)[:-1]]).astype(np.int64) \
                if len(n_elem) else np.zeros(0, np.int64)
        self.offsets = np.ascontiguousarray(self.offsets, dtype=np.int64)
        self.data = np.ascontiguousarray(self.data, dtype=np.float64)

    @property
    def rank(self):
        return int(self.dimension.size)

    @property
    def n_blocks(self):
        return int(self.begin.shape[0])

    @property
    def block_dims(self):
        return self.end - self.begin + 1

    def c(self) -> _OrcBS:
        d = self.data if self.data.size else np.zeros(1)
        self._keep = [d]
        return _OrcBS(self.rank, _p64(self.dimension), self.n_blocks, _p64(self.begin),
                      _p64(self.end), _p64(self.strides), _p64(self.offsets), _pd(d))


def _legs(pairs):
    pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
    return (np.ascontiguousarray(pairs[:, 0]), np.ascontiguousarray(pairs[:, 1]), pairs.shape[0])


def match(A: HostBS, B: HostBS, pairs):
    """Reference-order pair list (A block, B block)."""
    al, bl, nc = _legs(pairs)
    ca, cb = A.c(), B.c()
    n = lib().orc_match(ctypes.byref(ca), ctypes.byref(cb), nc, _p64(al), _p64(bl), None, None, 0)
    pa = np.zeros(max(n, 1), np.int64)
    pb = np.zeros(max(n, 1), np.int64)
    lib().orc_match(ctypes.byref(ca), ctypes.byref(cb), nc, _p64(al), _p64(bl), _p64(pa), _p64(pb), n)
    return pa[:n], pb[:n]


class UndefinedRead(IndexError):
    """Mode 2: the reference CPU path as written would read past the end of a
    tensor's values; its result is undefined there."""


def _raise_mode2(st: int) -> None:
    if st == 6:
        raise UndefinedRead("reference CPU path reads past the end of a tensor's values")
    if st != 0:
        raise IndexError("reference CPU path indexes a block table column out of range")


def contract(A: HostBS, B: HostBS, pairs, mode: int = 0):
    """Reference-layout contraction.  Returns (begin, end, offsets, data) or for a
    rank-0 result the scalar.  mode: 0 accurate, 1 plain double, 2 as-written
    reference CPU strides (raises IndexError where the reference throws, and
    UndefinedRead where it would read past a tensor's values)."""
    al, bl, nc = _legs(pairs)
    ca, cb = A.c(), B.c()
    L = lib()
    ro = A.rank + B.rank - 2 * nc
    size = L.orc_contract_size(ctypes.byref(ca), ctypes.byref(cb), nc, _p64(al), _p64(bl))
    npairs = L.orc_match(ctypes.byref(ca), ctypes.byref(cb), nc, _p64(al), _p64(bl), None, None, 0)
    ob = np.zeros((max(npairs, 1), max(ro, 1)), np.int64)
    oe = np.zeros_like(ob)
    off = np.zeros(max(npairs, 1), np.int64)
    data = np.zeros(max(size, 1), np.float64)
    st = L.orc_contract(ctypes.byref(ca), ctypes.byref(cb), nc, _p64(al), _p64(bl), mode,
                        _p64(ob), _p64(oe), _p64(off), _pd(data))
    _raise_mode2(st)
    if ro == 0:
        return float(data[0])
    return ob[:npairs, :ro], oe[:npairs, :ro], off[:npairs], data[:size]


def contract_blocks(A: HostBS, B: HostBS, pairs):
    """The reference layout's block list without its values: pair list (A
    block, B block), output begin/end and offsets (orc_match + the box and
    offset loop of orc_contract with no data), for results too large to hold."""
    al, bl, nc = _legs(pairs)
    pa, pb = match(A, B, pairs)
    ca, cb = A.c(), B.c()
    ro = A.rank + B.rank - 2 * nc
    n = pa.size
    ob = np.zeros((max(n, 1), max(ro, 1)), np.int64)
    oe = np.zeros_like(ob)
    off = np.zeros(max(n, 1), np.int64)
    st = lib().orc_contract(ctypes.byref(ca), ctypes.byref(cb), nc, _p64(al), _p64(bl), 0,
                            _p64(ob), _p64(oe), _p64(off), None)
    assert st == 0
    return pa, pb, ob[:n, :ro], oe[:n, :ro], off[:n]


def pair_values(A: HostBS, B: HostBS, pairs, i: int, j: int, mode: int = 0, j_block: int = 0):
    al, bl, nc = _legs(pairs)
    ca, cb = A.c(), B.c()
    fa = [l for l in range(A.rank) if l not in set(al.tolist())]
    fb = [l for l in range(B.rank) if l not in set(bl.tolist())]
    m = int(np.prod([A.end[i, l] - A.begin[i, l] + 1 for l in fa])) if fa else 1
    n = int(np.prod([B.end[j, l] - B.begin[j, l] + 1 for l in fb])) if fb else 1
    out = np.zeros(m * n, np.float64)
    st = lib().orc_pair_values(ctypes.byref(ca), ctypes.byref(cb), nc, _p64(al), _p64(bl), i, j,
                               j_block, mode, _pd(out))
    _raise_mode2(st)
    return out.reshape(n, m).T  # column-major m x n


def query(T: HostBS, idx) -> float:
    idx = np.ascontiguousarray(idx, dtype=np.int64)
    c = T.c()
    return lib().orc_query(ctypes.byref(c), _p64(idx))


def densify(T: HostBS) -> np.ndarray:
    """Dense column-major array (returned as a numpy array indexed [i0, i1, ...])."""
    total = int(np.prod(T.dimension)) if T.rank else 1
    out = np.zeros(total, np.float64)
    c = T.c()
    lib().orc_densify(ctypes.byref(c), _pd(out))
    return out.reshape(tuple(T.dimension.tolist())[::-1]).transpose() if T.rank else out


def hard_transpose(T: HostBS, perm) -> HostBS:
    perm = np.ascontiguousarray(perm, dtype=np.int64)
    out = np.zeros(max(T.data.size, 1), np.float64)
    c = T.c()
    lib().orc_hard_transpose(ctypes.byref(c), _p64(perm), _pd(out))
    return HostBS(T.dimension[perm], T.begin[:, perm], T.end[:, perm], out[:T.data.size])


def dense_contract(Ad: np.ndarray, Bd: np.ndarray, pairs) -> np.ndarray:
    """Dense contraction of zero-filled tensors: result legs are A's free legs then
    B's free legs, as in the reference (src/tensor/dense.h:184-292)."""
    pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
    return np.tensordot(Ad, Bd, axes=(pairs[:, 0].tolist(), pairs[:, 1].tolist()))


def assemble_dense(dimension, begin, end, offsets, data) -> np.ndarray:
    """Densify a reference-layout result (column-major blocks, overlaps add)."""
    T = HostBS(np.asarray(dimension), begin, end, data, offsets=offsets)
    return densify(T)


if __name__ == "__main__":  # pragma: no cover
    print(build(force="--force" in sys.argv))


def slice_boxes(begin, end, divisor):
    """Restates BlockSparseTensor::slice (src/gpu/block_sparse.cuh:1124-1176): every
    block (rows of begin/end, [n_blocks, rank]) is cut into prod(divisor)
    sub-boxes of block_dim / divisor per leg, numbered with leg 0 fastest
    (index_to_indices over generate_index_table(divisor), src/util/space.h:11-45),
    blocks in order.  A block dimension that the divisor does not divide raises
    ValueError ("current slice does not support residues").  The data are not
    moved: the new tensor reads the old buffer through each sub-box's own
    column-major strides."""
    begin = np.asarray(begin, np.int64)
    end = np.asarray(end, np.int64)
    divisor = np.asarray(divisor, np.int64)
    dims = end - begin + 1
    if np.any(dims % divisor):
        raise ValueError("current slice does not support residues")
    sub = dims // divisor
    nsub = int(np.prod(divisor))
    nb, ne = [], []
    for i in range(begin.shape[0]):
        for j in range(nsub):
            idx, t = [], j
            for d in divisor:
                idx.append(t % d)
                t //= d
            b = begin[i] + np.asarray(idx) * sub[i]
            nb.append(b)
            ne.append(b + sub[i] - 1)
    return np.asarray(nb, np.int64).reshape(-1, begin.shape[1]), \
        np.asarray(ne, np.int64).reshape(-1, begin.shape[1])
