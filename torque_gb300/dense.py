"""Python mirrors of torque::gpu::DenseTensor<T> and SparseTensor<T>.

Same constructors, members and errors as the reference classes
(src/gpu/dense.cuh:52-604, src/gpu/sparse.cuh:81-436).  A dense tensor is a
block-sparse tensor with one block spanning the whole box; an element-sparse
tensor is a block-sparse tensor of one-element blocks (its contraction pairs
nonzeros with equal contracted coordinates and sums products that land on the
same output coordinate: the reduced layout).  Every operation runs on the GPU
through libtorque_gb300.so.  Differences from the reference are listed in
include/torque_gb300/sparse.hpp.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import TQ_MEM_HOST, check, load
from .block_sparse import BlockSparseTensor, _DT, _i64, _p64


def index_table(dimension) -> np.ndarray:
    """Column-major strides (torque::util::generate_index_table, src/util/space.h:11-24)."""
    d = _i64(dimension)
    return np.concatenate([[1], np.cumprod(d)[:-1]]).astype(np.int64) if d.size else d


class DenseTensor:
    def __init__(self, dimension=None, source_data=None, dtype=np.float64, _bs=None):
        if _bs is not None:
            self._bs = _bs
            self.dimension = _bs.dimension
        else:
            self.dimension = _i64(dimension)
            r = self.dimension.size
            if source_data is None:
                dt = _DT[np.dtype(dtype)]
                h = ctypes.c_void_p()
                if r == 0:
                    check(load().tq_bs_create_empty(dt, 0, None, ctypes.byref(h)))
                else:
                    b = np.zeros(r, np.int64)
                    e = self.dimension - 1
                    check(load().tq_bs_create_zeros(dt, r, _p64(self.dimension), 1, _p64(b),
                                                    _p64(e), None, None, ctypes.byref(h)))
                self._bs = BlockSparseTensor(_handle=h)
            else:
                data = np.ascontiguousarray(np.asarray(source_data, dtype)).ravel(order="F")
                if r == 0:
                    self._bs = BlockSparseTensor([], data[:1], [], [], dtype=dtype)
                else:
                    self._bs = BlockSparseTensor(self.dimension, data,
                                                 np.zeros((r, 1), np.int64),
                                                 (self.dimension - 1).reshape(r, 1), dtype=dtype)
        self.rank = int(self.dimension.size)
        self.index_table = index_table(self.dimension)

    def initialize(self, source_data):
        d = np.ascontiguousarray(np.asarray(source_data, self._bs.dtype)).ravel(order="F")
        check(load().tq_bs_set_data(self._bs.handle, d.ctypes.data_as(ctypes.c_void_p), TQ_MEM_HOST,
                                    None))

    def _check(self, idx):
        idx = _i64(idx)
        if idx.size != self.rank:
            raise _lib.TorqueError(_lib.TQ_ERR_INVALID, "Rank does not match")
        if np.any(idx >= self.dimension):
            raise _lib.TorqueError(_lib.TQ_ERR_INVALID, "Indices out of boundary")
        return idx

    def query(self, indices):
        self._check(indices)
        return self._bs.query(indices)

    def modify(self, indices, number):
        self._check(indices)
        self._bs.modify(indices, number)

    def to_number(self):
        return self._bs.to_number()

    def contract(self, tensor: "DenseTensor", contracting_indices, **schedule) -> "DenseTensor":
        """contracting_indices: n x 2 (column 0 this tensor's legs); schedule:
        precision / slices / tile_n / native_fill as in BlockSparseTensor.contract."""
        return DenseTensor(_bs=self._bs.contract(tensor._bs, contracting_indices, **schedule))

    def hard_transpose(self, permutation) -> "DenseTensor":
        return DenseTensor(_bs=self._bs.hard_transpose(permutation))

    def data(self) -> np.ndarray:
        """All elements, column-major."""
        return self._bs.data()


class SparseTensor:
    def __init__(self, dimension=None, source_data=None, indices=None, table=None,
                 dtype=np.float64, _bs=None):
        if _bs is not None:
            self._bs = _bs
            self.dimension = _bs.dimension
            self.rank = int(self.dimension.size)
            self.index_table = index_table(self.dimension)
            self._refresh()
            return
        self.dimension = _i64(dimension)
        self.rank = int(self.dimension.size)
        self.index_table = index_table(self.dimension) if table is None else _i64(table)
        self._dtype = dtype
        if source_data is None:
            self._bs = BlockSparseTensor(self.dimension, dtype=dtype)
            self.indices = np.zeros(0, np.int64)
        else:
            self.initialize(source_data, indices)

    def initialize(self, source_data, indices):
        """One element per linear index (decoded through the index table,
        largest stride first, as index_to_indices, src/util/space.h:27-58)."""
        dtype = getattr(self, "_dtype", np.float64)
        data = np.ascontiguousarray(np.asarray(source_data, dtype))
        idx = _i64(indices)
        self.indices = idx.copy()
        if self.rank == 0:
            self._bs = BlockSparseTensor([], data[:1], [], [], dtype=dtype)
            return
        order = np.argsort(-self.index_table, kind="stable")
        pts = np.zeros((idx.size, self.rank), np.int64)
        x = idx.copy()
        for q in order:
            pts[:, q] = x // self.index_table[q]
            x = x % self.index_table[q]
        if np.any(pts >= self.dimension):
            raise _lib.TorqueError(_lib.TQ_ERR_INVALID, "Indices out of boundary")
        self._bs = BlockSparseTensor(self.dimension, data[:idx.size], pts.T, pts.T, dtype=dtype)

    def _refresh(self):
        _, b, _, _, _ = self._bs.metadata()
        self.indices = (b.T @ self.index_table).astype(np.int64) if b.size else \
            np.zeros(0, np.int64)

    def query(self, indices):
        if _i64(indices).size != self.rank:
            raise _lib.TorqueError(_lib.TQ_ERR_INVALID, "Rank does not match")
        return self._bs.query(indices)

    def modify(self, indices, number):
        if _i64(indices).size != self.rank:
            raise _lib.TorqueError(_lib.TQ_ERR_INVALID, "Rank does not match")
        self._bs.modify(indices, number)
        self._refresh()

    def to_number(self):
        return self._bs.to_number()

    def contract(self, tensor: "SparseTensor", contracting_indices) -> "SparseTensor":
        """Matching nonzeros found by sorting both operands by their contracted
        index (tq_bs_contract_elements); a contraction to a scalar takes the
        block path."""
        ci = np.asarray(contracting_indices, dtype=np.int64).reshape(-1, 2)
        if self.rank + tensor.rank > 2 * ci.shape[0]:
            from .block_sparse import contract_elements
            return SparseTensor(_bs=contract_elements(self._bs, tensor._bs, ci))
        return SparseTensor(_bs=self._bs.contract(tensor._bs, ci, layout="reduced"))

    def soft_transpose(self, permutation):
        p = _i64(permutation)
        if p.size != self.rank:
            raise _lib.TorqueError(_lib.TQ_ERR_INVALID,
                                   "The number of permutation does not match the rank of tensor")
        self._bs = self._bs.hard_transpose(p)
        self.dimension = self.dimension[p]
        self.index_table = self.index_table[p]

    def hard_transpose(self, permutation) -> "SparseTensor":
        return SparseTensor(_bs=self._bs.hard_transpose(permutation))

    def values(self) -> np.ndarray:
        return self._bs.data()
