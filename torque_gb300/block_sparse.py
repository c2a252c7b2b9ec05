"""Python mirror of torque::gpu::BlockSparseTensor<T> over the C ABI.

Same names, argument meaning and error behaviour as the reference class
(src/gpu/block_sparse.cuh:143-1181): metadata matrices are rank x n_blocks
(column = block, the arma::umat convention), legs are column-major with leg 0
fastest, API misuse raises TorqueError (the reference's ``Error``).  Every
operation runs on the GPU through libtorque_gb300.so; nothing here computes.
"""
from __future__ import annotations

import ctypes
from typing import Optional, Sequence

import numpy as np

from . import _lib
from ._lib import TQ_F16, TQ_F32, TQ_F64, TQ_MEM_DEVICE, TQ_MEM_HOST, ContractOpts, check, load

_DT = {np.dtype(np.float64): TQ_F64, np.dtype(np.float32): TQ_F32,
       np.dtype(np.float16): TQ_F16}
_NP = {TQ_F64: np.float64, TQ_F32: np.float32, TQ_F16: np.float16}


def _i64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.int64))


def _p64(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)) if a.size else None


def _stream(stream) -> Optional[int]:
    if stream is None:
        return None
    if hasattr(stream, "cuda_stream"):
        return stream.cuda_stream
    return int(stream)


def _blocks(points, rank: int) -> np.ndarray:
    """rank x n_blocks (arma::umat layout) -> flat [b*rank + l]."""
    a = np.asarray(points, dtype=np.int64)
    if rank == 0:
        return np.zeros((0, 0), np.int64)
    if a.ndim == 1:
        a = a.reshape(rank, -1)
    if a.shape[0] != rank:
        raise _lib.TorqueError(_lib.TQ_ERR_INVALID, "Rank does not match")
    return np.ascontiguousarray(a.T)


class BlockSparseTensor:
    """A list of dense boxes (blocks) of a rank-r tensor, data on the GPU."""

    def __init__(self, dimension=None, source_data=None, begin_points=None, end_points=None,
                 index_tables=None, dtype=np.float64, stream=None, _handle=None):
        load()
        self._h = ctypes.c_void_p()
        if _handle is not None:
            self._h = _handle
            return
        dim = _i64(dimension if dimension is not None else [])
        rank = dim.size
        dt = _DT[np.dtype(dtype)]
        if source_data is None:
            # BlockSparseTensor(const arma::uvec & dimension)
            check(load().tq_bs_create_empty(dt, rank, _p64(dim), ctypes.byref(self._h)))
            return
        data, kind = self._data_arg(source_data, dtype)
        b = _blocks(begin_points, rank)
        e = _blocks(end_points, rank)
        t = None if index_tables is None else _blocks(index_tables, rank)
        self._keep = data
        check(load().tq_bs_create(dt, rank, _p64(dim), b.shape[0] if rank else 0, _p64(b), _p64(e),
                                  None if t is None else _p64(t), self._ptr(data), kind,
                                  _stream(stream), ctypes.byref(self._h)))
        self._keep = None

    @classmethod
    def zeros(cls, dimension, begin_points, end_points, index_tables=None, dtype=np.float64,
              stream=None) -> "BlockSparseTensor":
        """The block list with every element zero (tq_bs_create_zeros)."""
        dim = _i64(dimension)
        rank = dim.size
        b = _blocks(begin_points, rank)
        e = _blocks(end_points, rank)
        t = None if index_tables is None else _blocks(index_tables, rank)
        h = ctypes.c_void_p()
        check(load().tq_bs_create_zeros(_DT[np.dtype(dtype)], rank, _p64(dim),
                                        b.shape[0] if rank else 0, _p64(b), _p64(e),
                                        None if t is None else _p64(t), _stream(stream),
                                        ctypes.byref(h)))
        return cls(_handle=h)

    # ------------------------------------------------------------ helpers
    @staticmethod
    def _data_arg(src, dtype):
        if hasattr(src, "data_ptr"):  # a torch tensor on the device
            return src, TQ_MEM_DEVICE
        return np.ascontiguousarray(np.asarray(src, dtype=dtype)), TQ_MEM_HOST

    @staticmethod
    def _ptr(data):
        if hasattr(data, "data_ptr"):
            return ctypes.c_void_p(data.data_ptr())
        return data.ctypes.data_as(ctypes.c_void_p)

    @property
    def handle(self):
        return self._h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                load().tq_bs_destroy(h)
            except Exception:  # interpreter shutdown
                pass
            self._h = ctypes.c_void_p()

    def _shape(self):
        dt = ctypes.c_int32()
        rank = ctypes.c_int32()
        nb = ctypes.c_int64()
        ne = ctypes.c_int64()
        check(load().tq_bs_shape(self._h, ctypes.byref(dt), ctypes.byref(rank), ctypes.byref(nb),
                                 ctypes.byref(ne)))
        return dt.value, rank.value, nb.value, ne.value

    # ------------------------------------------------------------ metadata
    @property
    def dtype(self):
        return np.dtype(_NP[self._shape()[0]])

    @property
    def rank(self) -> int:
        return self._shape()[1]

    @property
    def n_blocks(self) -> int:
        return self._shape()[2]

    @property
    def n_elem(self) -> int:
        return self._shape()[3]

    def metadata(self):
        """(dimension, begin_points, end_points, index_tables, block_offsets); the
        point matrices are rank x n_blocks."""
        _, r, nb, _ = self._shape()
        dim = np.zeros(r, np.int64)
        b = np.zeros((nb, r), np.int64)
        e = np.zeros((nb, r), np.int64)
        t = np.zeros((nb, r), np.int64)
        off = np.zeros(nb, np.int64)
        check(load().tq_bs_metadata(self._h, _p64(dim), _p64(b), _p64(e), _p64(t), _p64(off)))
        return dim, b.T.copy(), e.T.copy(), t.T.copy(), off

    @property
    def dimension(self):
        return self.metadata()[0]

    @property
    def begin_points(self):
        return self.metadata()[1]

    @property
    def end_points(self):
        return self.metadata()[2]

    @property
    def index_tables(self):
        return self.metadata()[3]

    @property
    def block_offsets(self):
        return self.metadata()[4]

    @property
    def blocks_dimension(self):
        _, b, e, _, _ = self.metadata()
        return e - b + 1

    @property
    def block_n_elem(self):
        return np.prod(self.blocks_dimension, axis=0)

    def data(self) -> np.ndarray:
        """Host copy of the block data (all blocks back to back)."""
        dt, r, _, ne = self._shape()
        out = np.zeros(1 if r == 0 else ne, _NP[dt])
        if out.size:
            check(load().tq_bs_copy_data(self._h, out.ctypes.data_as(ctypes.c_void_p), TQ_MEM_HOST,
                                         None))
        return out

    def set_data(self, source_data, stream=None, asynchronous=False):
        """Overwrite every element (tq_bs_set_data): a numpy array (host, copied
        before return) or a torch CUDA tensor, n_elem elements of the tensor's
        dtype in the tensor's layout.  asynchronous=True only enqueues the copy
        on `stream` (tq_bs_set_data_async): the source must stay alive and
        unchanged until the stream has passed it (page-locked host memory then
        copies while other streams compute)."""
        n = self.n_elem if self.rank else 1
        data, kind = self._data_arg(source_data, self.dtype)
        size = data.numel() if hasattr(data, "numel") else data.size
        if size < n:
            raise ValueError("source holds %d elements; the tensor has %d" % (size, n))
        fn = load().tq_bs_set_data_async if asynchronous else load().tq_bs_set_data
        check(fn(self._h, self._ptr(data), kind, _stream(stream)))

    def device_ptr(self) -> int:
        p = ctypes.c_void_p()
        check(load().tq_bs_device_data(self._h, ctypes.byref(p)))
        return p.value or 0

    # ------------------------------------------------------------ element access
    def to_number(self):
        v = np.zeros(1, self.dtype)
        check(load().tq_bs_to_number(self._h, v.ctypes.data_as(ctypes.c_void_p)))
        return v[0]

    def query(self, indices: Sequence[int]):
        idx = _i64(indices)
        if idx.size != self.rank:
            raise _lib.TorqueError(_lib.TQ_ERR_INVALID, "Rank does not match")
        v = np.zeros(1, self.dtype)
        check(load().tq_bs_query(self._h, _p64(idx), v.ctypes.data_as(ctypes.c_void_p)))
        return v[0]

    def modify(self, indices: Sequence[int], number):
        idx = _i64(indices)
        if idx.size != self.rank:
            raise _lib.TorqueError(_lib.TQ_ERR_INVALID, "Rank does not match")
        v = np.asarray([number], self.dtype)
        check(load().tq_bs_modify(self._h, _p64(idx), v.ctypes.data_as(ctypes.c_void_p)))

    def append_block(self, source_data, begin_point, end_point, index_table=None, stream=None):
        self.append_blocks(source_data, np.asarray(begin_point).reshape(-1, 1),
                           np.asarray(end_point).reshape(-1, 1),
                           None if index_table is None else np.asarray(index_table).reshape(-1, 1),
                           stream)

    def append_blocks(self, source_data, begin_points, end_points, index_tables=None, stream=None):
        r = self.rank
        b = _blocks(begin_points, r)
        e = _blocks(end_points, r)
        t = None if index_tables is None else _blocks(index_tables, r)
        data, kind = self._data_arg(source_data, self.dtype)
        check(load().tq_bs_append_blocks(self._h, b.shape[0], _p64(b), _p64(e),
                                         None if t is None else _p64(t), self._ptr(data), kind,
                                         _stream(stream)))

    # ------------------------------------------------------------ operations
    def contract(self, tensor: "BlockSparseTensor", contracting_indices, precision="native",
                 layout="reference", slices=0, tile_n=0, native_fill=0,
                 stream=None) -> "BlockSparseTensor":
        """Contract legs contracting_indices[k][0] of self with [k][1] of tensor
        (an n x 2 matrix, as in the reference).  precision, slices, tile_n and
        native_fill are the schedule (tq_contract_opts)."""
        ci = np.asarray(contracting_indices, dtype=np.int64).reshape(-1, 2)
        al, bl = _i64(ci[:, 0]), _i64(ci[:, 1])
        opts = make_opts(precision, layout, slices, tile_n, native_fill)
        h = ctypes.c_void_p()
        check(load().tq_bs_contract(self._h, tensor._h, ci.shape[0], _p64(al), _p64(bl),
                                    ctypes.byref(opts), _stream(stream), ctypes.byref(h)))
        return BlockSparseTensor(_handle=h)

    def hard_transpose(self, permutation, stream=None) -> "BlockSparseTensor":
        perm = _i64(permutation)
        if perm.size != self.rank:
            raise _lib.TorqueError(_lib.TQ_ERR_INVALID,
                                   "The number of permutation does not match the rank of tensor")
        h = ctypes.c_void_p()
        check(load().tq_bs_hard_transpose(self._h, _p64(perm), _stream(stream), ctypes.byref(h)))
        return BlockSparseTensor(_handle=h)

    def fuse_legs(self, leg: int, bounds_a, bounds_b, pair_offset, stream=None):
        """Legs leg and leg+1 fused (tq_bs_fuse_legs): bounds_* are the sector
        boundaries of the two legs, pair_offset[a, b] the start of sector pair
        (a, b) in the fused leg."""
        ba, bb = _i64(bounds_a), _i64(bounds_b)
        off = _i64(np.asarray(pair_offset).reshape(ba.size - 1, bb.size - 1).ravel(order="F"))
        h = ctypes.c_void_p()
        check(load().tq_bs_fuse_legs(self._h, int(leg), ba.size - 1, _p64(ba), bb.size - 1,
                                     _p64(bb), _p64(off), _stream(stream), ctypes.byref(h)))
        return BlockSparseTensor(_handle=h)

    def fuse_sectors(self, leg: int, leg_a, leg_b, modulus=None, stream=None):
        """Charge-ordered fusion of legs leg, leg+1 carrying sectors leg_a,
        leg_b (sectors.Leg); returns (tensor, fused Leg)."""
        from .sectors import fuse_sector_order
        fused, off = fuse_sector_order(leg_a, leg_b, modulus)
        ba = np.concatenate([[0], np.cumsum(leg_a.sizes)])
        bb = np.concatenate([[0], np.cumsum(leg_b.sizes)])
        return self.fuse_legs(leg, ba, bb, off, stream), fused

    def split_leg(self, leg: int, bounds_a, bounds_b, pair_offset, stream=None):
        """Inverse of fuse_legs (tq_bs_split_leg): leg `leg` back into two legs,
        with the sector bounds and pair offsets that fused them."""
        ba, bb = _i64(bounds_a), _i64(bounds_b)
        off = _i64(np.asarray(pair_offset).reshape(ba.size - 1, bb.size - 1).ravel(order="F"))
        h = ctypes.c_void_p()
        check(load().tq_bs_split_leg(self._h, int(leg), ba.size - 1, _p64(ba), bb.size - 1,
                                     _p64(bb), _p64(off), _stream(stream), ctypes.byref(h)))
        return BlockSparseTensor(_handle=h)

    def split_sectors(self, leg: int, leg_a, leg_b, modulus=None, stream=None):
        """Inverse of fuse_sectors: the charge-ordered fused leg `leg` back into
        legs carrying sectors leg_a, leg_b (sectors.Leg)."""
        from .sectors import fuse_sector_order
        fused, off = fuse_sector_order(leg_a, leg_b, modulus)
        ba = np.concatenate([[0], np.cumsum(leg_a.sizes)])
        bb = np.concatenate([[0], np.cumsum(leg_b.sizes)])
        return self.split_leg(leg, ba, bb, off, stream)

    @classmethod
    def from_charges(cls, legs, source_data=None, total=0, modulus=None, dtype=np.float64,
                     stream=None) -> "BlockSparseTensor":
        """A charge-conserving tensor over sectors.Leg legs (tq_bs_create_charges):
        one block per sector tuple with sum(direction * charge) == total (mod
        modulus), leg 0 fastest; data in block order, or zeros."""
        ns, q, sz, d = charge_args(legs)
        h = ctypes.c_void_p()
        data, kind = (None, TQ_MEM_HOST) if source_data is None else \
            cls._data_arg(source_data, dtype)
        check(load().tq_bs_create_charges(_DT[np.dtype(dtype)], len(legs), _p64(ns), _p64(q),
                                          _p64(sz), d.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                          int(total), int(modulus or 0),
                                          None if data is None else cls._ptr(data), kind,
                                          _stream(stream), ctypes.byref(h)))
        return cls(_handle=h)

    def svd(self, row_legs, max_keep: int = 0, cutoff: float = 0.0, stream=None):
        """Block-level truncated SVD (tq_bs_svd): row_legs against the other
        legs; returns (U[row legs..., bond], S[bond], V[bond, other legs...])
        keeping at most max_keep values (0: all) above cutoff * the largest."""
        rl = _i64(row_legs)
        u, sv, v = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        check(load().tq_bs_svd(self._h, rl.size, _p64(rl), int(max_keep), float(cutoff),
                               _stream(stream), ctypes.byref(u), ctypes.byref(sv),
                               ctypes.byref(v)))
        return (BlockSparseTensor(_handle=u), BlockSparseTensor(_handle=sv),
                BlockSparseTensor(_handle=v))

    def qr(self, row_legs, stream=None):
        """Block-level QR (tq_bs_qr): row_legs against the other legs; returns
        (Q[row legs..., bond], R[bond, other legs...]), each class factored as
        Q R with orthonormal Q columns and R upper trapezoidal, diagonal >= 0."""
        rl = _i64(row_legs)
        q, r = ctypes.c_void_p(), ctypes.c_void_p()
        check(load().tq_bs_qr(self._h, rl.size, _p64(rl), _stream(stream), ctypes.byref(q),
                              ctypes.byref(r)))
        return BlockSparseTensor(_handle=q), BlockSparseTensor(_handle=r)

    def slice(self, divisor, stream=None) -> "BlockSparseTensor":
        d = _i64(divisor)
        h = ctypes.c_void_p()
        check(load().tq_bs_slice(self._h, _p64(d), _stream(stream), ctypes.byref(h)))
        return BlockSparseTensor(_handle=h)

    def clone(self, stream=None) -> "BlockSparseTensor":
        h = ctypes.c_void_p()
        check(load().tq_bs_clone(self._h, _stream(stream), ctypes.byref(h)))
        return BlockSparseTensor(_handle=h)


def contract_elements(A: "BlockSparseTensor", B: "BlockSparseTensor", contracting_indices,
                      stream=None) -> "BlockSparseTensor":
    """Element-sparse contraction (one-element blocks) by sort-join
    (tq_bs_contract_elements): one-element result blocks in output-index order."""
    ci = np.asarray(contracting_indices, dtype=np.int64).reshape(-1, 2)
    al, bl = _i64(ci[:, 0]), _i64(ci[:, 1])
    h = ctypes.c_void_p()
    check(load().tq_bs_contract_elements(A._h, B._h, ci.shape[0], _p64(al), _p64(bl),
                                         _stream(stream), ctypes.byref(h)))
    return BlockSparseTensor(_handle=h)


def charge_args(legs):
    """(sectors per leg, charges, sizes, directions) arrays of tq_charge_blocks."""
    ns = _i64([len(l.charges) for l in legs])
    q = _i64([c for l in legs for c in l.charges])
    sz = _i64([x for l in legs for x in l.sizes])
    d = np.ascontiguousarray([int(l.direction) for l in legs], dtype=np.int32)
    return ns, q, sz, d


def charge_block_list(legs, total=0, modulus=None):
    """The block list tq_charge_blocks makes: (begin, end) as n_blocks x rank."""
    ns, q, sz, d = charge_args(legs)
    n = ctypes.c_int64()
    dp = d.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    lib = load()
    check(lib.tq_charge_blocks(len(legs), _p64(ns), _p64(q), _p64(sz), dp, int(total),
                               int(modulus or 0), 0, ctypes.byref(n), None, None))
    r = len(legs)
    b = np.zeros(max(n.value, 1) * r, np.int64)
    e = np.zeros_like(b)
    check(lib.tq_charge_blocks(r, _p64(ns), _p64(q), _p64(sz), dp, int(total), int(modulus or 0),
                               n.value, ctypes.byref(n), _p64(b), _p64(e)))
    return b[:n.value * r].reshape(-1, r), e[:n.value * r].reshape(-1, r)


def contract_blocks(A: "BlockSparseTensor", B: "BlockSparseTensor", contracting_indices,
                    layout="reference", stream=None):
    """The block list A.contract(B, ...) would produce, from the symbolic stage
    alone (tq_contract_blocks: nothing computed, no result data allocated).
    Returns dict(begin, end, offsets: [n_blocks, rank] / [n_blocks] int64,
    n_elem, and for the reference layout pair_a / pair_b: each output block's
    A and B block)."""
    ci = np.asarray(contracting_indices, dtype=np.int64).reshape(-1, 2)
    al, bl = _i64(ci[:, 0]), _i64(ci[:, 1])
    lay = _lib.LAYOUTS[layout]
    nb, ne = ctypes.c_int64(), ctypes.c_int64()
    lib = load()
    check(lib.tq_contract_blocks(A._h, B._h, ci.shape[0], _p64(al), _p64(bl), lay, 0,
                                 ctypes.byref(nb), ctypes.byref(ne), None, None, None, None,
                                 None, _stream(stream)))
    n = nb.value
    rank = A.rank + B.rank - 2 * ci.shape[0]
    begin = np.zeros((max(n, 1), max(rank, 1)), np.int64)
    end = np.zeros_like(begin)
    off = np.zeros(max(n, 1), np.int64)
    ref = layout == "reference"
    pa = np.zeros(max(n, 1), np.int64) if ref else None
    pb = np.zeros(max(n, 1), np.int64) if ref else None
    if n:
        check(lib.tq_contract_blocks(A._h, B._h, ci.shape[0], _p64(al), _p64(bl), lay, n,
                                     ctypes.byref(nb), ctypes.byref(ne), _p64(begin),
                                     _p64(end), _p64(off), _p64(pa) if ref else None,
                                     _p64(pb) if ref else None, _stream(stream)))
    out = {"begin": begin[:n, :rank], "end": end[:n, :rank], "offsets": off[:n],
           "n_elem": ne.value}
    if ref:
        out["pair_a"], out["pair_b"] = pa[:n], pb[:n]
    return out


def make_opts(precision="native", layout="reference", slices=0, tile_n=0, native_fill=0):
    """tq_contract_opts from names: precision native|ozaki|bf16x3|tensor, layout
    reference|reduced; slices, tile_n (32/64/96) and native_fill (per mille)
    apply to the tensor-core forms."""
    return ContractOpts(_lib.PRECISIONS[precision], _lib.LAYOUTS[layout], int(slices), int(tile_n),
                        int(native_fill), 0)


class ContractionPlan:
    """The symbolic stage of a contraction, kept for repeated numeric runs
    (tq_plan_create / tq_plan_execute)."""

    def __init__(self, A: BlockSparseTensor, B: BlockSparseTensor, contracting_indices,
                 precision="native", layout="reference", slices=0, tile_n=0, native_fill=0,
                 stream=None):
        ci = np.asarray(contracting_indices, dtype=np.int64).reshape(-1, 2)
        al, bl = _i64(ci[:, 0]), _i64(ci[:, 1])
        opts = make_opts(precision, layout, slices, tile_n, native_fill)
        self.layout = opts.layout
        self._p = ctypes.c_void_p()
        h = ctypes.c_void_p()
        self.A, self.B = A, B  # keep the operands alive
        check(load().tq_plan_create(A._h, B._h, ci.shape[0], _p64(al), _p64(bl),
                                    ctypes.byref(opts), _stream(stream), ctypes.byref(self._p),
                                    ctypes.byref(h)))
        self.result = BlockSparseTensor(_handle=h)

    def execute(self, stream=None):
        check(load().tq_plan_execute(self._p, _stream(stream)))
        return self.result

    def execute_to(self, dst, stream=None):
        """Numeric stage with the result written into dst (tq_plan_execute_to):
        a torch tensor on the GPU, a page-locked torch CPU tensor (written by
        the kernels over the host link as they run) or a numpy array (one copy
        after the GEMM).  dst holds result.n_elem elements of the result's
        dtype; host destinations are complete on return."""
        n = self.result.n_elem if self.result.rank else 1
        dt = np.dtype(self.result.dtype)
        if hasattr(dst, "data_ptr"):
            ptr = dst.data_ptr()
            kind = TQ_MEM_DEVICE if dst.is_cuda else TQ_MEM_HOST
            size = dst.numel() * dst.element_size()
        else:
            if not (isinstance(dst, np.ndarray) and dst.flags.c_contiguous and dst.dtype == dt):
                raise ValueError("dst must be a contiguous %s array" % dt)
            ptr, kind, size = dst.ctypes.data, TQ_MEM_HOST, dst.nbytes
        if size < n * dt.itemsize:
            raise ValueError("dst holds %d bytes; the result needs %d" % (size, n * dt.itemsize))
        check(load().tq_plan_execute_to(self._p, ctypes.c_void_p(ptr), kind, _stream(stream)))

    def check(self, stream=None):
        """Raise if a bounded device wait of the last execute gave up (syncs)."""
        check(load().tq_plan_check(self._p, _stream(stream)))

    def set_profiling(self, enable: bool = True):
        check(load().tq_plan_set_profiling(self._p, 1 if enable else 0))

    def last_timings(self):
        """(prepare_ms, gemm_ms) of the last profiled execute, from CUDA events
        recorded on the launching stream."""
        a = ctypes.c_float()
        b = ctypes.c_float()
        check(load().tq_plan_last_timings(self._p, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    @property
    def flops(self) -> float:
        f = ctypes.c_double()
        n = ctypes.c_int64()
        check(load().tq_plan_flops(self._p, ctypes.byref(f), ctypes.byref(n)))
        return f.value

    @property
    def n_pairs(self) -> int:
        f = ctypes.c_double()
        n = ctypes.c_int64()
        check(load().tq_plan_flops(self._p, ctypes.byref(f), ctypes.byref(n)))
        return n.value

    def reschedule(self, precision="native", slices=0, tile_n=0, native_fill=0, stream=None):
        """A new schedule for this plan (tq_plan_reschedule); the layout stays."""
        o = make_opts(precision, "reference", slices, tile_n, native_fill)
        o.layout = self.layout
        check(load().tq_plan_reschedule(self._p, ctypes.byref(o), _stream(stream)))

    def features(self, target_rel_err: float, stream=None) -> np.ndarray:
        """The cost model's TQ_N_FEATURES inputs for this contraction (tq_plan_features)."""
        f = (ctypes.c_float * _lib.TQ_N_FEATURES)()
        check(load().tq_plan_features(self._p, float(target_rel_err), f, _stream(stream)))
        return np.ctypeslib.as_array(f).copy()

    def autotune(self, target_rel_err: float, candidates, reps: int = 3, stream=None):
        """Exhaustive autotuning (tq_autotune) over candidate schedules, each a
        dict of make_opts keywords.  Returns (best index or -1, [(status, ms,
        rel_err)]); the plan keeps the winner's schedule."""
        n = len(candidates)
        arr = (_lib.TuneEntry * max(n, 1))()
        for i, c in enumerate(candidates):
            o = make_opts(c.get("precision", "native"), "reference", c.get("slices", 0),
                          c.get("tile_n", 0), c.get("native_fill", 0))
            o.layout = self.layout
            arr[i].opts = o
        best = ctypes.c_int32()
        check(load().tq_autotune(self._p, float(target_rel_err), arr, n, int(reps),
                                 ctypes.byref(best), _stream(stream)))
        return best.value, [(arr[i].status, arr[i].ms, arr[i].rel_err) for i in range(n)]

    def __del__(self):
        p = getattr(self, "_p", None)
        if p is not None and p.value:
            try:
                load().tq_plan_destroy(p)
            except Exception:
                pass
            self._p = ctypes.c_void_p()


class Batch:
    """Many planned contractions as one numeric stage (tq_batch_*): the
    tensor-core plans of each wave share one persistent GEMM launch; the whole
    batch can be captured once as a CUDA graph and replayed."""

    def __init__(self, plans, waves=None, stream=None):
        self.plans = list(plans)  # keep the plans (and their tensors) alive
        n = len(self.plans)
        arr = (ctypes.c_void_p * max(n, 1))(*[p._p.value for p in self.plans])
        w = None
        if waves is not None:
            w = (ctypes.c_int32 * max(n, 1))(*[int(x) for x in waves])
        self._b = ctypes.c_void_p()
        check(load().tq_batch_create(arr, n, w, _stream(stream), ctypes.byref(self._b)))

    def execute(self, stream=None):
        check(load().tq_batch_execute(self._b, _stream(stream)))

    def graph_launch(self, stream=None):
        check(load().tq_batch_graph_launch(self._b, _stream(stream)))

    def check(self, stream=None):
        check(load().tq_batch_check(self._b, _stream(stream)))

    @property
    def kernels(self) -> int:
        k = ctypes.c_int64()
        check(load().tq_batch_kernels(self._b, ctypes.byref(k)))
        return k.value

    def __del__(self):
        b = getattr(self, "_b", None)
        if b is not None and b.value:
            try:
                load().tq_batch_destroy(b)
            except Exception:
                pass
            self._b = ctypes.c_void_p()
