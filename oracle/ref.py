"""Python access to the reference's own CPU block-sparse tensor (oracle/_ref/).

TEST INFRASTRUCTURE ONLY.  ``build_ref.py`` compiles the reference's
``BlockSparseTensor<T>``, T double or float (src/tensor/block_sparse.h, block_sparse.cpp of
Walter-Feng/Torque) against the project's Armadillo API subset, in two
variants: ``"asis"`` (the headers unchanged) and ``"fixed"`` (the CPU
contract's two stride lookups corrected, block_sparse.h:531,538).  The
libraries exist only where the reference's sources were available to compile
them; ``available()`` says whether they are here.

Tensors are passed as ``oracle.HostBS`` and results come back in the same
form as ``oracle.contract`` (reference layout: output begin/end
[n_blocks, rank], offsets, values; a float for a rank-0 result), so a test
can compare the two directly.
"""
from __future__ import annotations

import ctypes
import glob
import os

import numpy as np

from . import build_ref
from .oracle import HostBS

_libs: dict = {}
_blas_keep: list = []   # loaded BLAS libraries stay open while registered


class RefError(RuntimeError):
    """The reference threw: ``status`` 1 for its own Error type, 2 for any
    other exception (an Armadillo-style bounds error)."""

    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


def available(variant: str = "fixed") -> bool:
    return os.path.exists(os.path.join(build_ref.OUT, build_ref.LIBS[variant]))


def lib(variant: str = "fixed"):
    if variant not in _libs:
        path = os.path.join(build_ref.OUT, build_ref.LIBS[variant])
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = ctypes.CDLL(path)
        U = ctypes.POINTER(ctypes.c_uint64)
        PP = ctypes.POINTER(ctypes.c_void_p)
        L.ref_last_error.restype = ctypes.c_char_p
        L.ref_tensor_new.restype = ctypes.c_int32
        L.ref_tensor_new.argtypes = [ctypes.c_int32, ctypes.c_int32, U, ctypes.c_int64, U, U,
                                     ctypes.c_void_p, PP]
        L.ref_tensor_new_empty.restype = ctypes.c_int32
        L.ref_tensor_new_empty.argtypes = [ctypes.c_int32, ctypes.c_int32, U, PP]
        L.ref_tensor_free.argtypes = [ctypes.c_void_p]
        L.ref_append_block.restype = ctypes.c_int32
        L.ref_append_block.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, U, U,
                                       U]
        L.ref_contract.restype = ctypes.c_int32
        L.ref_contract.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, U, PP]
        L.ref_hard_transpose.restype = ctypes.c_int32
        L.ref_hard_transpose.argtypes = [ctypes.c_void_p, U, PP]
        L.ref_query.restype = ctypes.c_int32
        L.ref_query.argtypes = [ctypes.c_void_p, ctypes.c_int32, U,
                                ctypes.POINTER(ctypes.c_double)]
        L.ref_modify.restype = ctypes.c_int32
        L.ref_modify.argtypes = [ctypes.c_void_p, ctypes.c_int32, U, ctypes.c_double]
        L.ref_tensor_info.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32),
                                      ctypes.POINTER(ctypes.c_int32),
                                      ctypes.POINTER(ctypes.c_int64),
                                      ctypes.POINTER(ctypes.c_int64)]
        L.ref_tensor_read.argtypes = [ctypes.c_void_p, U, U, U, U, U, ctypes.c_void_p]
        L.ref_block_in_range.restype = ctypes.c_int64
        L.ref_block_in_range.argtypes = [ctypes.c_int32, U, ctypes.c_int32, U, U,
                                         ctypes.c_int32, ctypes.c_int64, U, U, U, U, U,
                                         ctypes.c_int64]
        L.ref_set_dgemm.argtypes = [ctypes.c_void_p]
        L.ref_product_seconds.restype = ctypes.c_double
        _libs[variant] = L
    return _libs[variant]


# element types: the reference's double and float instantiations
_CODE = {np.dtype(np.float64): 0, np.dtype(np.float32): 1}
_NP = {0: np.float64, 1: np.float32}


def _u(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))


def _check(L, status: int):
    if status:
        raise RefError(status, L.ref_last_error().decode())


class RefTensor:
    """An owned handle on a reference tensor."""

    def __init__(self, L, handle: ctypes.c_void_p):
        self.L, self.h = L, handle

    @property
    def dtype(self):
        dt, r, nb, ne = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int64()
        self.L.ref_tensor_info(self.h, ctypes.byref(dt), ctypes.byref(r), ctypes.byref(nb),
                               ctypes.byref(ne))
        return _NP[dt.value]

    @classmethod
    def empty(cls, dimension, variant: str = "fixed", dtype=np.float64) -> "RefTensor":
        """BlockSparseTensor<T>(dimension): no blocks (a rank-0 tensor holds 0);
        T is double or float after dtype."""
        L = lib(variant)
        dim = np.ascontiguousarray(dimension, np.uint64).reshape(-1)
        h = ctypes.c_void_p()
        _check(L, L.ref_tensor_new_empty(_CODE[np.dtype(dtype)], dim.size,
                                         _u(dim if dim.size else np.zeros(1, np.uint64)),
                                         ctypes.byref(h)))
        return cls(L, h)

    @classmethod
    def from_host(cls, T: HostBS, variant: str = "fixed", dtype=np.float64) -> "RefTensor":
        """The constructor from values (column-major blocks), the values rounded
        to dtype (double or float); blocks with other index tables are added
        one by one with append_block, which keeps the given table."""
        if T.n_blocks == 0:
            return cls.empty(T.dimension, variant, dtype)
        dims = T.end - T.begin + 1
        compact = np.ones_like(dims)
        if T.rank > 1:
            compact[:, 1:] = np.cumprod(dims[:, :-1], axis=1)
        if not np.array_equal(T.strides, compact):
            t = cls.empty(T.dimension, variant, dtype)
            for b in range(T.n_blocks):
                o, n = int(T.offsets[b]), int(np.prod(dims[b]))
                t.append_block(T.data[o:o + n], T.begin[b], T.end[b], T.strides[b])
            return t
        L = lib(variant)
        dim = np.ascontiguousarray(T.dimension, np.uint64)
        beg = np.ascontiguousarray(T.begin, np.uint64)   # [n_blocks, rank] = rank x n col-major
        end = np.ascontiguousarray(T.end, np.uint64)
        data = np.ascontiguousarray(T.data, dtype)
        h = ctypes.c_void_p()
        _check(L, L.ref_tensor_new(_CODE[np.dtype(dtype)], T.rank, _u(dim), T.n_blocks, _u(beg),
                                   _u(end), data.ctypes.data_as(ctypes.c_void_p),
                                   ctypes.byref(h)))
        return cls(L, h)

    def __del__(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.L.ref_tensor_free(self.h)
            self.h = None

    def read(self):
        """(dimension, begin [nb, rank], end, index tables [nb, rank], offsets,
        values); a rank-0 tensor has empty metadata and one value."""
        dt, rank, nb, ne = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int64()
        self.L.ref_tensor_info(self.h, ctypes.byref(dt), ctypes.byref(rank), ctypes.byref(nb),
                               ctypes.byref(ne))
        r, n = rank.value, nb.value
        dim = np.zeros(max(r, 1), np.uint64)
        beg = np.zeros(max(r * n, 1), np.uint64)
        end = np.zeros_like(beg)
        tab = np.zeros_like(beg)
        off = np.zeros(max(n, 1), np.uint64)
        data = np.zeros(max(ne.value, 1), _NP[dt.value])
        self.L.ref_tensor_read(self.h, _u(dim), _u(beg), _u(end), _u(tab), _u(off),
                               data.ctypes.data_as(ctypes.c_void_p))
        shape = (n, r)
        return (dim[:r].astype(np.int64), beg[:r * n].reshape(shape).astype(np.int64),
                end[:r * n].reshape(shape).astype(np.int64),
                tab[:r * n].reshape(shape).astype(np.int64), off[:n].astype(np.int64),
                data[:ne.value])

    def host(self) -> HostBS:
        """The tensor as a HostBS (values widened to float64)."""
        dim, beg, end, tab, off, data = self.read()
        return HostBS(dim, beg, end, data, strides=tab, offsets=off)

    def contract(self, other: "RefTensor", pairs) -> "RefTensor":
        legs = _legs(pairs)
        h = ctypes.c_void_p()
        _check(self.L, self.L.ref_contract(self.h, other.h, legs.size // 2, _u(legs),
                                           ctypes.byref(h)))
        return RefTensor(self.L, h)

    def hard_transpose(self, perm) -> "RefTensor":
        p = np.ascontiguousarray(perm, np.uint64)
        h = ctypes.c_void_p()
        _check(self.L, self.L.ref_hard_transpose(self.h, _u(p), ctypes.byref(h)))
        return RefTensor(self.L, h)

    def query(self, idx) -> float:
        i = np.ascontiguousarray(idx, np.uint64).reshape(-1)
        v = ctypes.c_double()
        _check(self.L, self.L.ref_query(self.h, i.size, _u(i if i.size else np.zeros(1, np.uint64)),
                                        ctypes.byref(v)))
        return v.value

    def modify(self, idx, number: float) -> None:
        i = np.ascontiguousarray(idx, np.uint64).reshape(-1)
        _check(self.L, self.L.ref_modify(self.h, i.size, _u(i if i.size else np.zeros(1, np.uint64)),
                                         float(number)))

    def append_block(self, data, begin, end, table) -> None:
        d = np.ascontiguousarray(data, self.dtype)
        b, e, t = (np.ascontiguousarray(x, np.uint64).reshape(-1) for x in (begin, end, table))
        _check(self.L, self.L.ref_append_block(self.h, b.size, d.ctypes.data_as(ctypes.c_void_p),
                                               _u(b), _u(e), _u(t)))


def _legs(pairs) -> np.ndarray:
    p = np.asarray(pairs, np.uint64).reshape(-1, 2)
    return np.ascontiguousarray(p.T.reshape(-1))          # n x 2 column-major


def contract(A: HostBS, B: HostBS, pairs, variant: str = "fixed", dtype=np.float64):
    """The reference's CPU contract, in double or (dtype float32) float.
    Returns (begin, end, offsets, values) in the reference layout, or a float
    for a rank-0 result; raises RefError where the reference throws."""
    a, b = RefTensor.from_host(A, variant, dtype), RefTensor.from_host(B, variant, dtype)
    dim, beg, end, _, off, data = a.contract(b, pairs).read()
    if dim.size == 0:
        return float(data[0])
    return beg, end, off, data


def hard_transpose(T: HostBS, perm, variant: str = "fixed") -> HostBS:
    return RefTensor.from_host(T, variant).hard_transpose(perm).host()


def query(T: HostBS, idx, variant: str = "fixed") -> float:
    return RefTensor.from_host(T, variant).query(idx)


def block_in_range(pairs, a_begin, a_end, b_begin, b_end, variant: str = "fixed",
                   boxes: bool = False):
    """Indices of the B blocks (rows of b_begin/b_end, [n_b, rank]) whose
    contracted intervals meet the A block (a_begin/a_end, [rank]); with
    boxes=True also each pair's output box as (indices, begin [count, rank_out],
    end [count, rank_out])."""
    L = lib(variant)
    legs = _legs(pairs)
    ab = np.ascontiguousarray(a_begin, np.uint64)
    ae = np.ascontiguousarray(a_end, np.uint64)
    bb = np.ascontiguousarray(b_begin, np.uint64)
    be = np.ascontiguousarray(b_end, np.uint64)
    nb = bb.shape[0]
    ro = ab.size + bb.shape[1] - 2 * (legs.size // 2)
    found = np.zeros(max(nb, 1), np.uint64)
    nbeg = np.zeros(max(nb * max(ro, 1), 1), np.uint64) if boxes else None
    nend = np.zeros_like(nbeg) if boxes else None
    n = L.ref_block_in_range(legs.size // 2, _u(legs), ab.size, _u(ab), _u(ae), bb.shape[1], nb,
                             _u(bb), _u(be), _u(found), _u(nbeg) if boxes else None,
                             _u(nend) if boxes else None, nb)
    if n < 0:
        raise RefError(2, L.ref_last_error().decode())
    idx = found[:n].astype(np.int64)
    if not boxes:
        return idx
    return (idx, nbeg[:n * ro].reshape(n, ro).astype(np.int64),
            nend[:n * ro].reshape(n, ro).astype(np.int64))


def use_blas(threads: int = 1, variant: str = "fixed") -> str | None:
    """Route the reference's matrix products through the OpenBLAS that scipy
    ships (the reference reaches BLAS through Armadillo), with the given
    thread count.  Returns the library's file name, or None if none is found
    (the products then use the plain loop)."""
    try:
        import scipy
    except ImportError:
        return None
    libdir = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
    for path in sorted(glob.glob(os.path.join(libdir, "libscipy_openblas*.so"))):
        blas = ctypes.CDLL(path)
        for gemm, setter in (("scipy_dgemm_", "scipy_openblas_set_num_threads"),
                             ("dgemm_", "openblas_set_num_threads")):
            if hasattr(blas, gemm):
                if hasattr(blas, setter):
                    getattr(blas, setter)(ctypes.c_int(threads))
                fn = ctypes.cast(getattr(blas, gemm), ctypes.c_void_p)
                lib(variant).ref_set_dgemm(fn)
                _blas_keep.append(blas)
                return os.path.basename(path)
    return None


def use_loop(variant: str = "fixed") -> None:
    lib(variant).ref_set_dgemm(None)


def product_seconds(variant: str = "fixed") -> float:
    return lib(variant).ref_product_seconds()


def reset_product_seconds(variant: str = "fixed") -> None:
    lib(variant).ref_reset_product_seconds()
