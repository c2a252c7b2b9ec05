"""Inputs of the cases pinned by ``ref_outputs.npz``, and the per-block value
digest the large cases are stored as.

The outputs in ``ref_outputs.npz`` come from the reference's own CPU
``BlockSparseTensor<double>`` (src/tensor/block_sparse.h, block_sparse.cpp of
Walter-Feng/Torque), compiled from its sources and run by
``make_ref_outputs.py``.  Every input here is regenerated, not stored: numpy's
PCG64 stream (``np.random.default_rng``) is the same on every platform, and
``input_digest`` of each case is stored beside its outputs so a test can
confirm it rebuilt the same inputs.

Cases:
* ``u1_85`` / ``u1_85_swapped``: the 85-block U(1) rank-4 pair (sector sizes
  3,5,8,5,3; 325 matched pairs) contracted over legs (2,3) x (0,1), once with
  the contracting-index rows in order and once swapped;
* ``ragged_*``: boxes drawn at random, overlapping one another and meeting the
  other operand's boxes on part of their contracted intervals (the sub-box
  rule of block_in_range), some A blocks with no partner;
* ``vector_dot``: rank-1 operands contracted to a scalar;
* ``one_block_many_partners``: one A block meeting three B blocks; the
  reference as it is reads the index table of A's block 1, 2 and throws;
* ``custom_tables_r3_k1``: a ragged contraction whose operands store their
  odd blocks row-major (index tables given to append_block);
* ``transpose_r4``: leg permutations of a ragged rank-4 tensor whose blocks
  have legs of extent 1 (equal stride-table entries);
* ``transpose_r4_rowmajor``: the same permutations of a ragged rank-4 tensor
  whose odd blocks are stored row-major (no extent-1 legs: see below);
* ``modify_r3``: element writes and reads on overlapping blocks;
* ``FLOAT_CASES``: three of the contractions again through the reference's
  ``BlockSparseTensor<float>`` (inputs rounded to float32);
* ``query_r3``: element reads of an overlapping rank-3 tensor (overlaps add).
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

_ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if _ROOT not in sys.path:
    sys.path.insert(0, _ROOT)

from oracle.oracle import HostBS  # noqa: E402

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_outputs.npz")


def _random_boxes(rng, dims, n_blocks, max_extent=4):
    begin = np.zeros((n_blocks, len(dims)), np.int64)
    end = np.zeros_like(begin)
    for b in range(n_blocks):
        for l, d in enumerate(dims):
            lo = int(rng.integers(0, d))
            ext = int(rng.integers(1, min(max_extent, d - lo) + 1))
            begin[b, l], end[b, l] = lo, lo + ext - 1
    return begin, end


def random_tensor(rng, dims, n_blocks, max_extent=4) -> HostBS:
    dims = np.asarray(dims, np.int64)
    begin, end = _random_boxes(rng, dims, n_blocks, max_extent)
    n = int(np.prod(end - begin + 1, axis=1).sum())
    return HostBS(dims, begin, end, rng.standard_normal(n))


def u1_85(swapped: bool = False):
    from torque_gb300 import workloads
    c = workloads.small_u1()
    A = HostBS(c.A.dimension, c.A.begin, c.A.end, c.a_data)
    B = HostBS(c.B.dimension, c.B.begin, c.B.end, c.b_data)
    pairs = np.asarray(c.pairs, np.int64)
    return A, B, (pairs[::-1].copy() if swapped else pairs)


def ragged(seed: int, dims_a, dims_b, pairs, n_a: int = 7, n_b: int = 8, max_extent: int = 4):
    rng = np.random.default_rng(seed)
    return (random_tensor(rng, dims_a, n_a, max_extent), random_tensor(rng, dims_b, n_b, max_extent),
            np.asarray(pairs, np.int64))


# name -> builder returning (A, B, contracting-index pairs)
CONTRACTIONS = {
    "u1_85": lambda: u1_85(False),
    "u1_85_swapped": lambda: u1_85(True),
    "ragged_r3_k1": lambda: ragged(11, [6, 9, 5], [9, 4, 7], [[1, 0]]),
    "ragged_r3_k1_last": lambda: ragged(12, [5, 6, 8], [7, 6, 8], [[2, 2]]),
    "ragged_r3_k2": lambda: ragged(13, [7, 6, 5], [6, 7, 4], [[1, 0], [0, 1]]),
    "ragged_r3_k2_unsorted": lambda: ragged(14, [7, 6, 5], [5, 7, 4], [[2, 0], [0, 1]]),
    "ragged_r4_r2_k2": lambda: ragged(15, [5, 6, 4, 7], [4, 6], [[2, 0], [1, 1]], n_a=9, n_b=6),
    "ragged_r2_r4_k1": lambda: ragged(16, [6, 8], [5, 8, 3, 4], [[1, 1]], n_a=5, n_b=9),
    "vector_dot": lambda: ragged(17, [12], [12], [[0, 0]], n_a=4, n_b=5, max_extent=6),
    "custom_tables_r3_k1": lambda: custom_tables_case(),
    "one_block_many_partners": lambda: (
        HostBS(np.array([4, 6]), [[0, 0]], [[3, 5]], np.random.default_rng(18).standard_normal(24)),
        HostBS(np.array([6, 3]), [[0, 0], [2, 1], [4, 0]], [[1, 2], [3, 2], [5, 1]],
               np.random.default_rng(19).standard_normal(6 + 4 + 4)),
        np.array([[1, 0]], np.int64)),
}

# contractions also stored from the reference's float instantiation
FLOAT_CASES = ("u1_85", "ragged_r3_k2_unsorted", "custom_tables_r3_k1")

TRANSPOSE_PERMS = ([3, 1, 0, 2], [1, 0, 2, 3], [0, 1, 2, 3], [2, 3, 1, 0])


def transpose_r4() -> HostBS:
    rng = np.random.default_rng(21)
    T = random_tensor(rng, [4, 5, 3, 6], 8, max_extent=3)
    # force some legs of extent 1 so that stride-table entries repeat
    T.end[1, 0], T.end[1, 1] = T.begin[1, 0], T.begin[1, 1]
    T.end[4, 2] = T.begin[4, 2]
    T.end[6, :3] = T.begin[6, :3]
    n = int(np.prod(T.end - T.begin + 1, axis=1).sum())
    return HostBS(T.dimension, T.begin, T.end, rng.standard_normal(n))


def transpose_r4_rowmajor() -> HostBS:
    """A ragged rank-4 tensor whose odd blocks are stored row-major.  Every leg
    of every block has extent 2 or 3: with a leg of extent 1 a row-major
    index table has two equal entries, and the reference's hard_transpose
    (block_sparse.h:607-651, through index_to_indices with a sort of the table,
    space.h:44-59) then gives the extent-1 leg the quotient of its neighbour
    and writes outside the block."""
    rng = np.random.default_rng(25)
    dims = np.array([4, 5, 3, 6], np.int64)
    nb = 8
    begin = np.zeros((nb, 4), np.int64)
    end = np.zeros_like(begin)
    for b in range(nb):
        for l, d in enumerate(dims):
            lo = int(rng.integers(0, d - 1))
            ext = int(rng.integers(2, min(3, d - lo) + 1))
            begin[b, l], end[b, l] = lo, lo + ext - 1
    n = int(np.prod(end - begin + 1, axis=1).sum())
    return with_custom_tables(HostBS(dims, begin, end, rng.standard_normal(n)))


def transpose_cases():
    """Name -> tensor for the transposition fixtures."""
    return {"transpose_r4": transpose_r4(), "transpose_r4_rowmajor": transpose_r4_rowmajor()}


def query_r3():
    rng = np.random.default_rng(22)
    T = random_tensor(rng, [6, 5, 7], 9, max_extent=4)
    points = np.stack([rng.integers(0, d, 64) for d in T.dimension], 1).astype(np.int64)
    return T, points


def with_custom_tables(T: HostBS) -> HostBS:
    """The same boxes and values with every odd block stored row-major (last
    leg fastest): index table entries are the products of the later legs'
    extents, as append_block accepts them."""
    dims = T.end - T.begin + 1
    tables = T.strides.copy()
    data = T.data.copy()
    for b in range(1, T.n_blocks, 2):
        d = dims[b]
        t = np.ones_like(d)
        for l in range(len(d) - 2, -1, -1):
            t[l] = t[l + 1] * d[l + 1]
        tables[b] = t
        o, n = int(T.offsets[b]), int(np.prod(d))
        # column-major values -> the same elements in row-major order
        data[o:o + n] = T.data[o:o + n].reshape(tuple(d[::-1])).transpose().reshape(-1)
    return HostBS(T.dimension, T.begin, T.end, data, strides=tables, offsets=T.offsets)


def custom_tables_case():
    """A ragged rank-3 x rank-3 contraction over one leg whose operands store
    their odd blocks row-major."""
    A, B, pairs = ragged(24, [6, 5, 7], [5, 6, 4], [[1, 0]])
    return with_custom_tables(A), with_custom_tables(B), pairs


def modify_r3():
    """An overlapping rank-3 tensor and a seeded sequence of element writes and
    reads: writes inside overlaps (the first block holding the element gets
    the value, the others zero), outside every block (a nonzero value appends
    a one-element block, a zero does nothing), and reads after them."""
    rng = np.random.default_rng(23)
    T = random_tensor(rng, [5, 6, 4], 7, max_extent=3)
    ops = []
    for q in range(48):
        idx = [int(rng.integers(0, d)) for d in T.dimension]
        if q % 3 == 2:
            ops.append(("query", idx, 0.0))
        else:
            value = 0.0 if q % 7 == 0 else float(np.round(rng.standard_normal(), 6))
            ops.append(("modify", idx, value))
    return T, ops


def input_digest(*tensors) -> str:
    h = hashlib.sha256()
    for T in tensors:
        for a in (T.dimension, T.begin, T.end, T.data):
            h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def block_sizes(begin, end) -> np.ndarray:
    return np.prod(np.asarray(end) - np.asarray(begin) + 1, axis=1).astype(np.int64)


def value_digest(offsets, sizes, data) -> np.ndarray:
    """Per block: [sum, weighted sum (weights cos(0.618 k) over the block's
    elements in storage order), sum of |v|, max |v|, first, last element]."""
    out = np.zeros((len(sizes), 6), np.float64)
    for i, (o, n) in enumerate(zip(offsets, sizes)):
        v = data[o:o + n]
        w = np.cos(0.618 * np.arange(n))
        out[i] = [v.sum(), (v * w).sum(), np.abs(v).sum(), np.abs(v).max(), v[0], v[-1]]
    return out


def digest_close(got, want, sizes, tol) -> bool:
    """Digests of two results agree when every element agrees within
    tol * max|C| (max|C| from the stored digest): the three sums may then
    differ by the block size times that, the other entries by that."""
    scale = tol * max(float(np.max(want[:, 3])), 1e-300)
    bound = np.repeat(np.asarray(sizes, np.float64)[:, None] * scale, 6, axis=1)
    bound[:, 3:] = scale
    return bool(np.all(np.abs(np.asarray(got) - want) <= bound))


def load():
    with np.load(FIXTURE, allow_pickle=False) as z:
        return {k: z[k] for k in z.files}
