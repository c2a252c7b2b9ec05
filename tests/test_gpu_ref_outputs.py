"""The CUDA path against the reference's own CPU outputs.

tests/golden/ref_outputs.npz holds what the reference's
``BlockSparseTensor<double>`` (src/tensor/block_sparse.h, block_sparse.cpp),
compiled from its sources with its CPU contract's two stride lookups
corrected (block_sparse.h:531,538), returned on the cases of
tests/golden/ref_cases.py: the 85-block U(1) pair (both orders of the
contracting-index rows), ragged overlapping boxes met on part of their
contracted intervals, a one-leg scalar, a rank-4 transposition with extent-1
legs and overlapping element reads.  Through the C ABI: block lists, offsets
and index tables bit-exact; FP64 values within 1e-12 of max|C|; the
tensor-core Ozaki form (five slices, sector-aligned cases only) within 1e-10;
transposed values bit-exact.
"""
import sys

import numpy as np
import pytest

from conftest import GOLDEN

if GOLDEN not in sys.path:
    sys.path.insert(0, GOLDEN)
import ref_cases as rc  # noqa: E402

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOLOZ = 1e-10


@pytest.fixture(scope="module")
def fx():
    return rc.load()


def to_gpu(tq, T, dtype=np.float64):
    return tq.BlockSparseTensor(T.dimension, T.data.astype(dtype), T.begin.T, T.end.T,
                                T.strides.T, dtype=dtype)


def check(C, fx, key, tol):
    if key + "scalar" in fx:
        want = float(fx[key + "scalar"])
        assert C.rank == 0
        assert abs(C.to_number() - want) <= tol * max(abs(want), 1.0)
        return
    dim, b, e, t, o = C.metadata()
    assert np.array_equal(b.T, fx[key + "begin"]) and np.array_equal(e.T, fx[key + "end"])
    assert np.array_equal(o, fx[key + "offsets"])
    sizes = rc.block_sizes(b.T, e.T)
    data = C.data()
    if key + "values" in fx:
        want = fx[key + "values"]
        assert data.shape == want.shape
        assert np.max(np.abs(data - want)) <= tol * max(np.max(np.abs(want)), 1e-300)
    else:
        got = rc.value_digest(o, sizes, data)
        assert rc.digest_close(got, fx[key + "digest"], sizes, tol)


@pytest.mark.parametrize("name", list(rc.CONTRACTIONS))
def test_native_fp64_matches_reference(tq, fx, name):
    A, B, pairs = rc.CONTRACTIONS[name]()
    assert rc.input_digest(A, B) == str(fx[name + "__input"])
    C = to_gpu(tq, A).contract(to_gpu(tq, B), pairs)
    check(C, fx, name + "__fixed__", TOL64)


@pytest.mark.parametrize("name", rc.FLOAT_CASES)
def test_native_fp32_matches_reference_float(tq, fx, name):
    """Float tensors against the reference's float instantiation on the same
    inputs rounded to float32: block lists bit-exact, values within 1e-5 of
    max|C| (both accumulate in float, in different orders)."""
    A, B, pairs = rc.CONTRACTIONS[name]()
    C = to_gpu(tq, A, np.float32).contract(to_gpu(tq, B, np.float32), pairs)
    key = name + "__f32__"
    dim, b, e, t, o = C.metadata()
    assert np.array_equal(b.T, fx[key + "begin"]) and np.array_equal(e.T, fx[key + "end"])
    assert np.array_equal(o, fx[key + "offsets"])
    data = C.data().astype(np.float64)
    sizes = rc.block_sizes(b.T, e.T)
    if key + "values" in fx:
        want = fx[key + "values"].astype(np.float64)
        assert np.max(np.abs(data - want)) <= 1e-5 * np.max(np.abs(want))
    else:
        assert rc.digest_close(rc.value_digest(o, sizes, data), fx[key + "digest"], sizes, 1e-5)


@pytest.mark.parametrize("name", ["u1_85", "u1_85_swapped"])
def test_ozaki_matches_reference(tq, fx, name):
    A, B, pairs = rc.CONTRACTIONS[name]()
    C = to_gpu(tq, A).contract(to_gpu(tq, B), pairs, precision="ozaki", slices=5)
    check(C, fx, name + "__fixed__", TOLOZ)


@pytest.mark.parametrize("tname", ["transpose_r4", "transpose_r4_rowmajor"])
def test_transpose_matches_reference(tq, fx, tname):
    T = rc.transpose_cases()[tname]
    G = to_gpu(tq, T)
    for k, perm in enumerate(rc.TRANSPOSE_PERMS):
        key = "%s__%d__" % (tname, k)
        R = G.hard_transpose(perm)
        dim, b, e, t, o = R.metadata()
        assert np.array_equal(b.T, fx[key + "begin"]) and np.array_equal(e.T, fx[key + "end"])
        assert np.array_equal(t.T, fx[key + "tables"])
        assert np.array_equal(o, fx[key + "offsets"])
        assert np.array_equal(R.data(), fx[key + "values"])


def test_query_matches_reference(tq, fx):
    Q, points = rc.query_r3()
    G = to_gpu(tq, Q)
    want = fx["query_r3__values"]
    got = np.array([G.query(p) for p in points])
    assert np.max(np.abs(got - want)) <= 1e-14 * np.max(np.abs(want))


def test_modify_matches_reference(tq, fx):
    """A seeded sequence of element writes and reads on overlapping blocks
    (block_sparse.h:322-411): the reads, and the tensor afterwards (appended
    one-element blocks with their all-zero index tables, offsets, values),
    equal the reference's."""
    M, ops = rc.modify_r3()
    assert rc.input_digest(M) == str(fx["modify_r3__input"])
    G = to_gpu(tq, M)
    reads = []
    for kind, idx, value in ops:
        if kind == "modify":
            G.modify(idx, value)
        else:
            reads.append(G.query(idx))
    want = fx["modify_r3__reads"]
    assert np.max(np.abs(np.asarray(reads) - want)) <= 1e-14 * np.max(np.abs(want))
    dim, b, e, t, o = G.metadata()
    assert np.array_equal(b.T, fx["modify_r3__begin"]) and np.array_equal(e.T, fx["modify_r3__end"])
    assert np.array_equal(t.T, fx["modify_r3__tables"])
    assert np.array_equal(o, fx["modify_r3__offsets"])
    assert np.array_equal(G.data(), fx["modify_r3__values"])
