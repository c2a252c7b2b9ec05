"""The dense and element-sparse classes (torque_gb300.dense) on the reference's
known-answer tests: test/gpu/dense_test.cu:7-300 and
test/gpu/sparse_test.cu:31-319 (float32 in the reference; both float32 and
float64 here), plus a dense check against numpy tensordot."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

A12 = [1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12]


@pytest.fixture(params=[np.float32, np.float64])
def dt(request):
    return request.param


def test_dense_initialization_and_transposition(tq, dt):
    from torque_gb300.dense import DenseTensor
    t = DenseTensor([4, 3], dtype=dt)
    assert t.query([1, 1]) == 0
    t.initialize(A12)
    assert t.query([1, 2]) == 10
    t = t.hard_transpose([1, 0])  # 3 x 4
    assert t.query([1, 2]) == 7
    tt = t.hard_transpose([1, 0])
    for i in range(3):
        for j in range(4):
            assert t.query([i, j]) == tt.query([j, i])
    u = DenseTensor([2, 2, 3], dtype=dt)
    assert u.query([1, 1, 0]) == 0
    u.initialize(A12)
    assert u.query([0, 1, 2]) == 11
    v = DenseTensor([2, 2, 3], A12, dtype=dt)
    assert v.query([0, 0, 2]) == 9 and v.query([0, 1, 2]) == 11
    v = v.hard_transpose([0, 2, 1])
    assert v.query([0, 2, 0]) == 9 and v.query([0, 2, 1]) == 11
    w = v.hard_transpose([1, 0, 2])
    assert w.query([2, 0, 0]) == 9 and w.query([2, 0, 1]) == 11
    s = DenseTensor([], dtype=dt)
    assert s.rank == 0 and s.query([]) == 0
    s.modify([], 1)
    assert s.query([]) == 1
    with pytest.raises(tq.TorqueError):
        u.query([2, 0, 0])
    with pytest.raises(tq.TorqueError):
        u.query([0, 0])


def test_dense_contractions(tq, dt):
    from torque_gb300.dense import DenseTensor
    vec = DenseTensor([5], [0, 1, 2, 3, 4], dtype=dt)
    assert vec.contract(vec, [[0, 0]]).to_number() == 30
    m = DenseTensor([3, 3], list(range(9)), dtype=dt)
    ref = np.arange(9.0).reshape(3, 3, order="F")
    sq = m.contract(m, [[1, 0]])
    for i in range(3):
        for j in range(3):
            assert sq.query([i, j]) == (ref @ ref)[i, j]
    assert m.contract(m, [[1, 0], [0, 1]]).to_number() == np.sum(ref * ref.T)
    t = DenseTensor([2, 2, 2], list(range(8)), dtype=dt)
    v2 = DenseTensor([2], [1, 2], dtype=dt)
    c = t.contract(v2, [[0, 0]])
    assert [c.query(x) for x in ([0, 0], [1, 0], [0, 1], [1, 1])] == [2, 8, 14, 20]
    c = t.contract(v2, [[1, 0]])
    assert [c.query(x) for x in ([0, 0], [1, 0], [0, 1], [1, 1])] == [4, 7, 16, 19]
    assert t.contract(v2, [[2, 0]]).query([1, 0]) == 11
    t3 = DenseTensor([2, 2, 3], list(range(12)), dtype=dt)
    mat = DenseTensor([2, 2], [1, 2, 3, 4], dtype=dt)
    c = t3.contract(mat, [[0, 1], [1, 0]])
    assert [c.query([k]) for k in range(3)] == [19, 59, 99]


def test_dense_against_numpy(tq):
    from torque_gb300.dense import DenseTensor
    rng = np.random.default_rng(3)
    a = rng.standard_normal((7, 9, 5))
    b = rng.standard_normal((5, 9, 4))
    A = DenseTensor(a.shape, a.ravel(order="F"))
    B = DenseTensor(b.shape, b.ravel(order="F"))
    C = A.contract(B, [[2, 0], [1, 1]])
    want = np.tensordot(a, b, axes=([2, 1], [0, 1]))
    got = C.data().reshape(want.shape, order="F")
    assert np.max(np.abs(got - want)) <= 1e-12 * np.max(np.abs(want))
    Z = A.contract(B, [[2, 0], [1, 1]], precision="ozaki", layout="reference")
    gz = Z.data().reshape(want.shape, order="F")
    assert np.max(np.abs(gz - want)) <= 1e-10 * np.max(np.abs(want))
    T = A.hard_transpose([2, 0, 1])
    assert np.array_equal(T.data().reshape((5, 7, 9), order="F"), a.transpose(2, 0, 1))


def test_sparse_known_answers(tq, dt):
    from torque_gb300.dense import SparseTensor, index_table
    t = SparseTensor([4, 3], dtype=dt)
    assert t.query([1, 1]) == 0
    t.initialize(A12, list(range(12)))
    assert t.query([1, 2]) == 10
    t.soft_transpose([1, 0])
    assert t.query([1, 2]) == 7
    tt = t.hard_transpose([1, 0])
    for i in range(3):
        for j in range(4):
            assert t.query([i, j]) == tt.query([j, i])
    u = SparseTensor([2, 2, 3], A12, list(range(12)), index_table([2, 2, 3]), dtype=dt)
    assert u.query([0, 0, 2]) == 9 and u.query([0, 1, 2]) == 11
    u.soft_transpose([0, 2, 1])
    assert u.query([0, 2, 0]) == 9 and u.query([0, 2, 1]) == 11
    w = u.hard_transpose([1, 0, 2])
    assert w.query([2, 0, 0]) == 9 and w.query([2, 0, 1]) == 11
    s = SparseTensor([], dtype=dt)
    assert s.rank == 0 and s.query([]) == 0
    s.modify([], 1)
    assert s.query([]) == 1
    vec = SparseTensor([5], [0, 1, 2, 3, 4], list(range(5)), dtype=dt)
    assert vec.contract(vec, [[0, 0]]).to_number() == 30
    m = SparseTensor([3, 3], list(range(9)), list(range(9)), dtype=dt)
    sq = m.contract(m, [[1, 0]])
    ref = [[15, 42, 69], [18, 54, 90], [21, 66, 111]]
    for i in range(3):
        for j in range(3):
            assert sq.query([i, j]) == ref[i][j]
    r = np.arange(9.0).reshape(3, 3, order="F")
    assert m.contract(m, [[1, 0], [0, 1]]).to_number() == np.sum(r * r.T)
    t3 = SparseTensor([2, 2, 2], list(range(8)), list(range(8)), dtype=dt)
    v2 = SparseTensor([2], [1, 2], [0, 1], dtype=dt)
    c = t3.contract(v2, [[0, 0]])
    assert [c.query(x) for x in ([0, 0], [1, 0], [0, 1], [1, 1])] == [2, 8, 14, 20]
    c = t3.contract(v2, [[1, 0]])
    assert [c.query(x) for x in ([0, 0], [1, 0], [0, 1], [1, 1])] == [4, 7, 16, 19]
    assert t3.contract(v2, [[2, 0]]).query([1, 0]) == 11
    t4 = SparseTensor([2, 2, 3], list(range(12)), list(range(12)), dtype=dt)
    mat = SparseTensor([2, 2], [1, 2, 3, 4], list(range(4)), dtype=dt)
    c = t4.contract(mat, [[0, 1], [1, 0]])
    assert [c.query([k]) for k in range(3)] == [19, 59, 99]
    # every output element is kept, in ascending linear order
    assert list(c.indices) == [0, 1, 2]


def test_sparse_random_against_dense(tq):
    """Random element-sparse tensors (20% fill) contracted over two legs,
    against numpy on the zero-filled arrays."""
    from torque_gb300.dense import SparseTensor
    rng = np.random.default_rng(11)
    da, db = (6, 5, 7), (7, 5, 4)
    a = np.where(rng.random(da) < 0.2, rng.standard_normal(da), 0.0)
    b = np.where(rng.random(db) < 0.2, rng.standard_normal(db), 0.0)
    ia, ib = np.flatnonzero(a.ravel(order="F")), np.flatnonzero(b.ravel(order="F"))
    A = SparseTensor(da, a.ravel(order="F")[ia], ia)
    B = SparseTensor(db, b.ravel(order="F")[ib], ib)
    C = A.contract(B, [[2, 0], [1, 1]])
    want = np.tensordot(a, b, axes=([2, 1], [0, 1]))
    got = np.zeros(want.size)
    got[C.indices] = C.values()
    got = got.reshape(want.shape, order="F")
    assert np.max(np.abs(got - want)) <= 1e-12 * max(np.max(np.abs(want)), 1e-300)
    assert np.all(np.diff(C.indices) > 0)


@pytest.mark.parametrize("dtype,tol", [(np.float64, 1e-12), (np.float32, 1e-5),
                                       (np.float16, 1e-3)])
def test_sort_join_matches_block_matcher(tq, dtype, tol):
    """The sort-join element contraction (tq_bs_contract_elements) against the
    block path over the same one-element blocks (all-pairs interval matching,
    reduced layout): the same output elements in the same order, values within
    the type's tolerance; repeated nonzeros (duplicate coordinates) are summed."""
    from torque_gb300 import block_sparse as bs
    rng = np.random.default_rng(23)
    da, db = (40, 16, 12), (16, 12, 30)
    na, nb = 3000, 2500
    pa = np.stack([rng.integers(0, d, na) for d in da], 1)
    pb = np.stack([rng.integers(0, d, nb) for d in db], 1)
    pa[1] = pa[0]  # a duplicate coordinate
    va = rng.standard_normal(na).astype(dtype)
    vb = rng.standard_normal(nb).astype(dtype)
    A = tq.BlockSparseTensor(da, va, pa.T, pa.T, dtype=dtype)
    B = tq.BlockSparseTensor(db, vb, pb.T, pb.T, dtype=dtype)
    pairs = [[1, 0], [2, 1]]
    S = bs.contract_elements(A, B, pairs)
    R = A.contract(B, pairs, layout="reduced")
    ds, sb, se, st, so = S.metadata()
    dr, rb, re_, rt, ro = R.metadata()
    assert np.array_equal(sb, rb) and np.array_equal(se, re_) and np.array_equal(so, ro)
    x, y = S.data().astype(np.float64), R.data().astype(np.float64)
    assert np.max(np.abs(x - y)) <= tol * np.max(np.abs(y))
    # against numpy on the dense arrays (duplicates summed)
    a = np.zeros(da)
    np.add.at(a, tuple(pa.T), va.astype(np.float64))
    b = np.zeros(db)
    np.add.at(b, tuple(pb.T), vb.astype(np.float64))
    want = np.tensordot(a, b, axes=([1, 2], [0, 1]))
    got = want * 0
    got[tuple(sb)] = x
    assert np.max(np.abs(got - want)) <= 10 * tol * np.max(np.abs(want))
