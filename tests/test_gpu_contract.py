"""Parity of the CUDA contraction path with the oracle (through the C ABI via
the Python mirror).  Integer work (pair list, boxes, offsets) is bit-exact;
FP64 values agree within 1e-12 of max|C| (the reference's tolerance claim),
FP32 within 1e-5, half (binary16 storage, FP32 accumulation, one rounding of
each output element) within 1e-3 against the oracle on the same rounded
inputs."""
import numpy as np
import pytest

from oracle import oracle as orc
from torque_gb300 import workloads

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 1e-5
TOL16 = 1e-3


def to_gpu(tq, dim, begin, end, data, tables=None, dtype=np.float64):
    return tq.BlockSparseTensor(dim, np.asarray(data, dtype), np.asarray(begin).T,
                                np.asarray(end).T,
                                None if tables is None else np.asarray(tables).T, dtype=dtype)


def host(dim, begin, end, data, tables=None):
    return orc.HostBS(np.asarray(dim), begin, end, data, strides=tables)


@pytest.fixture(scope="module")
def small():
    return workloads.small_u1()


def check_reference_layout(tq, A, B, hA, hB, pairs, dtype=np.float64, tol=TOL64):
    C = A.contract(B, pairs)
    ob, oe, off, want = orc.contract(hA, hB, pairs, mode=0)
    dim, b, e, t, o = C.metadata()
    assert np.array_equal(b.T, ob) and np.array_equal(e.T, oe)
    assert np.array_equal(o, off)
    dims = oe - ob + 1
    st = np.ones_like(dims)
    st[:, 1:] = np.cumprod(dims[:, :-1], axis=1)
    assert np.array_equal(t.T, st)
    got = C.data().astype(np.float64)
    assert got.shape == want.shape
    assert np.max(np.abs(got - want)) <= tol * max(np.max(np.abs(want)), 1e-300)
    return C


def test_small_u1_reference_layout(tq, small):
    c = small
    A = to_gpu(tq, c.A.dimension, c.A.begin, c.A.end, c.a_data)
    B = to_gpu(tq, c.B.dimension, c.B.begin, c.B.end, c.b_data)
    hA = host(c.A.dimension, c.A.begin, c.A.end, c.a_data)
    hB = host(c.B.dimension, c.B.begin, c.B.end, c.b_data)
    C = check_reference_layout(tq, A, B, hA, hB, c.pairs)
    assert C.n_blocks == 325


def test_small_u1_reduced_layout(tq, small):
    c = small
    A = to_gpu(tq, c.A.dimension, c.A.begin, c.A.end, c.a_data)
    B = to_gpu(tq, c.B.dimension, c.B.begin, c.B.end, c.b_data)
    hA = host(c.A.dimension, c.A.begin, c.A.end, c.a_data)
    hB = host(c.B.dimension, c.B.begin, c.B.end, c.b_data)
    C = A.contract(B, c.pairs, layout="reduced")
    assert C.n_blocks == 85
    dim, b, e, t, o = C.metadata()
    ob, oe, off, data = orc.contract(hA, hB, c.pairs, mode=0)
    boxes = np.unique(np.concatenate([ob, oe], 1), axis=0)
    order = np.lexsort(boxes[:, :4].T)  # leg 0 least significant: column-major sector order
    assert np.array_equal(b.T, boxes[order, :4]) and np.array_equal(e.T, boxes[order, 4:])
    got = orc.densify(host(dim, b.T, e.T, C.data(), t.T))
    want = orc.dense_contract(orc.densify(hA), orc.densify(hB), c.pairs)
    assert np.max(np.abs(got - want)) <= TOL64 * np.max(np.abs(want))


def test_small_u1_float32(tq, small):
    c = small
    A = to_gpu(tq, c.A.dimension, c.A.begin, c.A.end, c.a_data, dtype=np.float32)
    B = to_gpu(tq, c.B.dimension, c.B.begin, c.B.end, c.b_data, dtype=np.float32)
    a32 = c.a_data.astype(np.float32).astype(np.float64)
    b32 = c.b_data.astype(np.float32).astype(np.float64)
    hA = host(c.A.dimension, c.A.begin, c.A.end, a32)
    hB = host(c.B.dimension, c.B.begin, c.B.end, b32)
    check_reference_layout(tq, A, B, hA, hB, c.pairs, np.float32, TOL32)


def test_small_u1_float16(tq, small):
    c = small
    A = to_gpu(tq, c.A.dimension, c.A.begin, c.A.end, c.a_data, dtype=np.float16)
    B = to_gpu(tq, c.B.dimension, c.B.begin, c.B.end, c.b_data, dtype=np.float16)
    a16 = c.a_data.astype(np.float16).astype(np.float64)
    b16 = c.b_data.astype(np.float16).astype(np.float64)
    hA = host(c.A.dimension, c.A.begin, c.A.end, a16)
    hB = host(c.B.dimension, c.B.begin, c.B.end, b16)
    C = check_reference_layout(tq, A, B, hA, hB, c.pairs, np.float16, TOL16)
    assert C.dtype == np.float16
    # the rank-0 path (every leg contracted) in half, scaled to stay far below
    # the binary16 maximum (65504)
    X = to_gpu(tq, c.A.dimension, c.A.begin, c.A.end, 0.25 * c.a_data, dtype=np.float16)
    x16 = (0.25 * c.a_data).astype(np.float16).astype(np.float64)
    full = np.array([[0, 0], [1, 1], [2, 2], [3, 3]])
    s = A.contract(X, full).to_number()
    want = float(np.dot(a16, x16))
    assert abs(float(s) - want) <= TOL16 * abs(want)


def test_non_adjacent_free_legs(tq, small):
    """Contract the middle legs: A's free legs (0, 3) are not stride-contiguous,
    so the operand view keeps two row legs (general addressing path)."""
    c = small
    A = to_gpu(tq, c.A.dimension, c.A.begin, c.A.end, c.a_data)
    B = to_gpu(tq, c.B.dimension, c.B.begin, c.B.end, c.b_data)
    hA = host(c.A.dimension, c.A.begin, c.A.end, c.a_data)
    hB = host(c.B.dimension, c.B.begin, c.B.end, c.b_data)
    for pairs in ([[1, 0], [2, 1]], [[3, 2], [0, 3]], [[1, 3]]):
        check_reference_layout(tq, A, B, hA, hB, np.array(pairs))


@pytest.mark.parametrize("perm", [[1, 0, 2, 3], [3, 2, 1, 0], [0, 1, 3, 2], [2, 0, 3, 1],
                                  [0, 2, 3, 1], [0, 1, 2, 3]])
def test_hard_transpose_bit_exact(tq, small, perm):
    c = small
    A = to_gpu(tq, c.A.dimension, c.A.begin, c.A.end, c.a_data)
    hA = host(c.A.dimension, c.A.begin, c.A.end, c.a_data)
    T = A.hard_transpose(perm)
    want = orc.hard_transpose(hA, perm)
    dim, b, e, t, o = T.metadata()
    assert np.array_equal(dim, want.dimension)
    assert np.array_equal(b.T, want.begin) and np.array_equal(e.T, want.end)
    assert np.array_equal(T.data(), want.data)


@pytest.mark.parametrize("perm", [[0, 2, 1], [1, 0, 2], [2, 1, 0], [0, 1, 2]])
def test_hard_transpose_long_legs(tq, perm):
    """Blocks longer than one 32-wide tile on every leg (several tiles per
    block on both transposed legs, ragged edges), bit-exact with the oracle."""
    from torque_gb300.sectors import Leg, charge_blocks
    legs = [Leg([0, 1], [37, 70], 1), Leg([0, 1], [33, 5], -1), Leg([0, 1], [3, 41], 1)]
    bl = charge_blocks(legs, 0, modulus=2)
    data = np.random.default_rng(8).standard_normal(bl.n_elem)
    A = to_gpu(tq, bl.dimension, bl.begin, bl.end, data)
    want = orc.hard_transpose(host(bl.dimension, bl.begin, bl.end, data), perm)
    T = A.hard_transpose(perm)
    dim, b, e, t, o = T.metadata()
    assert np.array_equal(b.T, want.begin) and np.array_equal(e.T, want.end)
    assert np.array_equal(T.data(), want.data)


@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.float16])
def test_hard_transpose_all_permutations_dtypes(tq, dtype):
    """Every permutation of a rank-4 U(1) tensor with ragged sector sizes (odd
    block sizes, so block starts fall on every alignment; planes of one to
    several hundred elements; tiles read with 16-byte loads and with scalar
    loads), in float64, float32 and half: bit-exact with the oracle, and the
    inverse permutation restores the input."""
    import itertools
    from torque_gb300.sectors import Leg, charge_blocks
    legs = [Leg([0, 1, 2], [3, 50, 7], 1), Leg([0, 1, 2], [1, 48, 9], 1),
            Leg([0, 1, 2], [6, 2, 11], -1), Leg([0, 1, 2], [5, 4, 3], -1)]
    bl = charge_blocks(legs, 0)
    data = np.random.default_rng(12).standard_normal(bl.n_elem).astype(dtype)
    A = to_gpu(tq, bl.dimension, bl.begin, bl.end, data, dtype=dtype)
    hA = host(bl.dimension, bl.begin, bl.end, data.astype(np.float64))
    for perm in itertools.permutations(range(4)):
        T = A.hard_transpose(list(perm))
        want = orc.hard_transpose(hA, list(perm))
        dim, b, e, t, o = T.metadata()
        assert np.array_equal(b.T, want.begin) and np.array_equal(e.T, want.end)
        got = T.data()
        assert got.dtype == np.dtype(dtype)
        assert np.array_equal(got.astype(np.float64), want.data), perm
        # the inverse permutation runs from the result's device metadata
        back = T.hard_transpose(list(np.argsort(perm)))
        assert np.array_equal(back.data(), data), perm


@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.float16])
@pytest.mark.parametrize("perm", [[1, 0], [1, 0, 2], [1, 0, 3, 2], [1, 0, 2, 3]])
def test_hard_transpose_whole_planes(tq, dtype, perm):
    """Legs 0 and 1 swapped: planes contiguous on both sides move as whole
    planes through shared memory (bulk copies in and out, ragged 16-byte ends
    by threads), with plane sides odd and even in every combination (each
    takes its own conflict-free lane order), sides below 16 and planes too
    large for a stage taking the other paths; block starts on every
    alignment.  Bit-exact with the oracle, and the inverse restores the input."""
    from torque_gb300.sectors import Leg, charge_blocks
    sizes = [[17, 32, 5, 48], [23, 16, 40, 3], [2, 33], [31, 18]]
    legs = [Leg(list(range(len(z))), z, 1 if k % 2 == 0 else -1) for k, z in
            enumerate(sizes[:len(perm)])]
    bl = charge_blocks(legs, 0, modulus=2)
    data = np.random.default_rng(14).standard_normal(bl.n_elem).astype(dtype)
    A = to_gpu(tq, bl.dimension, bl.begin, bl.end, data, dtype=dtype)
    want = orc.hard_transpose(host(bl.dimension, bl.begin, bl.end, data.astype(np.float64)), perm)
    T = A.hard_transpose(perm)
    dim, b, e, t, o = T.metadata()
    assert np.array_equal(b.T, want.begin) and np.array_equal(e.T, want.end)
    assert np.array_equal(T.data().astype(np.float64), want.data)
    assert np.array_equal(T.hard_transpose(list(np.argsort(perm))).data(), data)


@pytest.mark.parametrize("perm", [[1, 0, 2], [0, 2, 1], [2, 1, 0]])
def test_hard_transpose_row_major_input(tq, perm):
    """Blocks stored row-major (index tables (d1 d2, d2, 1)): the transpose
    takes the general-stride path and is bit-exact with the oracle."""
    from torque_gb300.sectors import Leg, charge_blocks
    legs = [Leg([0, 1], [9, 40], 1), Leg([0, 1], [33, 5], -1), Leg([0, 1], [3, 17], 1)]
    bl = charge_blocks(legs, 0, modulus=2)
    d = bl.block_dims
    tables = np.stack([d[:, 1] * d[:, 2], d[:, 2], np.ones(len(d), np.int64)], axis=1)
    data = np.random.default_rng(13).standard_normal(bl.n_elem)
    A = to_gpu(tq, bl.dimension, bl.begin, bl.end, data, tables=tables)
    hA = host(bl.dimension, bl.begin, bl.end, data, tables=tables)
    T = A.hard_transpose(perm)
    want = orc.hard_transpose(hA, perm)
    assert np.array_equal(T.data(), want.data)


def test_partial_overlaps_and_custom_strides(tq):
    rng = np.random.default_rng(5)
    dimA = [6, 7, 5]
    bA, eA = [[0, 0, 0], [2, 3, 1], [1, 0, 2]], [[3, 4, 2], [5, 6, 4], [4, 2, 4]]
    nA = 4 * 5 * 3 + 4 * 4 * 4 + 4 * 3 * 3
    dA = rng.standard_normal(nA)
    dimB = [7, 4]
    bB, eB = [[1, 0], [4, 1], [0, 2]], [[5, 2], [6, 3], [2, 3]]
    # B's blocks stored row-major: index tables (d1, 1) instead of (1, d0)
    tB = [[3, 1], [3, 1], [2, 1]]
    dB = rng.standard_normal(5 * 3 + 3 * 3 + 3 * 2)
    A = to_gpu(tq, dimA, bA, eA, dA)
    B = to_gpu(tq, dimB, bB, eB, dB, tB)
    hA = host(dimA, bA, eA, dA)
    hB = host(dimB, bB, eB, dB, tB)
    check_reference_layout(tq, A, B, hA, hB, np.array([[1, 0]]))
    # a second operand over A's legs 0 and 2, stored with permuted strides
    dimD = [6, 5]
    bD, eD = [[0, 0], [3, 2], [2, 1]], [[4, 3], [5, 4], [3, 4]]
    tD = [[4, 1], [3, 1], [4, 1]]
    dD = rng.standard_normal(5 * 4 + 3 * 3 + 2 * 4)
    D = to_gpu(tq, dimD, bD, eD, dD, tD)
    hD = host(dimD, bD, eD, dD, tD)
    for pairs in ([[0, 0]], [[2, 1]], [[0, 0], [2, 1]], [[2, 1], [0, 0]]):
        check_reference_layout(tq, A, D, hA, hD, np.array(pairs))
    # full contraction to a scalar over two legs: A[0:2, 1:3, 2] x B as a 2-leg tensor
    s = A.contract(A, [[0, 0], [1, 1], [2, 2]]).to_number()
    assert abs(s - orc.contract(hA, hA, [[0, 0], [1, 1], [2, 2]])) <= 1e-12 * abs(s)


def test_empty_and_unmatched(tq):
    A = tq.BlockSparseTensor([4, 4])
    B = tq.BlockSparseTensor([4, 4])
    C = A.contract(B, [[1, 0]])
    assert C.n_blocks == 0 and C.query([1, 1]) == 0
    A.append_block(np.ones(4), [0, 0], [1, 1])
    B.append_block(np.ones(4), [2, 2], [3, 3])
    C = A.contract(B, [[1, 0]])
    assert C.n_blocks == 0
    assert A.contract(B, [[1, 0], [0, 1]]).to_number() == 0
    assert A.contract(B, [[1, 0]], layout="reduced").n_blocks == 0


def test_allocation_failure_is_reported(tq, small):
    c = small
    A = to_gpu(tq, c.A.dimension, c.A.begin, c.A.end, c.a_data)
    B = to_gpu(tq, c.B.dimension, c.B.begin, c.B.end, c.b_data)
    lib = tq.load()
    for after in (0, 1, 3, 6):
        lib.tq_debug_fail_alloc_after(after)
        try:
            with pytest.raises(tq.TorqueError) as ei:
                A.contract(B, c.pairs)
            assert ei.value.status == 3
        finally:
            lib.tq_debug_fail_alloc_after(-1)
    C = A.contract(B, c.pairs)  # the library still works afterwards
    assert C.n_blocks == 325


@pytest.mark.parametrize("layout", ["reference", "reduced"])
@pytest.mark.parametrize("dtype,tol", [(np.float64, TOL64), (np.float32, TOL32),
                                       (np.float16, TOL16)])
def test_split_k_few_tiles_long_k(tq, layout, dtype, tol):
    """Few output tiles with a long fused K: the native kernel cuts each tile
    into K chunks (boundaries inside pairs) and sums the partials in chunk
    order.  A[a,c,d] x B[c,d,e], a and e small, c and d long U(1) legs."""
    from torque_gb300.sectors import Leg, charge_blocks
    fa = Leg([0, 1], [5, 6], +1)
    cl = Leg([-2, -1, 0, 1, 2], [30, 50, 90, 50, 30], -1)
    fe = Leg([0, 1], [4, 7], -1)
    A = charge_blocks([fa, cl, cl.flipped()])
    B = charge_blocks([cl.flipped(), cl, fe])
    rng = np.random.default_rng(17)
    # the oracle sees the inputs rounded to the tensor's type
    a = rng.standard_normal(A.n_elem).astype(dtype).astype(np.float64)
    b = rng.standard_normal(B.n_elem).astype(dtype).astype(np.float64)
    pairs = np.array([[1, 0], [2, 1]])
    gA = to_gpu(tq, A.dimension, A.begin, A.end, a, dtype=dtype)
    gB = to_gpu(tq, B.dimension, B.begin, B.end, b, dtype=dtype)
    hA = host(A.dimension, A.begin, A.end, a)
    hB = host(B.dimension, B.begin, B.end, b)
    if layout == "reference":
        check_reference_layout(tq, gA, gB, hA, hB, pairs, dtype, tol)
    else:
        C = gA.contract(gB, pairs, layout="reduced")
        dim, bb, ee, tt, oo = C.metadata()
        got = orc.densify(orc.HostBS(dim, bb.T, ee.T, C.data().astype(np.float64), tt.T))
        want = orc.dense_contract(orc.densify(hA), orc.densify(hB), pairs)
        assert np.max(np.abs(got - want)) <= tol * np.max(np.abs(want))
        # deterministic: the chunk partials are summed in a fixed order
        assert np.array_equal(C.data(), gA.contract(gB, pairs, layout="reduced").data())
