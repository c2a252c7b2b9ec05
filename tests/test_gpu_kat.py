"""The reference's known-answer tests (test/gpu/block_sparse_test.cu) run through
the Python mirror of torque::gpu::BlockSparseTensor, in float32 (as the
reference), float64 and half (binary16, the reference's third instantiation;
the known answers are small integers, exact in every type)."""
import numpy as np
import pytest

from conftest import kat_spec, spec_arrays
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def make(tq, spec, dtype):
    dim, b, e, t, d = spec_arrays(spec)
    T = tq.BlockSparseTensor(dim, dtype=dtype)
    if b.shape[0]:
        T.append_blocks(d.astype(dtype), b.T, e.T, None if t is None else t.T)
    return T


@pytest.mark.parametrize("dtype", [np.float16, np.float32, np.float64])
def test_kat_ops(tq, kat, dtype):
    for case in kat["cases"]:
        dim, b, e, t, d = spec_arrays(case)
        if b.shape[0]:
            T = tq.BlockSparseTensor(dim, d.astype(dtype), b.T, e.T, None if t is None else t.T,
                                     dtype=dtype)
        else:
            T = tq.BlockSparseTensor(dim, dtype=dtype)
        for op in case["ops"]:
            if op[0] == "query":
                assert T.query(op[1]) == op[2], (case["name"], op)
            elif op[0] == "modify":
                T.modify(op[1], op[2])
            elif op[0] == "append":
                T.append_block(np.asarray(op[4], dtype), op[1], op[2], op[3])
            elif op[0] == "transpose":
                T = T.hard_transpose(op[1])


@pytest.mark.parametrize("dtype", [np.float16, np.float32, np.float64])
@pytest.mark.parametrize("layout", ["reference", "reduced"])
def test_kat_contractions(tq, kat, dtype, layout):
    for case in kat["contractions"]:
        A = make(tq, kat_spec(kat, case["A"]), dtype)
        if case["B"] == "A":
            B = A
        else:
            bspec = [c for c in kat["contractions"] if c["name"] == case["B"]][0]["B"] \
                if isinstance(case["B"], str) else case["B"]
            B = make(tq, bspec, dtype)
        C = A.contract(B, case["pairs"], layout=layout)
        if "scalar" in case:
            assert C.rank == 0
            assert C.to_number() == case["scalar"], case["name"]
            continue
        for idx, val in case.get("queries", []):
            assert C.query(idx) == val, (case["name"], idx)
        if "dense_column_major" in case:
            dim = C.dimension
            got = [C.query([i, j]) for j in range(dim[1]) for i in range(dim[0])]
            assert got == case["dense_column_major"], case["name"]


def test_errors(tq):
    A = tq.BlockSparseTensor([4, 3])
    B = tq.BlockSparseTensor([5, 3])
    with pytest.raises(tq.TorqueError, match="do not match"):
        A.contract(B, [[0, 0]])
    with pytest.raises(tq.TorqueError, match="out of boundary"):
        A.query([4, 0])
    with pytest.raises(tq.TorqueError, match="Rank does not match"):
        A.query([1])
    with pytest.raises(tq.TorqueError, match="permutation"):
        A.hard_transpose([0, 0])


@pytest.mark.parametrize("divisor", [[1, 1, 1, 1], [1, 3, 1, 1], [2, 1, 4, 1], [3, 3, 2, 2]])
def test_slice_boxes_and_data(tq, divisor):
    """slice (block_sparse.cuh:1124-1176) against the oracle's restatement: the
    sub-box list bit-exact, offsets the exclusive scan of the sub-box sizes, and
    the data buffer copied unchanged (the reference reinterprets it through the
    sub-boxes' own column-major strides rather than moving it)."""
    # blocks whose dimensions every divisor above divides
    dims = np.array([12, 12, 8, 8])
    begin = np.array([[0, 0, 0, 0], [6, 0, 4, 0], [0, 6, 0, 4]])
    end = np.array([[5, 5, 3, 3], [11, 5, 7, 3], [5, 11, 3, 7]])
    rng = np.random.default_rng(9)
    n = int(np.prod(end - begin + 1, axis=1).sum())
    data = rng.standard_normal(n)
    T = tq.BlockSparseTensor(dims, data, begin.T, end.T)
    S = T.slice(divisor)
    want_b, want_e = orc.slice_boxes(begin, end, divisor)
    dim, b, e, t, o = S.metadata()
    assert np.array_equal(b.T, want_b) and np.array_equal(e.T, want_e)
    sizes = np.prod(want_e - want_b + 1, axis=1)
    assert np.array_equal(o, np.concatenate([[0], np.cumsum(sizes)[:-1]]))
    assert np.array_equal(S.data(), data)


def test_slice_rejects_residues(tq):
    T = tq.BlockSparseTensor([6, 6], np.ones(36), [[0], [0]], [[5], [5]])
    with pytest.raises(tq.TorqueError) as ei:
        T.slice([4, 1])
    assert "residues" in str(ei.value)
    with pytest.raises(ValueError):
        orc.slice_boxes([[0, 0]], [[5, 5]], [4, 1])
