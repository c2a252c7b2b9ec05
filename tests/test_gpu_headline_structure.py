"""Index parity on the full uneven U(1) pair (33 sectors of up to 48 per leg,
23,969 blocks per tensor, 593,505 matched pairs, sizes of the headline
benchmark): the device symbolic stage's pair list, output boxes and offsets
against the oracle's restatement of block_in_range and of the group assembly of
contract (src/tensor/block_sparse.cpp:42-148, src/gpu/block_sparse.cuh:620-674),
bit-exact.  The reference layout's data would hold 1.4e11 elements, so the
block list is read from the symbolic stage alone (tq_contract_blocks) and the
values are checked elsewhere."""
import numpy as np
import pytest

from oracle import oracle as orc
from torque_gb300 import workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def headline(tq):
    u = workloads.uneven_u1(data=False)
    A = tq.BlockSparseTensor.zeros(u.A.dimension, u.A.begin.T, u.A.end.T)
    B = tq.BlockSparseTensor.zeros(u.B.dimension, u.B.begin.T, u.B.end.T)
    hA = orc.HostBS(u.A.dimension, u.A.begin, u.A.end, np.zeros(0))
    hB = orc.HostBS(u.B.dimension, u.B.begin, u.B.end, np.zeros(0))
    want = orc.contract_blocks(hA, hB, u.pairs)
    yield u, A, B, want
    del A, B


def test_reference_layout_block_list_bit_exact(tq, headline):
    u, A, B, (pa, pb, ob, oe, off) = headline
    assert u.A.n_blocks == u.B.n_blocks == 23969
    got = tq.contract_blocks(A, B, u.pairs, layout="reference")
    assert pa.size == 593505 == got["pair_a"].size
    assert np.array_equal(got["pair_a"], pa) and np.array_equal(got["pair_b"], pb)
    assert np.array_equal(got["begin"], ob) and np.array_equal(got["end"], oe)
    assert np.array_equal(got["offsets"], off)
    sizes = np.prod(oe - ob + 1, axis=1)
    assert got["n_elem"] == int(sizes.sum())


def test_reduced_layout_boxes_are_the_distinct_pair_boxes(tq, headline):
    u, A, B, (pa, pb, ob, oe, off) = headline
    got = tq.contract_blocks(A, B, u.pairs, layout="reduced")
    boxes = np.unique(np.concatenate([ob, oe], 1), axis=0)
    # one block per distinct box, in column-major order of the box corners
    order = np.lexsort(boxes[:, :4].T)
    assert np.array_equal(got["begin"], boxes[order, :4])
    assert np.array_equal(got["end"], boxes[order, 4:])
    sizes = np.prod(boxes[order, 4:] - boxes[order, :4] + 1, axis=1)
    assert np.array_equal(got["offsets"], np.concatenate([[0], np.cumsum(sizes)[:-1]]))
    assert got["n_elem"] == int(sizes.sum())
