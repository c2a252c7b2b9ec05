"""Device index primitives against the oracle, bit-exact: nest_sum (block
offsets), and the matching + grouping of the reduced layout on structures whose
block counts make the scans and the radix sort run several tiles."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as orc
from torque_gb300 import sectors, workloads

pytestmark = pytest.mark.gpu


def oracle_nest_sum(x):
    out = np.zeros_like(x)
    t = 0
    for i, v in enumerate(x):
        out[i] = t
        t += int(v)
    return out, t


@pytest.mark.parametrize("n", [0, 1, 7, 2048, 2049, 100_000, 5_000_003])
def test_nest_sum(tq, n):
    import torch
    rng = np.random.default_rng(n)
    x = rng.integers(0, 5000, size=n).astype(np.int64)
    d_in = torch.from_numpy(x).cuda()
    d_out = torch.zeros(max(n, 1), dtype=torch.int64, device="cuda")
    d_tot = torch.zeros(1, dtype=torch.int64, device="cuda")
    lib = tq.load()
    st = lib.tq_nest_sum(ctypes.c_void_p(d_in.data_ptr()), n, ctypes.c_void_p(d_out.data_ptr()),
                         ctypes.c_void_p(d_tot.data_ptr()), None)
    assert st == 0
    torch.cuda.synchronize()
    want, total = oracle_nest_sum(x) if n < 200_000 else (
        np.concatenate([[0], np.cumsum(x)[:-1]]), int(x.sum()))
    assert np.array_equal(d_out.cpu().numpy()[:n], want)
    assert int(d_tot.item()) == total


def test_many_blocks_pair_list_and_grouping(tq):
    """Rank-4 U(1) tensors with 11 sectors per leg (891 blocks, 7,381 pairs): the pair list
    and output boxes of the reference layout match the oracle exactly, and the
    reduced layout groups them into the distinct output boxes in column-major
    sector order."""
    q = list(range(-5, 6))
    s = [1 + (abs(x) % 3) for x in q]
    legs = [sectors.Leg(q, s, d) for d in (+1, +1, -1, -1)]
    A = sectors.charge_blocks(legs)
    B = sectors.charge_blocks(legs)
    rng = np.random.default_rng(3)
    a = rng.standard_normal(A.n_elem)
    b = rng.standard_normal(B.n_elem)
    pairs = np.array([[2, 0], [3, 1]])
    gA = tq.BlockSparseTensor(A.dimension, a, A.begin.T, A.end.T)
    gB = tq.BlockSparseTensor(B.dimension, b, B.begin.T, B.end.T)
    hA = orc.HostBS(A.dimension, A.begin, A.end, a)
    hB = orc.HostBS(B.dimension, B.begin, B.end, b)
    C = gA.contract(gB, pairs)
    ob, oe, off, want = orc.contract(hA, hB, pairs, mode=0)
    dim, cb, ce, ct, co = C.metadata()
    assert C.n_blocks == ob.shape[0] == 7381
    assert np.array_equal(cb.T, ob) and np.array_equal(ce.T, oe) and np.array_equal(co, off)
    assert np.max(np.abs(C.data() - want)) <= 1e-12 * np.max(np.abs(want))
    R = gA.contract(gB, pairs, layout="reduced")
    boxes = np.unique(np.concatenate([ob, oe], 1), axis=0)
    order = np.lexsort(boxes[:, :4].T)
    _, rb, re_, rt, ro = R.metadata()
    assert np.array_equal(rb.T, boxes[order, :4]) and np.array_equal(re_.T, boxes[order, 4:])
