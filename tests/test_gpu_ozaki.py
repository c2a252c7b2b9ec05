"""Tensor-core forms (Ozaki integer slices, three-way bf16 split) against the
FP64 oracle.  Block metadata is bit-exact with the native path; values are
held to the stated error bound, written here as max|C - C_oracle| / max|C_oracle|:
    ozaki, 5 slices  <= 1e-10   (FP64-level target)
    ozaki, 6-7 slices <= 1e-11  (slice products with t+u >= 3 are accumulated
                                 in rounded fp32, which floors the error near 1e-12)
    bf16x3 (3 slices) <= 1e-6   (FP32-level)"""
import numpy as np
import pytest

from oracle import oracle as orc
from torque_gb300 import workloads

pytestmark = pytest.mark.gpu


def gpu_pair(tq, c, scale_a=None):
    a = c.a_data if scale_a is None else c.a_data * scale_a
    A = tq.BlockSparseTensor(c.A.dimension, a, c.A.begin.T, c.A.end.T)
    B = tq.BlockSparseTensor(c.B.dimension, c.b_data, c.B.begin.T, c.B.end.T)
    hA = orc.HostBS(c.A.dimension, c.A.begin, c.A.end, a)
    hB = orc.HostBS(c.B.dimension, c.B.begin, c.B.end, c.b_data)
    return A, B, hA, hB


def rel_err(got, want):
    return float(np.max(np.abs(got - want)) / max(np.max(np.abs(want)), 1e-300))


@pytest.mark.parametrize("precision,slices,tol", [("ozaki", 5, 1e-10), ("ozaki", 6, 1e-11),
                                                  ("ozaki", 7, 1e-11), ("bf16x3", 3, 1e-6)])
def test_small_u1_reference_layout(tq, precision, slices, tol):
    c = workloads.small_u1()
    A, B, hA, hB = gpu_pair(tq, c)
    C = A.contract(B, c.pairs, precision=precision, slices=slices)
    ob, oe, off, want = orc.contract(hA, hB, c.pairs, mode=0)
    dim, b, e, t, o = C.metadata()
    assert np.array_equal(b.T, ob) and np.array_equal(e.T, oe) and np.array_equal(o, off)
    err = rel_err(C.data(), want)
    print("%s s=%d reference layout: rel err %.3e" % (precision, slices, err))
    assert err <= tol


@pytest.mark.parametrize("precision,slices,tol", [("ozaki", 5, 1e-10), ("bf16x3", 3, 1e-6)])
def test_small_u1_reduced_layout(tq, precision, slices, tol):
    c = workloads.small_u1()
    A, B, hA, hB = gpu_pair(tq, c)
    C = A.contract(B, c.pairs, precision=precision, slices=slices, layout="reduced")
    N = A.contract(B, c.pairs, layout="reduced")
    assert np.array_equal(C.begin_points, N.begin_points)
    assert np.array_equal(C.block_offsets, N.block_offsets)
    dim, b, e, t, o = C.metadata()
    got = orc.densify(orc.HostBS(dim, b.T, e.T, C.data(), t.T))
    want = orc.dense_contract(orc.densify(hA), orc.densify(hB), c.pairs)
    err = rel_err(got, want)
    print("%s s=%d reduced layout: rel err %.3e" % (precision, slices, err))
    assert err <= tol


def scaled_bound(hA, hB, pa, pb):
    """Per output element of the 85-block U(1) pair (reference layout: one
    pair per output block, legs (2,3) of A against legs (0,1) of B, every pair
    covering its blocks' whole contracted range), the bound the sliced forms
    guarantee: rowmax_i(|A|) * sum_k |b_kj| + sum_k |a_ik| * colmax_j(|B|).
    Rows and columns are sliced relative to their own largest element, so the
    error scales with that element, not with each product; the bound is at
    least 2 (|A||B|)_ij."""
    out = []
    for i, j in zip(pa, pb):
        da = hA.end[i] - hA.begin[i] + 1
        db = hB.end[j] - hB.begin[j] + 1
        m, k, n = int(da[0] * da[1]), int(da[2] * da[3]), int(db[2] * db[3])
        a = np.abs(hA.data[hA.offsets[i]:hA.offsets[i] + m * k]).reshape(k, m).T   # m x k
        b = np.abs(hB.data[hB.offsets[j]:hB.offsets[j] + k * n]).reshape(n, k).T   # k x n
        bound = np.outer(a.max(1), b.sum(0)) + np.outer(a.sum(1), b.max(0))
        out.append(bound.reshape(-1, order="F"))
    return np.concatenate(out)


@pytest.mark.parametrize("precision,slices,tol", [("ozaki", 5, 1e-10), ("bf16x3", 3, 1e-5)])
def test_elementwise_bound(tq, precision, slices, tol):
    """The per-element error bound of the sliced forms:
    |C - C*|_ij <= tol * (rowmax_i|A| * sum_k|b_kj| + sum_k|a_ik| * colmax_j|B|);
    an element whose bound is zero must come out exactly zero.  Measured on
    this pair against the plain |A||B| per element: 1.2e-10 (five slices) and
    3.4e-6 (three slices); against the scaled bound at most half that."""
    c = workloads.small_u1()
    A, B, hA, hB = gpu_pair(tq, c)
    C = A.contract(B, c.pairs, precision=precision, slices=slices)
    ob, oe, off, want = orc.contract(hA, hB, c.pairs, mode=0)
    pa, pb = orc.match(hA, hB, c.pairs)
    bound = scaled_bound(hA, hB, pa, pb)
    assert bound.shape == want.shape
    err = np.abs(C.data() - want)
    assert np.all(err[bound == 0] == 0)
    nz = bound > 0
    worst = float(np.max(err[nz] / bound[nz]))
    print("%s s=%d: max |C - C*| / scaled bound per element %.3e" % (precision, slices, worst))
    assert worst <= tol


@pytest.mark.parametrize("scale", [1e-200, 1e150, 3.0])
def test_extreme_scales_and_zero_rows(tq, scale):
    """Per-row exponents follow the data: huge, tiny and zero rows."""
    c = workloads.small_u1()
    a = c.a_data.copy()
    a[:500] = 0.0  # whole rows of the first blocks vanish
    sa = np.where(np.arange(a.size) % 7 == 0, scale, 1.0)
    A, B, hA, hB = gpu_pair(tq, workloads.Contraction(c.name, c.A, c.B, a, c.b_data, c.pairs),
                            scale_a=sa)
    C = A.contract(B, c.pairs, precision="ozaki", slices=6)
    ob, oe, off, want = orc.contract(hA, hB, c.pairs, mode=0)
    got = C.data()
    # error relative to the per-pair |A||B| scale: each output block separately
    for q in range(len(off)):
        n = int(np.prod(oe[q] - ob[q] + 1))
        w = want[off[q]:off[q] + n]
        g = got[off[q]:off[q] + n]
        if np.max(np.abs(w)) == 0:
            assert np.all(g == 0)
        else:
            assert rel_err(g, w) <= 1e-9


def test_long_fused_k(tq):
    """Output blocks whose fused K spans many 336-column exact accumulator
    retirements (sectors up to 24 wide: k up to 576 per pair, tens of pairs per
    block),
    sampled blocks checked against the oracle."""
    u = workloads.uneven_u1(peak=24.0, seed=7)
    A, B, hA, hB = gpu_pair(tq, u)
    C = A.contract(B, u.pairs, precision="ozaki", layout="reduced")
    N = A.contract(B, u.pairs, layout="reduced")
    dim, b, e, t, o = C.metadata()
    gc, gn = C.data(), N.data()
    pa, pb = orc.match(hA, hB, u.pairs)
    rng = np.random.default_rng(0)
    # output block box -> oracle sum over its pairs, for a sample of blocks
    fa = [0, 1]
    fb = [2, 3]
    want_err = 0.0
    for q in rng.choice(C.n_blocks, 12, replace=False):
        bq, eq = b[:, q], e[:, q]
        sel = [(i, j) for i, j in zip(pa, pb)
               if np.array_equal(hA.begin[i, fa], bq[:2]) and np.array_equal(hB.begin[j, fb], bq[2:])]
        m = int(np.prod(eq[:2] - bq[:2] + 1))
        n = int(np.prod(eq[2:] - bq[2:] + 1))
        w = np.zeros((m, n))
        for i, j in sel:
            w += orc.pair_values(hA, hB, u.pairs, int(i), int(j))
        w = w.ravel(order="F")
        want_err = max(want_err, rel_err(gc[o[q]:o[q] + m * n], w))
        assert rel_err(gn[o[q]:o[q] + m * n], w) <= 1e-12
    print("long fused K: ozaki rel err %.3e" % want_err)
    assert want_err <= 1e-10


def test_plan_reuse_and_unsupported(tq):
    c = workloads.small_u1()
    A, B, hA, hB = gpu_pair(tq, c)
    P = tq.ContractionPlan(A, B, c.pairs, precision="ozaki", layout="reduced")
    r1 = P.execute().data().copy()
    r2 = P.execute().data()
    assert np.array_equal(r1, r2)  # deterministic
    # partially overlapping contracted intervals are rejected by the sliced forms
    X = tq.BlockSparseTensor([6, 6], np.ones(18), [[0, 3], [0, 0]], [[2, 5], [2, 2]])
    Y = tq.BlockSparseTensor([6, 4], np.ones(8), [[1], [0]], [[4], [1]])
    with pytest.raises(tq.TorqueError) as ei:
        X.contract(Y, [[1, 0]], precision="ozaki")
    assert ei.value.status == 5


def test_bounded_wait_gives_up_and_reports(tq):
    """The failure path of the tensor-core pipeline, without a GPU fault: with a
    1 ms wait limit and the producer held back for 50 ms before it issues
    anything, the MMA and epilogue roles give up their waits, the kernel drains
    and frees its tensor memory, and the check reports TQ_ERR_TIMEOUT (nothing
    is left in flight: the producer then sees the abort flag and issues no
    copy).  Contractions made after the reset run normally."""
    c = workloads.small_u1()
    A, B, hA, hB = gpu_pair(tq, c)
    lib = tq.load()
    lib.tq_debug_set_waits(1_000_000, 50_000_000)
    try:
        P = tq.ContractionPlan(A, B, c.pairs, precision="ozaki", slices=5, layout="reduced")
    finally:
        lib.tq_debug_set_waits(0, 0)
    P.execute()
    with pytest.raises(tq.TorqueError) as ei:
        P.check()
    assert ei.value.status == 6 and "gave up" in str(ei.value)
    del P
    # the library and the GPU carry on: a fresh plan (default limits) is exact
    C = A.contract(B, c.pairs, precision="ozaki", layout="reduced")
    N = A.contract(B, c.pairs, layout="reduced")
    assert rel_err(C.data(), N.data()) <= 1e-10
