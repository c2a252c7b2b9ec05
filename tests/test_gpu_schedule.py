"""Schedules of the tensor-core forms: tile widths, block grouping (poorly
filled output blocks sent to plain FP64), rescheduling a plan and the
exhaustive autotuner.  Block metadata stay bit-exact with the native form;
values are held to the FP64-level bound (max|C - C_oracle| / max|C_oracle|
<= 1e-10 for 5 slices) against the oracle."""
import numpy as np
import pytest

from oracle import oracle as orc
from torque_gb300 import workloads

pytestmark = pytest.mark.gpu


def operands(tq, c):
    A = tq.BlockSparseTensor(c.A.dimension, c.a_data, c.A.begin.T, c.A.end.T)
    B = tq.BlockSparseTensor(c.B.dimension, c.b_data, c.B.begin.T, c.B.end.T)
    hA = orc.HostBS(c.A.dimension, c.A.begin, c.A.end, c.a_data)
    hB = orc.HostBS(c.B.dimension, c.B.begin, c.B.end, c.b_data)
    return A, B, hA, hB


def rel_err(got, want):
    return float(np.max(np.abs(got - want)) / max(np.max(np.abs(want)), 1e-300))


@pytest.mark.parametrize("tile_n", [32, 64, 96])
@pytest.mark.parametrize("native_fill", [0, 300, 1000])
def test_tile_width_and_grouping_reference_layout(tq, tile_n, native_fill):
    c = workloads.small_u1()
    A, B, hA, hB = operands(tq, c)
    C = A.contract(B, c.pairs, precision="ozaki", tile_n=tile_n, native_fill=native_fill)
    ob, oe, off, want = orc.contract(hA, hB, c.pairs, mode=0)
    dim, b, e, t, o = C.metadata()
    assert np.array_equal(b.T, ob) and np.array_equal(e.T, oe) and np.array_equal(o, off)
    err = rel_err(C.data(), want)
    print("tile %d grouping %d: rel err %.3e" % (tile_n, native_fill, err))
    assert err <= 1e-10


@pytest.mark.parametrize("tile_n,native_fill", [(32, 0), (64, 150), (96, 500)])
def test_tile_width_and_grouping_long_k(tq, tile_n, native_fill):
    """Reduced layout with long fused K (sectors up to 24: several accumulator
    retirements per tile) against the native form."""
    u = workloads.uneven_u1(peak=24.0, seed=7)
    A, B, _, _ = operands(tq, u)
    N = A.contract(B, u.pairs, layout="reduced")
    C = A.contract(B, u.pairs, precision="ozaki", layout="reduced", tile_n=tile_n,
                   native_fill=native_fill)
    assert np.array_equal(C.block_offsets, N.block_offsets)
    assert np.array_equal(C.begin_points, N.begin_points)
    err = rel_err(C.data(), N.data())
    print("long K tile %d grouping %d: rel err %.3e" % (tile_n, native_fill, err))
    assert err <= 1e-10


def test_reschedule_keeps_symbolic_stage(tq):
    c = workloads.small_u1()
    A, B, hA, hB = operands(tq, c)
    P = tq.ContractionPlan(A, B, c.pairs, precision="ozaki", layout="reduced")
    r_oz = P.execute().data().copy()
    P.reschedule("native")
    r_nat = P.execute().data().copy()
    N = A.contract(B, c.pairs, layout="reduced")
    assert np.array_equal(r_nat, N.data())  # the native kernel, bit for bit
    P.reschedule("bf16x3", tile_n=32, native_fill=100)
    r_b3 = P.execute().data().copy()
    P.check()
    assert rel_err(r_oz, r_nat) <= 1e-10
    assert rel_err(r_b3, r_nat) <= 1e-6
    # a plain reference-layout plan has no free-box keys: no tensor-core schedule
    Q = tq.ContractionPlan(A, B, c.pairs)
    with pytest.raises(tq.TorqueError) as ei:
        Q.reschedule("ozaki")
    assert ei.value.status == 1


def test_autotune_small(tq):
    c = workloads.small_u1()
    A, B, _, _ = operands(tq, c)
    P = tq.ContractionPlan(A, B, c.pairs, precision="ozaki", layout="reduced")
    cands = [dict(precision="native"), dict(precision="ozaki", slices=5),
             dict(precision="ozaki", slices=4, tile_n=32),
             dict(precision="bf16x3", native_fill=250),
             dict(precision="ozaki", slices=9)]  # invalid: reported, not fatal
    best, entries = P.autotune(1e-10, cands, reps=2)
    st = [e[0] for e in entries]
    assert st[:4] == [0, 0, 0, 0] and st[4] == 1
    assert entries[0][2] == 0.0  # native against itself
    assert entries[1][2] <= 1e-10 and entries[3][2] <= 1e-6
    assert best in (0, 1, 2)
    assert entries[best][2] <= 1e-10
    ok = [i for i in range(4) if entries[i][2] <= 1e-10]
    assert entries[best][1] == min(entries[i][1] for i in ok)
    # the plan keeps the winner's schedule
    N = A.contract(B, c.pairs, layout="reduced")
    assert rel_err(P.execute().data(), N.data()) <= 1e-10


def test_batch_mixed_tile_widths(tq):
    """A batch whose plans use different tile widths and grouping: one launch
    per width, grouped blocks after it; results equal the plans run alone."""
    sweep = workloads.peps_sweep(n=6, seed=11)
    plans, refs, keep = [], [], []
    for k, su in enumerate(sweep):
        T = tq.BlockSparseTensor(su.T.dimension, su.t_data, su.T.begin.T, su.T.end.T)
        E1 = tq.BlockSparseTensor(su.E1.dimension, su.e1_data, su.E1.begin.T, su.E1.end.T)
        tile = (32, 64, 96)[k % 3]
        P = tq.ContractionPlan(E1, T, su.pairs1, precision="ozaki", layout="reduced",
                               tile_n=tile, native_fill=200 * (k % 2))
        N = E1.contract(T, su.pairs1, layout="reduced")
        plans.append(P)
        refs.append(N.data())
        keep += [T, E1, N]
    b = tq.Batch(plans)
    b.execute()
    b.check()
    for P, r in zip(plans, refs):
        assert rel_err(P.result.data(), r) <= 1e-10
