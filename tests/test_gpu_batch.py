"""Batches: PEPS-sweep site updates (E1 x T, then X x E2) planned separately and
run as one numeric stage — one persistent tensor-core launch per wave, and as a
replayed CUDA graph.  The batched results equal the plans run one by one
exactly (same tiles, same arithmetic); the FP64-level form stays within 1e-10
of the plain FP64 results."""
import numpy as np
import pytest

from oracle import oracle as orc
from torque_gb300 import workloads

pytestmark = pytest.mark.gpu


def gpu(tq, bl, data):
    return tq.BlockSparseTensor(bl.dimension, data, bl.begin.T, bl.end.T)


def make_plans(tq, instances, precision, slices=0):
    keep, p1, p2 = [], [], []
    for s in instances:
        T, E1, E2 = gpu(tq, s.T, s.t_data), gpu(tq, s.E1, s.e1_data), gpu(tq, s.E2, s.e2_data)
        P1 = tq.ContractionPlan(E1, T, s.pairs1, precision=precision, slices=slices,
                                layout="reduced")
        P2 = tq.ContractionPlan(P1.result, E2, s.pairs2, precision=precision, slices=slices,
                                layout="reduced")
        keep.append((T, E1, E2))
        p1.append(P1)
        p2.append(P2)
    return keep, p1, p2


def results(plans):
    return [p.result.data().copy() for p in plans]


@pytest.mark.parametrize("precision,slices,tol", [("ozaki", 5, 1e-10), ("bf16x3", 3, 1e-5)])
def test_batch_matches_sequential_and_fp64(tq, precision, slices, tol):
    inst = workloads.peps_sweep(24, seed=31)
    keep, p1, p2 = make_plans(tq, inst, precision, slices)
    # one by one
    for a, b in zip(p1, p2):
        a.execute()
        b.execute()
        a.check()
        b.check()
    one_by_one = results(p2)
    # zero the results, then one batch (two waves)
    for p in p1 + p2:
        p.result.data()  # materialise metadata before the batch
    batch = tq.Batch(p1 + p2, waves=[0] * len(p1) + [1] * len(p2))
    batch.execute()
    batch.check()
    batched = results(p2)
    for x, y in zip(one_by_one, batched):
        assert np.array_equal(x, y)
    # replayed graph, twice
    batch.graph_launch()
    batch.graph_launch()
    batch.check()
    for x, y in zip(one_by_one, results(p2)):
        assert np.array_equal(x, y)
    assert batch.kernels >= 4  # two waves: prepare + GEMM each
    # accuracy against plain FP64 and the oracle on one instance
    keep64, q1, q2 = make_plans(tq, inst, "native")
    for a, b in zip(q1, q2):
        a.execute()
        b.execute()
    for x, y in zip(batched, results(q2)):
        assert np.max(np.abs(x - y)) <= tol * np.max(np.abs(y))
    s = inst[0]
    hE1 = orc.HostBS(s.E1.dimension, s.E1.begin, s.E1.end, s.e1_data)
    hT = orc.HostBS(s.T.dimension, s.T.begin, s.T.end, s.t_data)
    hE2 = orc.HostBS(s.E2.dimension, s.E2.begin, s.E2.end, s.e2_data)
    X = orc.dense_contract(orc.densify(hE1), orc.densify(hT), s.pairs1)
    Y = orc.dense_contract(X, orc.densify(hE2), s.pairs2)
    R = q2[0].result
    dim, b, e, t, o = R.metadata()
    got = orc.densify(orc.HostBS(dim, b.T, e.T, R.data(), t.T))
    assert np.max(np.abs(got - Y)) <= 1e-12 * np.max(np.abs(Y))


def test_rescheduled_plan_invalidates_batch(tq):
    """A batch's device tables point into its plans' schedule arrays; once a
    plan is rescheduled the batch refuses to run (plain execute and graph
    replay) instead of reading freed memory, and a batch built again runs."""
    inst = workloads.peps_sweep(4, seed=32)
    keep, p1, p2 = make_plans(tq, inst, "ozaki", 5)
    batch = tq.Batch(p1 + p2, waves=[0] * len(p1) + [1] * len(p2))
    batch.graph_launch()
    batch.check()
    want = results(p2)
    p1[1].reschedule("ozaki", slices=5, tile_n=64)
    for call in (batch.execute, batch.graph_launch):
        with pytest.raises(tq.TorqueError) as ei:
            call()
        assert ei.value.status == 1 and "rescheduled" in str(ei.value)
    again = tq.Batch(p1 + p2, waves=[0] * len(p1) + [1] * len(p2))
    again.graph_launch()
    again.check()
    for x, y in zip(want, results(p2)):
        assert np.max(np.abs(x - y)) <= 1e-10 * np.max(np.abs(y))


@pytest.mark.parametrize("precision,slices,tol", [("ozaki", 5, 1e-10), ("bf16x3", 3, 1e-5)])
def test_full_sweep_256_instances_against_fp64(tq, precision, slices, tol):
    """The whole batched PEPS sweep of the benchmark (256 site updates, seed 3)
    as one replayed graph, every instance's result against the plain FP64 form
    of the same contractions (elementwise, scaled by the instance's max |C|)."""
    inst = workloads.peps_sweep(256, seed=3)
    keep, p1, p2 = make_plans(tq, inst, precision, slices)
    batch = tq.Batch(p1 + p2, waves=[0] * len(p1) + [1] * len(p2))
    batch.graph_launch()
    batch.check()
    got = results(p2)
    del batch, p1, p2, keep
    keep64, q1, q2 = make_plans(tq, inst, "native")
    worst = 0.0
    for q, (a, b) in enumerate(zip(q1, q2)):
        a.execute()
        b.execute()
        y = b.result.data()
        worst = max(worst, float(np.max(np.abs(got[q] - y)) / np.max(np.abs(y))))
    print("256-instance sweep, %s: max rel err vs FP64 %.3e" % (precision, worst))
    assert worst <= tol
