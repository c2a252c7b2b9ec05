"""tq_plan_execute_to: the numeric stage writing its result straight into a
caller's buffer — page-locked host memory (written by the kernels over the
host link as they run), device memory, or pageable host memory (one copy
after the GEMM).  Every destination receives exactly the bits tq_plan_execute
writes into the result tensor, for the plain, tensor-core and class-layout
paths; afterwards tq_plan_execute and batches write the result tensor again."""
import numpy as np
import pytest
import torch

from torque_gb300 import workloads

pytestmark = pytest.mark.gpu


def gpu(tq, bl, data):
    return tq.BlockSparseTensor(bl.dimension, data, bl.begin.T, bl.end.T)


def destinations(n):
    return {
        "pinned": torch.full((n,), np.nan, dtype=torch.float64, pin_memory=True),
        "device": torch.full((n,), np.nan, dtype=torch.float64, device="cuda"),
        "pageable": np.full(n, np.nan),
    }


def as_numpy(d):
    return d.cpu().numpy() if hasattr(d, "cpu") else d


@pytest.mark.parametrize("case", ["small", "uneven"])
@pytest.mark.parametrize("precision,slices,layout", [
    ("native", 0, "reference"), ("native", 0, "reduced"),
    ("ozaki", 5, "reference"), ("ozaki", 5, "reduced"), ("bf16x3", 3, "reduced")])
def test_execute_to_every_destination(tq, case, precision, slices, layout):
    if case == "uneven" and layout == "reference":
        pytest.skip("one output block per pair: too large a result for this case")
    c = workloads.small_u1() if case == "small" else workloads.uneven_u1(peak=12.0, qmax=4)
    A, B = gpu(tq, c.A, c.a_data), gpu(tq, c.B, c.b_data)
    kw = dict(precision=precision, slices=slices, layout=layout)
    Q = tq.ContractionPlan(A, B, c.pairs, **kw)
    Q.execute()
    Q.check()
    want = Q.result.data().copy()
    P = tq.ContractionPlan(A, B, c.pairs, **kw)  # never executed into its own result first
    for name, dst in destinations(want.size).items():
        P.execute_to(dst)
        P.check()
        torch.cuda.synchronize()
        assert np.array_equal(as_numpy(dst), want), name
    # a plain execute writes the result tensor again
    P.execute()
    assert np.array_equal(P.result.data(), want)


def test_execute_to_then_batch_writes_the_result_tensor(tq):
    c = workloads.uneven_u1(peak=12.0, qmax=4)
    A, B = gpu(tq, c.A, c.a_data), gpu(tq, c.B, c.b_data)
    P = tq.ContractionPlan(A, B, c.pairs, precision="ozaki", slices=5, layout="reduced")
    P.execute()
    want = P.result.data().copy()
    host = torch.zeros(want.size, dtype=torch.float64, pin_memory=True)
    P.execute_to(host)
    assert np.array_equal(host.numpy(), want)
    # a batch runs its own copy of the job: it writes the result tensor
    host.zero_()
    batch = tq.Batch([P])
    batch.execute()
    batch.check()
    assert np.array_equal(P.result.data(), want)
    assert not host.numpy().any()
    # a reschedule rebuilds the job array; both destinations stay right
    P.reschedule(precision="ozaki", slices=6)
    P.execute()
    want6 = P.result.data().copy()
    P.execute_to(host)
    assert np.array_equal(host.numpy(), want6)


def test_execute_to_scalar_and_errors(tq):
    c = workloads.small_u1()
    A = gpu(tq, c.A, c.a_data)
    P = tq.ContractionPlan(A, A, [[0, 0], [1, 1], [2, 2], [3, 3]])
    P.execute()
    want = P.result.to_number()
    out = torch.zeros(1, dtype=torch.float64, pin_memory=True)
    P.execute_to(out)
    assert out.item() == want
    with pytest.raises(ValueError):
        P.execute_to(np.zeros(0))
    with pytest.raises(ValueError):
        P.execute_to(np.zeros(4, np.float32))


def test_serving_loop_set_data_then_execute_to(tq):
    """New operand values copied into the existing tensors (set_data) and the
    same plan run again into a pinned host buffer give the contraction of the
    new values."""
    c = workloads.uneven_u1(peak=12.0, qmax=4)
    A, B = gpu(tq, c.A, c.a_data), gpu(tq, c.B, c.b_data)
    P = tq.ContractionPlan(A, B, c.pairs, precision="ozaki", slices=5, layout="reduced")
    host = torch.empty(P.result.n_elem, dtype=torch.float64, pin_memory=True)
    rng = np.random.default_rng(21)
    for _ in range(2):
        a2, b2 = rng.standard_normal(c.A.n_elem), rng.standard_normal(c.B.n_elem)
        A.set_data(a2)
        B.set_data(b2)
        P.execute_to(host)
        Q = tq.ContractionPlan(gpu(tq, c.A, a2), gpu(tq, c.B, b2), c.pairs, precision="ozaki",
                               slices=5, layout="reduced")
        Q.execute()
        assert np.array_equal(host.numpy(), Q.result.data())
    with pytest.raises(ValueError):
        A.set_data(np.zeros(3))


def test_set_data_async_on_a_copy_stream(tq):
    """Inputs copied by tq_bs_set_data_async on a side stream from page-locked
    memory, the compute stream waiting on an event: the result equals the
    contraction of the new values (and the synchronous form's)."""
    c = workloads.uneven_u1(peak=12.0, qmax=4)
    A, B = gpu(tq, c.A, c.a_data), gpu(tq, c.B, c.b_data)
    rng = np.random.default_rng(22)
    a2 = torch.from_numpy(rng.standard_normal(c.A.n_elem)).pin_memory()
    b2 = torch.from_numpy(rng.standard_normal(c.B.n_elem)).pin_memory()
    side = torch.cuda.Stream()
    done = torch.cuda.Event()
    A.set_data(a2.numpy(), stream=side, asynchronous=True)
    B.set_data(b2.numpy(), stream=side, asynchronous=True)
    done.record(side)
    torch.cuda.current_stream().wait_event(done)
    C = A.contract(B, c.pairs, precision="ozaki", slices=5, layout="reduced")
    W = gpu(tq, c.A, a2.numpy()).contract(gpu(tq, c.B, b2.numpy()), c.pairs, precision="ozaki",
                                          slices=5, layout="reduced")
    assert np.array_equal(C.data(), W.data())
