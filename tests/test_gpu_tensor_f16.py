"""Half tensors on the tensor cores (precision "tensor": tcgen05 kind::f16 with
fp16 A and B, fp32 accumulation in tensor memory, the retired accumulators
summed in fp32, one rounding of each result element to binary16).

Against the oracle on the same half-rounded inputs: within 1e-3 of max|C|
(the result's own rounding is 2^-11) and, element by element, within one
half ulp plus 1e-5 of max|C| (the fp32 accumulation); exact for
small-integer data, whose sums the fp32 accumulators hold exactly; close to
the plain half path (FP32 SIMT accumulation) element by element."""
import numpy as np
import pytest
import torch

from oracle import oracle as orc
from torque_gb300 import workloads

pytestmark = pytest.mark.gpu

TOL16 = 1e-3


def to_gpu(tq, bl, data):
    return tq.BlockSparseTensor(bl.dimension, np.asarray(data, np.float16), bl.begin.T, bl.end.T,
                                dtype=np.float16)


def host(bl, data):
    return orc.HostBS(np.asarray(bl.dimension), bl.begin, bl.end,
                      np.asarray(data, np.float16).astype(np.float64))


def dense_of(C):
    dim, b, e, t, o = C.metadata()
    return orc.densify(orc.HostBS(dim, b.T, e.T, C.data().astype(np.float64), t.T))


@pytest.mark.parametrize("layout", ["reference", "reduced"])
def test_small_u1_tensor_form(tq, layout):
    c = workloads.small_u1()
    A, B = to_gpu(tq, c.A, c.a_data), to_gpu(tq, c.B, c.b_data)
    C = A.contract(B, c.pairs, precision="tensor", layout=layout)
    assert C.dtype == np.float16
    want = orc.dense_contract(orc.densify(host(c.A, c.a_data)), orc.densify(host(c.B, c.b_data)),
                              c.pairs)
    got = dense_of(C)
    assert np.max(np.abs(got - want)) <= TOL16 * np.max(np.abs(want))
    # element by element, each stored element one rounding to half of a sum
    # whose fp32 accumulation error stays far below a half ulp (in the
    # reference layout every pair's block is rounded on its own)
    if layout == "reference":
        _, _, _, w = orc.contract(host(c.A, c.a_data), host(c.B, c.b_data), c.pairs, mode=0)
        g = C.data().astype(np.float64)
    else:
        w, g = want, got
    ulp = np.spacing(np.abs(w).astype(np.float16)).astype(np.float64)
    assert np.all(np.abs(g - w) <= ulp + 1e-5 * np.max(np.abs(w)))


@pytest.mark.parametrize("layout", ["reference", "reduced"])
def test_integer_data_exact(tq, layout):
    c = workloads.small_u1()
    rng = np.random.default_rng(40)
    a = rng.integers(-1, 2, c.A.n_elem).astype(np.float64)
    b = rng.integers(-1, 2, c.B.n_elem).astype(np.float64)
    C = to_gpu(tq, c.A, a).contract(to_gpu(tq, c.B, b), c.pairs, precision="tensor",
                                    layout=layout)
    want = orc.dense_contract(orc.densify(host(c.A, a)), orc.densify(host(c.B, b)), c.pairs)
    assert np.max(np.abs(want)) < 2048
    assert np.array_equal(dense_of(C), want)


def test_long_fused_k(tq):
    """Fused K far above one accumulator's 336 columns (many retirements)."""
    from torque_gb300.sectors import Leg, charge_blocks
    fa = Leg([0, 1], [5, 6], +1)
    cl = Leg([-2, -1, 0, 1, 2], [30, 50, 90, 50, 30], -1)
    fe = Leg([0, 1], [4, 7], -1)
    Abl = charge_blocks([fa, cl, cl.flipped()])
    Bbl = charge_blocks([cl.flipped(), cl, fe])
    rng = np.random.default_rng(17)
    a, b = rng.standard_normal(Abl.n_elem), rng.standard_normal(Bbl.n_elem)
    pairs = np.array([[1, 0], [2, 1]])
    C = to_gpu(tq, Abl, a).contract(to_gpu(tq, Bbl, b), pairs, precision="tensor",
                                    layout="reduced")
    want = orc.dense_contract(orc.densify(host(Abl, a)), orc.densify(host(Bbl, b)), pairs)
    got = dense_of(C)
    assert np.max(np.abs(got - want)) <= TOL16 * np.max(np.abs(want))


def test_uneven_case_plan_reuse_and_execute_to(tq):
    c = workloads.uneven_u1(peak=12.0, qmax=4)
    A, B = to_gpu(tq, c.A, c.a_data), to_gpu(tq, c.B, c.b_data)
    P = tq.ContractionPlan(A, B, c.pairs, precision="tensor", layout="reduced")
    P.execute()
    P.check()
    first = P.result.data().copy()
    # against the plain half path (FP32 accumulation), element by element
    N = A.contract(B, c.pairs, layout="reduced").data().astype(np.float64)
    d = np.abs(first.astype(np.float64) - N)
    ulp = np.spacing(np.abs(N).astype(np.float16)).astype(np.float64)
    assert np.all(d <= 2 * ulp + 1e-5 * np.max(np.abs(N)))
    # deterministic, and the same bits into a pinned host buffer
    P.execute()
    assert np.array_equal(P.result.data(), first)
    host_out = torch.zeros(first.size, dtype=torch.float16, pin_memory=True)
    P.execute_to(host_out)
    assert np.array_equal(host_out.numpy(), first)


def test_precision_and_dtype_must_agree(tq):
    c = workloads.small_u1()
    A64 = tq.BlockSparseTensor(c.A.dimension, c.a_data, c.A.begin.T, c.A.end.T)
    with pytest.raises(tq.TorqueError) as ei:
        A64.contract(A64, [[0, 0]], precision="tensor")
    assert ei.value.status == 5
    A16 = to_gpu(tq, c.A, c.a_data)
    with pytest.raises(tq.TorqueError) as ei:
        A16.contract(A16, [[0, 0]], precision="ozaki")
    assert ei.value.status == 5
    with pytest.raises(tq.TorqueError):
        A16.contract(A16, [[0, 0]], precision="tensor", slices=3)
