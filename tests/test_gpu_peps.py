"""The PEPS norm (4x4 open boundary, Z2, d=2, D=6, seed 1): double layers by
block-sparse contraction + leg fusion, network contracted exactly, against
the dense FP64 oracle.  Relative error of <psi|psi>:
    plain FP64 <= 1e-12,  Ozaki 5 slices <= 1e-10,  3 x bf16 <= 1e-4."""
import numpy as np
import pytest

from oracle import peps_oracle as po

pytestmark = pytest.mark.gpu


def dense_norm(L, D, d, seed):
    from torque_gb300 import peps
    ts, labels = {}, {}
    for s in peps.sites(L, D, d, seed):
        T = po.dense_site(s.blocks.dimension, s.blocks.begin, s.blocks.end, s.data)
        ts[(s.r, s.c)] = po.double_layer(T)
        labels[(s.r, s.c)] = peps._squeeze_labels(s.r, s.c, L)
    order = [(r, c) for c in range(L) for r in range(L)]
    return po.norm(ts, labels, order)


@pytest.fixture(scope="module")
def want4():
    return dense_norm(4, 6, 2, 1)


@pytest.mark.parametrize("precision,slices,tol", [("native", 0, 1e-12), ("ozaki", 5, 1e-10),
                                                  ("ozaki", 7, 1e-11), ("bf16x3", 3, 1e-4)])
def test_peps_norm_4x4(tq, want4, precision, slices, tol):
    from torque_gb300 import peps
    net = peps.network(tq, 4, 6, 2, 1, precision=precision, slices=slices)
    got, flops, secs = peps.contract_norm(tq, net, 4, precision=precision, slices=slices)
    err = abs(got - want4) / abs(want4)
    print("PEPS 4x4 %s s=%d: <psi|psi> = %.15e, oracle %.15e, rel err %.2e, %.3e flop"
          % (precision, slices, got, want4, err, flops))
    assert err <= tol


def test_fuse_legs_matches_dense_reshape(tq):
    """Fusion is a relabelling: densify(fused)[x_a-major pair range] equals the
    dense tensor with the two legs merged pair by pair."""
    from oracle import oracle as orc
    from torque_gb300.sectors import Leg, charge_blocks, fuse_sector_order
    la = Leg([-1, 0, 1], [2, 3, 2], +1)
    lb = Leg([0, 1], [2, 3], +1)
    lc = Leg([-1, 0, 1, 2], [1, 2, 2, 1], -1)
    bl = charge_blocks([la, lb, lc])
    rng = np.random.default_rng(5)
    data = rng.standard_normal(bl.n_elem)
    b, e = bl.points()
    T = tq.BlockSparseTensor(bl.dimension, data, b, e)
    F, fused = T.fuse_sectors(0, la, lb)
    dense = orc.densify(orc.HostBS(bl.dimension, bl.begin, bl.end, data))
    dim, fb, fe, ft, fo = F.metadata()
    got = orc.densify(orc.HostBS(dim, fb.T, fe.T, F.data(), ft.T))
    _, off = fuse_sector_order(la, lb)
    want = np.zeros((la.dim * lb.dim, lc.dim))
    for ia in range(len(la.sizes)):
        for ib in range(len(lb.sizes)):
            blk = dense[la.offsets[ia]:la.offsets[ia] + la.sizes[ia],
                        lb.offsets[ib]:lb.offsets[ib] + lb.sizes[ib], :]
            n = la.sizes[ia] * lb.sizes[ib]
            want[off[ia, ib]:off[ia, ib] + n, :] = blk.reshape(n, -1, order="F")
    assert np.array_equal(got, want)
    assert np.array_equal(F.data(), T.data())  # data untouched
    # a block that does not cover whole sectors cannot be fused
    P = tq.BlockSparseTensor([7, 5], np.ones(4), [[0], [0]], [[1], [1]])
    with pytest.raises(tq.TorqueError) as ei:
        P.fuse_legs(0, [0, 3, 7], [0, 2, 5], [[0, 6], [15, 23]])
    assert ei.value.status == 5
    with pytest.raises(tq.TorqueError) as ei:
        P.fuse_legs(0, [0, 3, 7], [0, 2, 5], [[0, 6], [15, 20]])  # ranges overlap
    assert ei.value.status == 1
