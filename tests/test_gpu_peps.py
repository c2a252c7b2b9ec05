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


@pytest.mark.parametrize("modulus", [None, 2])
def test_split_undoes_fuse_and_charge_construction(tq, modulus):
    """A charge-conserving tensor made through the C ABI (tq_bs_create_charges)
    has the Python constructor's block list; fusing two of its legs by charge
    and splitting them again (tq_bs_split_leg) gives back the same blocks,
    strides, offsets and data, bit for bit, without leaving the device."""
    from torque_gb300.sectors import Leg, charge_blocks
    la = Leg([-1, 0, 1], [2, 3, 2], +1)
    lb = Leg([0, 1], [2, 3], +1)
    lc = Leg([-1, 0, 1, 2], [1, 2, 2, 1], -1)
    ld = Leg([0, 1], [3, 1], -1)
    legs = [la, lb, lc, ld]
    bl = charge_blocks(legs, modulus=modulus)
    rng = np.random.default_rng(11)
    data = rng.standard_normal(bl.n_elem)
    T = tq.BlockSparseTensor.from_charges(legs, data, modulus=modulus)
    dim, b, e, t, o = T.metadata()
    assert np.array_equal(b.T, bl.begin) and np.array_equal(e.T, bl.end)
    assert np.array_equal(T.data(), data)
    for leg, (x, y) in ((0, (la, lb)), (1, (lb, lc)), (2, (lc, ld))):
        F, fused = T.fuse_sectors(leg, x, y, modulus)
        assert F.rank == 3
        S = F.split_sectors(leg, x, y, modulus)
        d2, b2, e2, t2, o2 = S.metadata()
        assert np.array_equal(d2, dim) and np.array_equal(b2, b) and np.array_equal(e2, e)
        assert np.array_equal(t2, t) and np.array_equal(o2, o)
        assert np.array_equal(S.data(), data)
    Z = tq.BlockSparseTensor.from_charges(legs, None, modulus=modulus)
    assert Z.n_blocks == bl.n_blocks and not np.any(Z.data())


def test_split_rejects_blocks_across_pairs(tq):
    """A block covering two sector pairs of the leg cannot be split."""
    T = tq.BlockSparseTensor([6, 2], np.ones(12), [[0], [0]], [[5], [1]])
    with pytest.raises(tq.TorqueError) as ei:
        T.split_leg(0, [0, 1, 2], [0, 3], [[0], [3]])
    assert "exactly one sector pair" in str(ei.value)
