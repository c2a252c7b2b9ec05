"""Block-level truncated SVD (tq_bs_svd) against numpy's SVD of the densified
matrix: singular values, reconstruction, isometric factors, and truncation
error equal to the discarded weight (Eckart-Young), FP64 tolerances."""
import numpy as np
import pytest

from oracle import oracle as orc
from torque_gb300.sectors import Leg, charge_blocks

pytestmark = pytest.mark.gpu


def dense(T):
    dim, b, e, t, o = T.metadata()
    return orc.densify(orc.HostBS(dim, b.T, e.T, T.data(), t.T))


def site(tq, seed):
    legs = [Leg([-1, 0, 1], [3, 5, 4], +1), Leg([0, 1], [4, 3], +1),
            Leg([-1, 0, 1, 2], [2, 4, 3, 2], -1), Leg([0, 1], [3, 4], -1)]
    bl = charge_blocks(legs)
    rng = np.random.default_rng(seed)
    data = rng.standard_normal(bl.n_elem)
    return tq.BlockSparseTensor.from_charges(legs, data)


@pytest.mark.parametrize("row_legs", [[0, 1], [2, 0], [3]])
def test_svd_full_rank(tq, row_legs):
    T = site(tq, 3)
    D = dense(T)
    U, S, V = T.svd(row_legs)
    cols = [l for l in range(4) if l not in row_legs]
    Dm = np.transpose(D, row_legs + cols)
    rs = int(np.prod([D.shape[l] for l in row_legs]))
    mat = Dm.reshape(rs, -1, order="F")
    want = np.linalg.svd(mat, compute_uv=False)
    got = np.sort(S.data())[::-1]
    want = want[want > 1e-13 * want[0]]
    assert got.size == want.size
    assert np.max(np.abs(got - want)) <= 1e-12 * want[0]
    u, sv, v = dense(U), dense(S), dense(V)
    k = u.shape[-1]
    um = u.reshape(rs, k, order="F")
    vm = v.reshape(k, -1, order="F")
    assert np.max(np.abs(um.T @ um - np.eye(k))) <= 1e-12
    assert np.max(np.abs(vm @ vm.T - np.eye(k))) <= 1e-12
    rec = (um * sv) @ vm
    assert np.max(np.abs(rec - mat)) <= 1e-12 * np.max(np.abs(mat))


@pytest.mark.parametrize("keep", [5, 17])
def test_svd_truncation(tq, keep):
    T = site(tq, 4)
    D = dense(T)
    mat = D.reshape(D.shape[0] * D.shape[1], -1, order="F")
    full = np.linalg.svd(mat, compute_uv=False)
    U, S, V = T.svd([0, 1], max_keep=keep)
    got = np.sort(S.data())[::-1]
    assert got.size == keep
    assert np.max(np.abs(got - full[:keep])) <= 1e-12 * full[0]
    u, sv, v = dense(U), dense(S), dense(V)
    k = u.shape[-1]
    rec = (u.reshape(-1, k, order="F") * sv) @ v.reshape(k, -1, order="F")
    err = np.linalg.norm(rec - mat)
    assert abs(err - np.sqrt(np.sum(full[keep:] ** 2))) <= 1e-10 * full[0]
    # cutoff: values below 0.3 of the largest go
    U2, S2, V2 = T.svd([0, 1], cutoff=0.3)
    assert np.array_equal(np.sort(S2.data())[::-1], np.sort(S2.data())[::-1])
    assert S2.data().size == int(np.sum(full > 0.3 * full[0]))


@pytest.mark.parametrize("row_legs", [[0, 1], [2, 0], [3], [0, 1, 3]])
def test_qr(tq, row_legs):
    """Q R reproduces the tensor, Q has orthonormal columns, and each class's
    R (its blocks side by side, in the order the library emits them) is upper
    trapezoidal with a non-negative diagonal; R = Q^T A."""
    T = site(tq, 6)
    D = dense(T)
    Q, R = T.qr(row_legs)
    cols = [l for l in range(4) if l not in row_legs]
    rs = int(np.prod([D.shape[l] for l in row_legs]))
    mat = np.transpose(D, row_legs + cols).reshape(rs, -1, order="F")
    q, rr = dense(Q), dense(R)
    k = q.shape[-1]
    qm = q.reshape(rs, k, order="F")
    rm = rr.reshape(k, -1, order="F")
    assert np.max(np.abs(qm.T @ qm - np.eye(k))) <= 1e-12
    assert np.max(np.abs(qm @ rm - mat)) <= 1e-12 * np.max(np.abs(mat))
    assert np.max(np.abs(qm.T @ mat - rm)) <= 1e-12 * np.max(np.abs(mat))
    # per class: R's blocks of one bond sector, side by side
    dim, b, e, t, o = R.metadata()
    data = R.data()
    sectors = {}
    for blk in range(b.shape[1]):
        sectors.setdefault(int(b[0, blk]), []).append(blk)
    assert sum(int(e[0, v[0]] - b[0, v[0]] + 1) for v in sectors.values()) == k
    for lo, blks in sectors.items():
        kc = int(e[0, blks[0]] - lo + 1)
        parts = []
        for blk in blks:
            n = int(np.prod(e[1:, blk] - b[1:, blk] + 1))
            parts.append(data[o[blk]:o[blk] + kc * n].reshape(kc, n, order="F"))
        rc = np.concatenate(parts, axis=1)
        assert np.all(np.tril(rc, -1) == 0.0)
        assert np.all(np.diag(rc) >= 0.0)


def test_qr_rejects_bad_legs(tq):
    T = site(tq, 7)
    with pytest.raises(tq.TorqueError):
        T.qr([])
    with pytest.raises(tq.TorqueError):
        T.qr([0, 1, 2, 3])
