"""Host-side block-list builders (CPU): the pruned U(1) enumeration equals the
brute-force one, charge-ordered fusion tiles the fused leg, and the seeded
workload generators are deterministic and respect their caps."""
import numpy as np
import pytest

from torque_gb300 import sectors as S
from torque_gb300 import workloads as W


def test_u1_enumeration_matches_brute_force():
    rng = np.random.default_rng(0)
    for _ in range(200):
        r = int(rng.integers(1, 6))
        legs = [S.Leg(list(range(-(k // 2), k - k // 2)), [1] * k, int(rng.choice([-1, 1])))
                for k in rng.integers(1, 7, r)]
        tot = int(rng.integers(-2, 3))
        fast = S._u1_tuples(legs, tot)
        shape = [len(l.charges) for l in legs]
        grids = np.meshgrid(*[np.arange(n) for n in shape], indexing="ij")
        sidx = np.stack([g.ravel(order="F") for g in grids], axis=1).astype(np.int64)
        q = sum(l.direction * np.asarray(l.charges)[sidx[:, i]] for i, l in enumerate(legs))
        assert np.array_equal(fast, sidx[q == tot])


def test_fusion_tiles_the_fused_leg():
    a = S.Leg([-1, 0, 1], [2, 3, 2], 1)
    b = S.Leg([0, 1], [2, 3], -1)
    fused, off = S.fuse_sector_order(a, b)
    assert fused.dim == a.dim * b.dim
    starts = sorted((off[i, j], a.sizes[i] * b.sizes[j]) for i in range(3) for j in range(2))
    run = 0
    for o, n in starts:
        assert o == run
        run += n
    assert list(fused.charges) == sorted(fused.charges)


def test_uneven_case_counts():
    u = W.uneven_u1(data=False)
    assert u.A.n_blocks == 23969 and u.A.dimension[0] == 488
    fl, npairs = W.pair_stats(u.A, u.B, u.pairs)
    assert npairs == 593505 and abs(fl - 7.1288767e13) / 7.13e13 < 1e-6


def test_random_contractions_deterministic_and_capped():
    a = W.random_contractions(6, seed=4, max_elem=1 << 21, max_blocks=20000, max_flops=2e9)
    b = W.random_contractions(6, seed=4, max_elem=1 << 21, max_blocks=20000, max_flops=2e9)
    for x, y in zip(a, b):
        assert x.index == y.index and np.array_equal(x.A.begin, y.A.begin)
        assert np.array_equal(x.pairs, y.pairs)
        fl, npairs = W.pair_stats(x.A, x.B, x.pairs)
        assert 0 < fl <= 2e9 and npairs <= 1 << 18
        assert x.A.n_elem <= 1 << 21 and x.B.n_elem <= 1 << 21
        assert 3 <= x.A.begin.shape[1] <= 6 and 1 <= x.pairs.shape[0] <= 3
        z = W.from_spec(x.spec())
        assert np.array_equal(z.B.end, x.B.end)


@pytest.mark.parametrize("modulus", [None, 2, 3])
def test_charge_blocks_c_abi_matches_python(modulus):
    """tq_charge_blocks (C ABI, host code) lists the same blocks in the same
    order (leg 0 fastest) as the Python constructor, for U(1) and Z_n."""
    from torque_gb300 import block_sparse
    from torque_gb300.sectors import Leg, charge_blocks
    legs = [Leg([-1, 0, 2], [2, 3, 1], +1), Leg([0, 1], [4, 2], +1),
            Leg([-2, 0, 1, 3], [1, 2, 2, 1], -1), Leg([1, 0], [3, 3], -1)]
    for total in (0, 1):
        want = charge_blocks(legs, total=total, modulus=modulus)
        b, e = block_sparse.charge_block_list(legs, total=total, modulus=modulus)
        assert np.array_equal(b, want.begin) and np.array_equal(e, want.end)
