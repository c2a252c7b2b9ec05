"""The oracle pinned against the reference's known answers, then checked
against an independent dense contraction (CPU only)."""
import numpy as np
import pytest

from conftest import kat_spec, spec_arrays
from oracle import oracle as orc
from torque_gb300 import workloads


def host_bs(spec):
    dim, b, e, t, d = spec_arrays(spec)
    return orc.HostBS(dim, b, e, d, strides=t)


def apply_ops(case):
    """Run a KAT op list on the oracle (query / transpose; append and modify
    are restated on the host arrays as the reference does them)."""
    dim, b, e, t, d = spec_arrays(case)
    T = orc.HostBS(dim, b, e, d, strides=t)
    for op in case["ops"]:
        if op[0] == "query":
            if T.rank == 0:
                got = float(T.data[0]) if T.data.size else 0.0
            else:
                got = orc.query(T, op[1])
            assert got == op[2], (case["name"], op)
        elif op[0] == "transpose":
            T = orc.hard_transpose(T, op[1])
        elif op[0] == "append":
            nb = np.vstack([T.begin, [op[1]]])
            ne = np.vstack([T.end, [op[2]]])
            nt = np.vstack([T.strides, [op[3]]])
            T = orc.HostBS(T.dimension, nb, ne, np.concatenate([T.data, op[4]]), strides=nt)
        elif op[0] == "modify":
            idx = np.asarray(op[1], np.int64)
            if T.rank == 0:
                T = orc.HostBS(T.dimension, T.begin, T.end, np.array([float(op[2])]))
                continue
            hits = [k for k in range(T.n_blocks)
                    if np.all(idx >= T.begin[k]) and np.all(idx <= T.end[k])]
            data = T.data.copy()
            if hits:
                for q, k in enumerate(hits):
                    a = T.offsets[k] + int(np.sum((idx - T.begin[k]) * T.strides[k]))
                    data[a] = op[2] if q == 0 else 0.0
                T = orc.HostBS(T.dimension, T.begin, T.end, data, strides=T.strides)
            elif op[2] != 0:
                T = orc.HostBS(T.dimension, np.vstack([T.begin, [idx]]), np.vstack([T.end, [idx]]),
                               np.concatenate([data, [op[2]]]),
                               strides=np.vstack([T.strides, [np.zeros_like(idx)]]))


def test_kat_tensor_ops(kat):
    for case in kat["cases"]:
        apply_ops(case)


@pytest.mark.parametrize("mode", [0, 1])
def test_kat_contractions(kat, mode):
    for case in kat["contractions"]:
        A = host_bs(kat_spec(kat, case["A"]))
        Bspec = case["B"]
        B = A if Bspec == "A" else host_bs(kat_spec(kat, Bspec) if isinstance(Bspec, str) else Bspec)
        if isinstance(Bspec, str) and Bspec != "A":
            B = host_bs([c for c in kat["contractions"] if c["name"] == Bspec][0]["B"])
        res = orc.contract(A, B, case["pairs"], mode=mode)
        if "scalar" in case:
            assert res == case["scalar"], case["name"]
            continue
        ob, oe, off, data = res
        ro = A.rank + B.rank - 2 * len(case["pairs"])
        dim = np.concatenate([np.delete(A.dimension, [p[0] for p in case["pairs"]]),
                              np.delete(B.dimension, [p[1] for p in case["pairs"]])])
        C = orc.HostBS(dim, ob, oe, data, offsets=off)
        assert C.rank == ro
        if "dense_column_major" in case:
            dense = orc.densify(C)
            assert np.array_equal(dense.ravel(order="F"), case["dense_column_major"]), case["name"]
        for idx, val in case.get("queries", []):
            assert orc.query(C, idx) == val, (case["name"], idx)


def small_host():
    c = workloads.small_u1()
    A = orc.HostBS(c.A.dimension, c.A.begin, c.A.end, c.a_data)
    B = orc.HostBS(c.B.dimension, c.B.begin, c.B.end, c.b_data)
    return c, A, B


def test_small_u1_structure():
    c, A, B = small_host()
    assert A.n_blocks == 85 and B.n_blocks == 85 and A.data.size == 54244
    pa, pb = orc.match(A, B, c.pairs)
    assert pa.size == 325
    # reference order: A ascending, then B ascending within each A block
    assert np.all(np.diff(pa) >= 0)
    for i in np.unique(pa):
        assert np.all(np.diff(pb[pa == i]) > 0)
    # distinct output boxes
    ob, oe, off, data = orc.contract(A, B, c.pairs, mode=1)
    assert len({tuple(x) for x in ob}) == 85
    assert c.flops() == 11590920.0


def test_small_u1_dense_parity():
    """Reference-layout result, densified (overlaps add as query does), equals the
    dense contraction of the zero-filled tensors."""
    c, A, B = small_host()
    ob, oe, off, data = orc.contract(A, B, c.pairs, mode=0)
    C = orc.HostBS(np.array([24] * 4), ob, oe, data, offsets=off)
    got = orc.densify(C)
    want = orc.dense_contract(orc.densify(A), orc.densify(B), c.pairs)
    scale = np.abs(orc.densify(A)).max() * np.abs(orc.densify(B)).max() * 576
    assert np.max(np.abs(got - want)) <= 1e-13 * scale
    # plain-double mode agrees with the compensated one to rounding
    _, _, _, d1 = orc.contract(A, B, c.pairs, mode=1)
    assert np.max(np.abs(d1 - data)) <= 1e-13 * np.max(np.abs(data))


def test_cpu_baseline_port_matches_oracle():
    """The timed CPU baseline (gather into matrices, then multiply) gives the
    reference-layout values of the accurate oracle to rounding."""
    c, A, B = small_host()
    pa, pb = orc.match(A, B, c.pairs)
    out, offs, threads = orc.pairs_baseline(A, B, c.pairs, pa, pb)
    ob, oe, off, want = orc.contract(A, B, c.pairs, mode=0)
    assert np.array_equal(offs, off) and threads >= 1
    assert np.max(np.abs(out - want)) <= 1e-13 * np.max(np.abs(want))


def test_reference_cpu_stride_defect():
    """The reference CPU path reads element strides from column j_block of each
    tensor's index tables (src/tensor/block_sparse.h:531,538).  With uneven blocks
    that gives wrong values; mode 2 reproduces it, mode 0 is the intended result."""
    c, A, B = small_host()
    ok, wrong = 0, 0
    pa, pb = orc.match(A, B, c.pairs)
    jb = 0
    for q in range(pa.size):
        jb = jb + 1 if q and pa[q] == pa[q - 1] else 0
        good = orc.pair_values(A, B, c.pairs, int(pa[q]), int(pb[q]), mode=0)
        bad = orc.pair_values(A, B, c.pairs, int(pa[q]), int(pb[q]), mode=2, j_block=jb)
        if np.allclose(good, bad):
            ok += 1
        else:
            wrong += 1
    assert wrong > 0 and ok > 0


def test_overlapping_boxes_and_partial_intervals():
    """Boxes that overlap partially on contracted legs: the sub-box rule of
    block_in_range, checked against the dense contraction."""
    rng = np.random.default_rng(5)
    dimA = np.array([6, 7, 5])
    A = orc.HostBS(dimA, [[0, 0, 0], [2, 3, 1], [1, 0, 2]], [[3, 4, 2], [5, 6, 4], [4, 2, 4]],
                   rng.standard_normal(4 * 5 * 3 + 4 * 4 * 4 + 4 * 3 * 3))
    dimB = np.array([7, 4])
    B = orc.HostBS(dimB, [[1, 0], [4, 1], [0, 2]], [[5, 2], [6, 3], [2, 3]],
                   rng.standard_normal(5 * 3 + 3 * 3 + 3 * 2))
    pairs = [[1, 0]]
    ob, oe, off, data = orc.contract(A, B, pairs, mode=0)
    C = orc.HostBS(np.array([6, 5, 4]), ob, oe, data, offsets=off)
    want = orc.dense_contract(orc.densify(A), orc.densify(B), pairs)
    assert np.allclose(orc.densify(C), want, rtol=0, atol=1e-12)


def test_slice_boxes_hand_case():
    """slice restated (block_sparse.cuh:1124-1176): a 4 x 6 block cut by (2, 3)
    gives six 2 x 2 sub-boxes, leg 0 fastest."""
    b, e = orc.slice_boxes([[1, 0]], [[4, 5]], [2, 3])
    assert b.tolist() == [[1, 0], [3, 0], [1, 2], [3, 2], [1, 4], [3, 4]]
    assert e.tolist() == [[2, 1], [4, 1], [2, 3], [4, 3], [2, 5], [4, 5]]
