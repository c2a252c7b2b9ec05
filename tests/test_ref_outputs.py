"""The oracle against the reference's own CPU code.

tests/golden/ref_outputs.npz holds outputs of the reference's
``BlockSparseTensor<double>`` (src/tensor/block_sparse.h, block_sparse.cpp),
compiled from its sources against the project's Armadillo API subset and run
by tests/golden/make_ref_outputs.py, in two builds: the headers as they are
("asis") and with the CPU contract's two stride lookups corrected
(block_sparse.h:531,538; "fixed").  The fixture tests run everywhere: the
oracle's reference-layout contraction (mode 0) must give the fixed build's
block list bit-exactly and its values within 1e-13 of max|C|, and the
oracle's restatement of the defect (mode 2) must give the as-is build's values
(or raise where it throws; where the as-is strides would read past a
tensor's values the reference's result is undefined, the case is marked so
and the as-is build is not run on it).  Transpositions are bit-exact; overlapping reads
sum in block order, as the reference does, and are bit-exact too.

The live tests need the compiled reference (oracle/_ref/, present only where
its sources are) and skip elsewhere: the reference's own known-answer cases
through the compiled code (which checks the Armadillo API subset), random
ragged cases against the oracle, the block matcher against orc_match, and a
regeneration of the fixture compared with the committed one.
"""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN, kat_spec, spec_arrays
from oracle import oracle as orc
from oracle import ref

if GOLDEN not in sys.path:
    sys.path.insert(0, GOLDEN)
import ref_cases as rc  # noqa: E402

TOL = 1e-13

live = pytest.mark.skipif(not (ref.available("fixed") and ref.available("asis")),
                          reason="the compiled reference (oracle/_ref) exists only where its "
                                 "sources are")


@pytest.fixture(scope="module")
def fx():
    return rc.load()


def compare_contraction(out, fx, key):
    """Compare an oracle result with the fixture entries under key."""
    if key + "scalar" in fx:
        want = float(fx[key + "scalar"])
        assert abs(out - want) <= TOL * max(abs(want), 1.0)
        return
    ob, oe, off, data = out
    assert np.array_equal(ob, fx[key + "begin"]) and np.array_equal(oe, fx[key + "end"])
    assert np.array_equal(off, fx[key + "offsets"])
    sizes = rc.block_sizes(ob, oe)
    if key + "values" in fx:
        want = fx[key + "values"]
        assert data.shape == want.shape
        assert np.max(np.abs(data - want)) <= TOL * max(np.max(np.abs(want)), 1e-300)
    else:
        got = rc.value_digest(off, sizes, data)
        assert rc.digest_close(got, fx[key + "digest"], sizes, TOL)


@pytest.mark.parametrize("name", list(rc.CONTRACTIONS))
def test_oracle_matches_reference_outputs(fx, name):
    A, B, pairs = rc.CONTRACTIONS[name]()
    assert rc.input_digest(A, B) == str(fx[name + "__input"])
    assert np.array_equal(pairs, fx[name + "__pairs"])
    for variant, mode in (("fixed", 0), ("asis", 2)):
        key = "%s__%s__" % (name, variant)
        if key + "undefined" in fx:
            with pytest.raises(orc.UndefinedRead):
                orc.contract(A, B, pairs, mode=mode)
            continue
        if key + "error" in fx:
            with pytest.raises(IndexError):
                orc.contract(A, B, pairs, mode=mode)
            continue
        compare_contraction(orc.contract(A, B, pairs, mode=mode), fx, key)


@pytest.mark.parametrize("name", rc.FLOAT_CASES)
def test_reference_float_outputs_agree_with_oracle(fx, name):
    """The reference's float instantiation on the same inputs rounded to
    float32: the block list is the double one, values within 1e-5 of max|C|
    of the oracle's float64 result on the rounded inputs."""
    A, B, pairs = rc.CONTRACTIONS[name]()
    r = lambda T: orc.HostBS(T.dimension, T.begin, T.end, T.data.astype(np.float32),
                             strides=T.strides, offsets=T.offsets)
    ob, oe, off, want = orc.contract(r(A), r(B), pairs, mode=0)
    key = "%s__f32__" % name
    assert np.array_equal(ob, fx[key + "begin"]) and np.array_equal(oe, fx[key + "end"])
    assert np.array_equal(off, fx[key + "offsets"])
    sizes = rc.block_sizes(ob, oe)
    if key + "values" in fx:
        got = fx[key + "values"].astype(np.float64)
        assert np.max(np.abs(got - want)) <= 1e-5 * np.max(np.abs(want))
    else:
        assert rc.digest_close(rc.value_digest(off, sizes, want), fx[key + "digest"], sizes, 1e-5)


def test_fixture_covers_both_builds(fx):
    """The stored cases include the as-is build's wrong values (uneven
    blocks), its bounds error (more partners than A blocks) and a scalar."""
    d = fx["u1_85__asis__digest"] - fx["u1_85__fixed__digest"]
    assert np.max(np.abs(d)) > 1e-3
    assert "index out of bounds" in str(fx["one_block_many_partners__asis__error"])
    assert "one_block_many_partners__fixed__values" in fx
    assert "vector_dot__fixed__scalar" in fx


@pytest.mark.parametrize("tname", ["transpose_r4", "transpose_r4_rowmajor"])
def test_oracle_transpose_matches_reference(fx, tname):
    T = rc.transpose_cases()[tname]
    assert rc.input_digest(T) == str(fx[tname + "__input"])
    for k, perm in enumerate(rc.TRANSPOSE_PERMS):
        key = "%s__%d__" % (tname, k)
        assert np.array_equal(fx[key + "perm"], perm)
        R = orc.hard_transpose(T, perm)
        assert np.array_equal(R.begin, fx[key + "begin"]) and np.array_equal(R.end, fx[key + "end"])
        assert np.array_equal(R.strides, fx[key + "tables"])
        assert np.array_equal(R.offsets, fx[key + "offsets"])
        assert np.array_equal(R.data, fx[key + "values"])


def test_oracle_query_matches_reference(fx):
    Q, points = rc.query_r3()
    assert rc.input_digest(Q) == str(fx["query_r3__input"])
    assert np.array_equal(points, fx["query_r3__points"])
    got = np.array([orc.query(Q, p) for p in points])
    assert np.array_equal(got, fx["query_r3__values"])
    assert np.count_nonzero(got) > 10


# ---- live: the compiled reference itself ----------------------------------

def _ref_from_spec(spec, variant):
    dim, b, e, t, d = spec_arrays(spec)
    T = ref.RefTensor.empty(dim, variant)
    o = 0
    for i in range(b.shape[0]):
        n = int(np.prod(e[i] - b[i] + 1))
        table = t[i] if t is not None else np.concatenate([[1], np.cumprod(e[i] - b[i] + 1)[:-1]])
        T.append_block(d[o:o + n], b[i], e[i], table)
        o += n
    return T


@live
@pytest.mark.parametrize("variant", ["fixed", "asis"])
def test_reference_build_passes_its_known_answers(kat, variant):
    """The reference's own known answers (test/gpu/block_sparse_test.cu:10-231,
    the same cases as test/block_sparse_tensor_test.cpp) through the compiled
    reference: a check of the Armadillo API subset it was compiled against."""
    for case in kat["cases"]:
        T = _ref_from_spec(case, variant)
        for op in case["ops"]:
            if op[0] == "query":
                assert T.query(op[1]) == op[2], (case["name"], op)
            elif op[0] == "modify":
                T.modify(op[1], op[2])
            elif op[0] == "append":
                T.append_block(np.asarray(op[4], np.float64), op[1], op[2], op[3])
            elif op[0] == "transpose":
                T = T.hard_transpose(op[1])
    for case in kat["contractions"]:
        A = _ref_from_spec(kat_spec(kat, case["A"]), variant)
        if case["B"] == "A":
            B = A
        else:
            bspec = [c for c in kat["contractions"] if c["name"] == case["B"]][0]["B"] \
                if isinstance(case["B"], str) else case["B"]
            B = _ref_from_spec(bspec, variant)
        C = A.contract(B, case["pairs"])
        if "scalar" in case:
            assert C.read()[5][0] == case["scalar"], case["name"]
            continue
        for idx, val in case.get("queries", []):
            assert C.query(idx) == val, (case["name"], idx)
        if "dense_column_major" in case:
            H = C.host()
            got = orc.densify(H).reshape(-1, order="F")
            assert np.array_equal(got, np.asarray(case["dense_column_major"], np.float64))


# No full contraction over two or more legs: the reference's rank-0 path
# splits the contraction index with the range's dimensions in place of their
# stride table (block_sparse.h:557-558), which gives a wrong scalar and can
# read outside the block for ragged ranges; only one-leg scalars are run.
RANDOM_SHAPES = [([6, 7, 5], [7, 4], [[1, 0]]), ([5, 6, 4], [6, 5, 3], [[1, 0], [0, 1]]),
                 ([4, 5, 6, 3], [6, 3, 4], [[2, 0], [3, 1]]), ([8], [8, 3], [[0, 0]]),
                 ([5, 4, 3], [3, 4, 5], [[0, 2], [2, 0]]), ([9], [9], [[0, 0]])]


@live
@pytest.mark.parametrize("seed", range(100, 124))
def test_live_random_cases_match_oracle(seed):
    da, db, pairs = RANDOM_SHAPES[seed % len(RANDOM_SHAPES)]
    A, B, pairs = rc.ragged(seed, da, db, pairs, n_a=6 + seed % 5, n_b=7 + seed % 4)
    for variant, mode in (("fixed", 0), ("asis", 2)):
        try:
            got = orc.contract(A, B, pairs, mode=mode)
        except orc.UndefinedRead:
            continue      # the as-is reference would read past its values: not run
        except IndexError:
            with pytest.raises(ref.RefError, match="out of bounds"):
                ref.contract(A, B, pairs, variant=variant)
            continue
        want = ref.contract(A, B, pairs, variant=variant)
        if isinstance(want, float):
            assert abs(got - want) <= TOL * max(abs(want), 1.0)
            continue
        for g, w in zip(got[:3], want[:3]):
            assert np.array_equal(g, w)
        assert np.max(np.abs(got[3] - want[3]), initial=0.0) <= \
            TOL * max(np.max(np.abs(want[3]), initial=0.0), 1e-300)


@live
def test_live_block_matcher_matches_oracle():
    """block_in_range (block_sparse.cpp:6-175) per A block of the 85-block U(1)
    pair: the partners, in order, are the oracle's pair list for that block."""
    A, B, pairs = rc.u1_85()
    pa, pb = orc.match(A, B, pairs)
    for i in range(A.n_blocks):
        found = ref.block_in_range(pairs, A.begin[i], A.end[i], B.begin, B.end)
        assert np.array_equal(found, pb[pa == i])


@live
def test_live_fixture_is_current(fx):
    """Regenerating the outputs with the compiled reference gives the
    committed fixture."""
    for name, make in rc.CONTRACTIONS.items():
        A, B, pairs = make()
        for variant in ("fixed", "asis"):
            key = "%s__%s__" % (name, variant)
            if key + "undefined" in fx:
                continue
            try:
                out = ref.contract(A, B, pairs, variant=variant)
            except ref.RefError as e:
                assert str(fx[key + "error"]) == str(e)
                continue
            if isinstance(out, float):
                assert float(fx[key + "scalar"]) == out
                continue
            assert np.array_equal(out[0], fx[key + "begin"])
            if key + "values" in fx:
                assert np.array_equal(out[3], fx[key + "values"])
            else:
                d = rc.value_digest(out[2], rc.block_sizes(out[0], out[1]), out[3])
                assert np.array_equal(d, fx[key + "digest"])


@live
@pytest.mark.parametrize("seed", range(200, 206))
def test_live_transpose_and_query_match_oracle(seed):
    """Random ragged tensors of rank 2 to 5 (overlapping boxes, extent-1 legs
    among them): every leg permutation through the reference's
    hard_transpose (block_sparse.h:607-651) and the oracle's, bit-exact, and
    64 element reads through its query (block_sparse.h:372-411), bit-exact."""
    import itertools
    rng = np.random.default_rng(seed)
    rank = 2 + seed % 4
    dims = rng.integers(2, 7, size=rank)
    T = rc.random_tensor(rng, dims, 6 + seed % 3, max_extent=3)
    perms = list(itertools.permutations(range(rank)))
    for p in perms[:: max(1, len(perms) // 12)]:
        R = ref.hard_transpose(T, p)
        O = orc.hard_transpose(T, p)
        assert np.array_equal(R.begin, O.begin) and np.array_equal(R.end, O.end)
        assert np.array_equal(R.strides, O.strides) and np.array_equal(R.offsets, O.offsets)
        assert np.array_equal(R.data, O.data)
    points = np.stack([rng.integers(0, d, 64) for d in dims], 1)
    R = ref.RefTensor.from_host(T)
    for p in points:
        assert R.query(p) == orc.query(T, p)


@live
def test_live_modify_fixture_is_current(fx):
    """Replaying the write/read sequence on the compiled reference gives the
    committed reads and final tensor."""
    M, ops = rc.modify_r3()
    assert rc.input_digest(M) == str(fx["modify_r3__input"])
    R = ref.RefTensor.from_host(M)
    reads = []
    for kind, idx, value in ops:
        if kind == "modify":
            R.modify(idx, value)
        else:
            reads.append(R.query(idx))
    assert np.array_equal(np.asarray(reads), fx["modify_r3__reads"])
    H = R.host()
    assert np.array_equal(H.begin, fx["modify_r3__begin"])
    assert np.array_equal(H.strides, fx["modify_r3__tables"])
    assert np.array_equal(H.data, fx["modify_r3__values"])
    assert H.n_blocks > M.n_blocks       # writes outside every block appended blocks


def _ref_partners_chunk(args):
    """Worker: the reference's block_in_range for a range of A blocks of the
    full uneven case; returns (A block, partner) pairs in order."""
    lo, hi = args
    from oracle import ref as r
    from torque_gb300 import workloads
    c = workloads.uneven_u1(data=False)
    out = []
    for i in range(lo, hi):
        found, nb, ne = r.block_in_range(c.pairs, c.A.begin[i], c.A.end[i], c.B.begin, c.B.end,
                                          boxes=True)
        out.append(np.concatenate([np.full((found.size, 1), i, np.int64), found[:, None], nb, ne],
                                  1))
    return np.concatenate(out) if out else np.zeros((0, 10), np.int64)


@live
def test_live_full_size_pair_list_is_the_references():
    """The full uneven case (23,969 blocks per tensor): the reference's own
    block matcher (block_in_range, block_sparse.cpp:6-175), run for every A
    block against all B blocks (5.7e8 interval tests, spread over worker
    processes), gives the oracle's 593,505-pair list in the same order, the
    same output boxes and offsets; the CUDA path's list equals the oracle's at
    this size (tests/test_gpu_headline_structure.py)."""
    import concurrent.futures
    import multiprocessing
    from torque_gb300 import workloads
    c = workloads.uneven_u1(data=False)
    z = np.zeros(1)
    A = orc.HostBS(c.A.dimension, c.A.begin, c.A.end, z)
    B = orc.HostBS(c.B.dimension, c.B.begin, c.B.end, z)
    pa, pb = orc.match(A, B, c.pairs)
    n = A.n_blocks
    workers = max(1, min(8, os.cpu_count() or 1))
    bounds = np.linspace(0, n, 4 * workers + 1).astype(int)
    chunks = [(int(bounds[k]), int(bounds[k + 1])) for k in range(len(bounds) - 1)]
    ctx = multiprocessing.get_context("spawn")
    with concurrent.futures.ProcessPoolExecutor(workers, mp_context=ctx) as ex:
        parts = list(ex.map(_ref_partners_chunk, chunks))
    got = np.concatenate(parts)
    assert got.shape[0] == 593505 == pa.size
    assert np.array_equal(got[:, 0], pa) and np.array_equal(got[:, 1], pb)
    # each pair's output box (A's free legs then B's), and the offsets as the
    # exclusive scan of the box sizes (nest_sum), as the oracle's block list
    _, _, ob, oe, off = orc.contract_blocks(A, B, c.pairs)
    assert np.array_equal(got[:, 2:6], ob) and np.array_equal(got[:, 6:10], oe)
    sizes = np.prod(got[:, 6:10] - got[:, 2:6] + 1, axis=1)
    assert np.array_equal(np.concatenate([[0], np.cumsum(sizes)[:-1]]), off)
