"""The cost model's stored training data (CPU): the exhaustive tuner's
measurements of the 2,000 random contractions of seed 4 load, match the
candidate table, and line up with the held-out contractions' structure,
which regenerates the same block lists."""
import numpy as np

from torque_gb300 import costmodel as cm, workloads


def test_dataset_and_held_out_specs():
    recs = cm.load_records(cm.DATASET)
    assert len(recs) == 2000
    train, test = cm.split(recs)
    assert len(train) == 1800 and len(test) == 200
    specs = cm.held_out_specs()
    assert [s["index"] for s in specs] == [r.index for r in test]
    for r in recs:
        assert r.features.shape == (32,) and np.all(np.isfinite(r.features))
        assert r.ms.shape == (len(cm.CANDIDATES),) and np.all(r.status == 0)
        assert r.err[0] == 0.0  # plain FP64 against itself
        for eps in cm.TARGETS:
            assert cm.best_feasible(r.ms, r.err, r.status, eps) >= 0
    X, T = cm.training_arrays(train)
    assert X.shape == (len(train) * len(cm.TARGETS), 32) and T.shape[1] == len(cm.CANDIDATES)
    assert np.all(T.min(axis=1) == 0.0)  # the best feasible candidate scores 0


def test_held_out_specs_rebuild_the_draws():
    specs = cm.held_out_specs()
    first = workloads.from_spec(specs[0])
    fl, npairs = workloads.pair_stats(first.A, first.B, first.pairs)
    assert npairs > 0 and fl > 0
    assert first.A.n_elem <= 1 << 21 and first.B.n_elem <= 1 << 21


def _rec(ms, err, status=None, flops=1e9):
    n = len(ms)
    return cm.TuneRecord(0, np.zeros(32, np.float32), flops,
                         np.zeros(n, np.int32) if status is None else np.asarray(status, np.int32),
                         np.asarray(ms, float), np.asarray(err, float))


def test_labels_and_regret_logic():
    """Training targets: log2 slowdown against the fastest candidate meeting the
    target, PENALTY for misses; the regret report falls back to the tuner."""
    n = len(cm.CANDIDATES)
    ms = np.full(n, 8.0)
    err = np.full(n, 1e-12)
    ms[3], ms[5] = 2.0, 1.0
    err[5] = 1e-7          # fastest, but too coarse for 1e-10
    r = _rec(ms, err)
    assert cm.best_feasible(r.ms, r.err, r.status, 1e-10) == 3
    assert cm.best_feasible(r.ms, r.err, r.status, 1e-6) == 5
    X, T = cm.training_arrays([r], targets=(1e-10,))
    assert X.shape == (1, 32) and abs(X[0, 0] - 10 / 16) < 1e-6
    assert T[0, 3] == 0.0 and T[0, 5] == cm.PENALTY and T[0, 0] == 2.0  # log2(8 / 2)
    rep = cm.regret_report([r], [5], 1e-10)   # a pick that misses: the tuner's choice runs
    assert rep["miss_rate"] == 1.0 and rep["mean_regret"] == 0.0
    rep = cm.regret_report([r], [0], 1e-10)
    assert rep["mean_regret"] == 3.0 and rep["ms_total"] == 8.0
    d = cm.default_choice(1e-10)
    c = cm.CANDIDATES[d]
    assert c["slices"] == 5 and c["tile_n"] == 96 and c["native_fill"] == 0
