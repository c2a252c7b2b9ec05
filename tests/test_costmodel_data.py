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
