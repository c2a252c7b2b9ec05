"""Schedule selection: the exhaustive autotuner's candidate table, the data it
generates, and the learned cost model trained on it.

A schedule is a tq_contract_opts (precision and slice count, tensor-core tile
width, block grouping).  The exhaustive tuner (tq_autotune) runs every
candidate on a planned contraction and measures its time and its error
against the plain FP64 result.  The cost model is a 3-layer FP32 perceptron
(tq_mlp_*: trained and evaluated by the library's own CUDA kernels) that reads
TQ_N_FEATURES features of the planned contraction (tq_plan_features: ranks,
contracted legs and dimension, sizes, flop-weighted block-size histograms and
the target accuracy) and scores every candidate; the proposal is the lowest
score.  Training target of candidate c for a target accuracy eps:
    log2(ms_c / ms_best(eps))   if c ran and its error is <= eps
    PENALTY                     otherwise
where ms_best(eps) is the fastest candidate meeting eps, so a score is the
predicted slowdown against the exhaustive choice, in octaves.  The tuner stays
the fallback (a proposal that misses the target is replaced by its choice) and
the yardstick (regret is measured against it).

Device memory for the training arrays comes from torch (plumbing only: every
forward, backward and update is a library kernel).
"""
from __future__ import annotations

import ctypes
import json
import os
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import check, load

PENALTY = 4.0
TARGETS = (1e-6, 1e-8, 1e-10, 1e-12)

_DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")
# the exhaustive tuner's measurements of the 2,000 random contractions of seed 4
# (made on a GB300 by `python -m torque_gb300.costmodel --n 2000 --seed 4`)
DATASET = os.path.join(_DATA, "tune_random_s4.npz")
# the held-out contractions' structure (workloads.RandomContraction.spec)
HELD_OUT = os.path.join(_DATA, "random_s4_heldout.json")


def _cands():
    c = [dict(precision="native")]
    for s in (3, 4, 5, 6, 7):
        for tile_n in (32, 64, 96):
            for fill in (0, 250):
                c.append(dict(precision="bf16x3" if s == 3 else "ozaki", slices=s, tile_n=tile_n,
                              native_fill=fill))
    return c


# candidate schedules, in the order of the cost model's outputs
CANDIDATES = _cands()


def describe(c: dict) -> str:
    if c["precision"] == "native":
        return "fp64"
    return "s%d/n%d/g%d" % (c["slices"], c["tile_n"], c["native_fill"])


@dataclass
class TuneRecord:
    """What the exhaustive tuner measured on one contraction."""
    index: int
    features: np.ndarray  # TQ_N_FEATURES, feature 0 (target) left at 0
    flops: float
    status: np.ndarray    # per candidate
    ms: np.ndarray
    err: np.ndarray


def device_tensor(blocks, seed: int, device="cuda"):
    """A BlockSparseTensor over `blocks` with float64 N(0,1) entries drawn on
    the device (torch's Philox generator seeded with `seed`)."""
    import torch
    from .block_sparse import BlockSparseTensor
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    data = torch.randn(max(blocks.n_elem, 1), generator=g, dtype=torch.float64, device=device)
    b, e = blocks.points()
    t = BlockSparseTensor(blocks.dimension, data[:blocks.n_elem], b, e)
    torch.cuda.synchronize()
    return t


def plan_random(rc, seed: int, layout="reduced"):
    """Tensors and a tensor-core plan (so any schedule can be set later) for a
    random contraction."""
    from .block_sparse import ContractionPlan
    A = device_tensor(rc.A, seed * 1000003 + 2 * rc.index)
    B = device_tensor(rc.B, seed * 1000003 + 2 * rc.index + 1)
    P = ContractionPlan(A, B, rc.pairs, precision="ozaki", layout=layout)
    return A, B, P


def tune_record(rc, seed: int, reps: int = 2, candidates=None) -> TuneRecord:
    cands = CANDIDATES if candidates is None else candidates
    A, B, P = plan_random(rc, seed)
    f = P.features(1.0)
    f[0] = 0.0
    _, entries = P.autotune(1.0, cands, reps=reps)
    st = np.array([e[0] for e in entries], np.int32)
    ms = np.array([e[1] for e in entries], np.float64)
    err = np.array([e[2] for e in entries], np.float64)
    return TuneRecord(rc.index, f, P.flops, st, ms, err)


def best_feasible(rec_ms, rec_err, rec_status, target):
    ok = (rec_status == 0) & (rec_err <= target)
    if not ok.any():
        return -1
    return int(np.argmin(np.where(ok, rec_ms, np.inf)))


def training_arrays(records, targets=TARGETS):
    """(X, T): one sample per record and target accuracy."""
    X, T = [], []
    for r in records:
        for eps in targets:
            b = best_feasible(r.ms, r.err, r.status, eps)
            if b < 0:
                continue
            x = r.features.copy()
            x[0] = -np.log10(eps) / 16.0
            ok = (r.status == 0) & (r.err <= eps)
            t = np.where(ok, np.log2(np.maximum(r.ms, 1e-6) / r.ms[b]), PENALTY)
            X.append(x)
            T.append(np.minimum(t, PENALTY).astype(np.float32))
    return np.asarray(X, np.float32), np.asarray(T, np.float32)


class MLP:
    """The cost model network: n_in -> width -> width -> n_out, ReLU, FP32 on
    the device (tq_mlp_*)."""

    def __init__(self, n_in=_lib.TQ_N_FEATURES, width=64, n_out=None, seed=0):
        load()
        self.n_in, self.width = n_in, width
        self.n_out = len(CANDIDATES) if n_out is None else n_out
        self._h = ctypes.c_void_p()
        check(load().tq_mlp_create(n_in, width, self.n_out, seed, ctypes.byref(self._h)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                load().tq_mlp_destroy(h)
            except Exception:
                pass
            self._h = ctypes.c_void_p()

    @property
    def n_params(self) -> int:
        n = ctypes.c_int64()
        check(load().tq_mlp_num_params(self._h, ctypes.byref(n)))
        return n.value

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.n_params, np.float32)
        check(load().tq_mlp_get_params(self._h, p.ctypes.data_as(ctypes.c_void_p)))
        return p

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.n_params
        check(load().tq_mlp_set_params(self._h, p.ctypes.data_as(ctypes.c_void_p)))

    @staticmethod
    def _dev(a):
        import torch
        return torch.as_tensor(np.ascontiguousarray(a, np.float32)).cuda()

    def forward(self, X: np.ndarray) -> np.ndarray:
        import torch
        x = self._dev(X)
        y = torch.empty((x.shape[0], self.n_out), dtype=torch.float32, device="cuda")
        check(load().tq_mlp_forward(self._h, ctypes.c_void_p(x.data_ptr()), x.shape[0],
                                    ctypes.c_void_p(y.data_ptr()), None))
        torch.cuda.synchronize()
        return y.cpu().numpy()

    def gradients(self, X, T, mask=None):
        """(loss, gradient of every parameter) of the masked mean squared error."""
        x, t = self._dev(X), self._dev(T)
        m = None if mask is None else self._dev(mask)
        g = np.zeros(self.n_params, np.float32)
        loss = np.zeros(1, np.float32)
        check(load().tq_mlp_gradients(self._h, ctypes.c_void_p(x.data_ptr()),
                                      ctypes.c_void_p(t.data_ptr()),
                                      None if m is None else ctypes.c_void_p(m.data_ptr()),
                                      x.shape[0], g.ctypes.data_as(ctypes.c_void_p),
                                      loss.ctypes.data_as(ctypes.c_void_p), None))
        return float(loss[0]), g

    def fit(self, X, T, steps=3000, lr=2e-3, log_every=0):
        """Full-batch Adam on the library's kernels; returns the loss curve
        (sampled every log_every steps)."""
        import torch
        x, t = self._dev(X), self._dev(T)
        loss = torch.zeros(1, dtype=torch.float32, device="cuda")
        curve = []
        for k in range(steps):
            check(load().tq_mlp_train_step(self._h, ctypes.c_void_p(x.data_ptr()),
                                           ctypes.c_void_p(t.data_ptr()), None, x.shape[0],
                                           ctypes.c_float(lr), ctypes.c_void_p(loss.data_ptr()),
                                           None))
            if log_every and (k % log_every == 0 or k == steps - 1):
                torch.cuda.synchronize()
                curve.append((k, float(loss.item())))
        torch.cuda.synchronize()
        return curve

    def propose(self, features: np.ndarray) -> np.ndarray:
        """Index of the lowest-scored candidate per feature row."""
        y = self.forward(np.atleast_2d(features))
        return np.argmin(y, axis=1)


def evaluate(records, choice_fn, target):
    """Per record: (chosen ms, best ms, chosen error) for the chooser
    choice_fn(record) -> candidate index."""
    out = []
    for r in records:
        b = best_feasible(r.ms, r.err, r.status, target)
        if b < 0:
            continue
        c = choice_fn(r)
        out.append((r.ms[c] if r.status[c] == 0 else np.inf, r.ms[b], r.err[c], r.flops))
    return np.asarray(out)


# ---------------------------------------------------------------- evaluation
DEFAULT_SLICES = {1e-6: 3, 1e-8: 4, 1e-10: 5, 1e-12: 6}


def default_choice(eps):
    """The schedule the library takes without the model: the slice count the
    target asks for (3 / 4 / 5 / 6 slices for 1e-6 / 1e-8 / 1e-10 / 1e-12),
    tile width 96, no grouping."""
    s = DEFAULT_SLICES.get(eps, 5)
    for i, c in enumerate(CANDIDATES):
        if c.get("slices") == s and c.get("tile_n") == 96 and c.get("native_fill") == 0:
            return i
    raise KeyError(s)


def split(records, n_test=200):
    """Training and held-out records: the last n_test by draw order are held out."""
    return records[:-n_test], records[-n_test:]


def train(records, seed=0, steps=3000, lr=2e-3, width=64, log_every=0):
    X, T = training_arrays(records)
    net = MLP(width=width, seed=seed)
    curve = net.fit(X, T, steps=steps, lr=lr, log_every=log_every)
    return net, curve


def model_choices(net, records, eps):
    X = np.array([r.features for r in records], np.float32)
    X[:, 0] = -np.log10(eps) / 16.0
    return net.propose(X)


def regret_report(records, choices, eps):
    """Per-target comparison of a chooser with the exhaustive tuner over
    records: mean / median / p90 of ms_chosen / ms_best - 1 (feasible picks),
    share of picks whose error misses eps, and total times."""
    rg, miss, t_pick, t_best, fl = [], 0, 0.0, 0.0, 0.0
    for r, c in zip(records, choices):
        b = best_feasible(r.ms, r.err, r.status, eps)
        if b < 0:
            continue
        ok = r.status[c] == 0 and r.err[c] <= eps
        if not ok:
            miss += 1
            c = b  # the exhaustive tuner is the fallback
        rg.append(r.ms[c] / r.ms[b] - 1.0)
        t_pick += r.ms[c]
        t_best += r.ms[b]
        fl += r.flops
    rg = np.asarray(rg)
    return dict(target=eps, n=len(rg), mean_regret=float(rg.mean()),
                median_regret=float(np.median(rg)), p90_regret=float(np.percentile(rg, 90)),
                miss_rate=miss / max(len(rg), 1), ms_total=t_pick, ms_best_total=t_best,
                tflops=fl / t_pick / 1e9 if t_pick else 0.0,
                tflops_best=fl / t_best / 1e9 if t_best else 0.0)


# ---------------------------------------------------------------- dataset
def generate(n=2000, seed=4, out="tune_random.npz", reps=1, start=0, checkpoint=100,
             max_elem=1 << 21, max_blocks=20000, max_flops=2e9, log=print):
    """Run the exhaustive tuner over the random contractions of `seed` and
    save what it measured (features, per-candidate status, ms, error, flops)
    to `out`, rewriting the file every `checkpoint` records."""
    import time

    from . import workloads
    rcs = workloads.random_contractions(n, seed=seed, max_elem=max_elem, max_blocks=max_blocks,
                                        max_flops=max_flops)
    recs = []
    t0 = time.time()
    for k, rc in enumerate(rcs[start:], start):
        recs.append(tune_record(rc, seed, reps=reps))
        if (k + 1) % checkpoint == 0 or k + 1 == n:
            save(recs, out, dict(seed=seed, max_elem=max_elem, max_blocks=max_blocks,
                                 max_flops=max_flops, reps=reps))
            log("%d records, %.0f s" % (k + 1, time.time() - t0))
    return recs


def save(recs, path, meta):
    np.savez_compressed(
        path, index=np.array([r.index for r in recs], np.int64),
        features=np.array([r.features for r in recs], np.float32),
        flops=np.array([r.flops for r in recs], np.float64),
        status=np.array([r.status for r in recs], np.int8),
        ms=np.array([r.ms for r in recs], np.float32),
        err=np.array([r.err for r in recs], np.float64),
        candidates=np.array([describe(c) for c in CANDIDATES]),
        meta=np.array([repr(meta)]))


def held_out_specs(path=HELD_OUT):
    with open(path) as f:
        return json.load(f)


def load_records(path):
    d = np.load(path)
    names = [str(x) for x in d["candidates"]]
    if names != [describe(c) for c in CANDIDATES]:
        raise ValueError("dataset was made with another candidate table")
    return [TuneRecord(int(i), f.astype(np.float32), float(fl), st.astype(np.int32),
                       m.astype(np.float64), e)
            for i, f, fl, st, m, e in zip(d["index"], d["features"], d["flops"], d["status"],
                                          d["ms"], d["err"])]


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser(description="exhaustive-tuner dataset for the cost model")
    ap.add_argument("--n", type=int, default=2000)
    ap.add_argument("--seed", type=int, default=4)
    ap.add_argument("--out", default="tune_random.npz")
    ap.add_argument("--reps", type=int, default=1)
    a = ap.parse_args()
    import torque_gb300
    torque_gb300.load()
    generate(a.n, a.seed, a.out, a.reps)
