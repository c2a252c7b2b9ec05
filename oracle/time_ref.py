"""Time the reference's own CPU contract (oracle/_ref, built by build_ref.py).

TEST INFRASTRUCTURE ONLY: a measurement of the reference's CPU path on the
workloads the GPU path is benchmarked on, single-threaded as the reference
is (its matrix products go to scipy's OpenBLAS with one thread, standing in
for the BLAS the reference links through Armadillo).  It runs only where the
reference's sources were compiled; the GPU bench's reference arm times the C
restatement instead.

    python -m oracle.time_ref [--samples 8] [--index-samples 64] [--sweep 256]

Legs (one JSON line at the end):
* small: the 85-block U(1) pair (325 pairs, 1.159e7 useful flop) in full,
  both builds, median of 5;
* uneven, index stage: the reference's block matcher (block_in_range,
  block_sparse.cpp:6-175) for a seeded sample of A blocks against all 23,969
  B blocks, scaled to every A block;
* uneven, numeric stage: A blocks drawn with probability proportional to
  their useful flops (seeded, with replacement), each contracted alone with
  its partner B blocks (stride-fixed build: on a one-block A the as-is build
  throws at the second partner); the total is the importance-sampling
  estimate mean(t_i / p_i), with its standard error;
* sweep: the first n site updates of the 256-instance PEPS sweep (two
  contractions each), stride-fixed build.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if _ROOT not in sys.path:
    sys.path.insert(0, _ROOT)

from oracle import build_ref, ref  # noqa: E402
from oracle import oracle as orc  # noqa: E402


def _sub(T: orc.HostBS, idx, rng) -> orc.HostBS:
    b, e = T.begin[idx], T.end[idx]
    n = int(np.prod(e - b + 1, axis=1).sum())
    return orc.HostBS(T.dimension, b, e, rng.standard_normal(n))


def small_leg() -> dict:
    from torque_gb300 import workloads
    c = workloads.small_u1()
    A = orc.HostBS(c.A.dimension, c.A.begin, c.A.end, c.a_data)
    B = orc.HostBS(c.B.dimension, c.B.begin, c.B.end, c.b_data)
    flops = c.flops()
    out = {"useful_flop": flops}
    for v in ("asis", "fixed"):
        ts = []
        for _ in range(5):
            ref.reset_product_seconds(v)
            t = time.perf_counter()
            ref.contract(A, B, c.pairs, variant=v)
            ts.append(time.perf_counter() - t)
        s = float(np.median(ts))
        out[v] = {"s": s, "gflops": flops / s / 1e9, "product_s": ref.product_seconds(v)}
    return out


def uneven_legs(samples: int, index_samples: int) -> dict:
    from torque_gb300 import workloads
    c = workloads.uneven_u1(data=False)
    z = np.zeros(1)
    A = orc.HostBS(c.A.dimension, c.A.begin, c.A.end, z)
    B = orc.HostBS(c.B.dimension, c.B.begin, c.B.end, z)
    pa, pb = orc.match(A, B, c.pairs)
    da, db = A.block_dims, B.block_dims
    m = np.prod(da[:, :2], axis=1).astype(float)
    k = np.prod(da[:, 2:], axis=1).astype(float)
    n = np.prod(db[:, 2:], axis=1).astype(float)
    f = 2.0 * m[pa] * n[pb] * k[pa]
    fa = np.bincount(pa, weights=f, minlength=A.n_blocks)
    total = float(f.sum())
    rng = np.random.default_rng(7)
    # index stage
    idx = rng.choice(A.n_blocks, size=index_samples, replace=False)
    t = time.perf_counter()
    for i in idx:
        ref.block_in_range(c.pairs, A.begin[i], A.end[i], B.begin, B.end)
    per_call = (time.perf_counter() - t) / index_samples
    index = {"sample_a_blocks": int(index_samples), "s_per_a_block": per_call,
             "s_all_a_blocks": per_call * A.n_blocks}
    # numeric stage
    p = fa / total
    draw = rng.choice(A.n_blocks, size=samples, replace=True, p=p)
    est, rows, prod_s = [], [], 0.0
    for i in draw.tolist():
        Ai = _sub(A, [i], rng)
        Bi = _sub(B, pb[pa == i], rng)
        ref.reset_product_seconds("fixed")
        t0 = time.perf_counter()
        ref.contract(Ai, Bi, c.pairs, variant="fixed")
        ti = time.perf_counter() - t0
        prod_s += ref.product_seconds("fixed")
        est.append(ti / p[i])
        rows.append([int(i), int((pa == i).sum()), float(fa[i]), ti])
    est = np.asarray(est)
    numeric = {"draws": int(samples), "estimate_s": float(est.mean()),
               "std_error_s": float(est.std(ddof=1) / np.sqrt(samples)) if samples > 1 else None,
               "sampled_s": float(sum(r[3] for r in rows)),
               "product_share_of_sampled": prod_s / max(sum(r[3] for r in rows), 1e-30),
               "blocks": rows}
    whole = index["s_all_a_blocks"] + numeric["estimate_s"]
    return {"useful_flop": total, "pairs": int(pa.size), "index": index, "numeric": numeric,
            "estimate_s": whole, "gflops": total / whole / 1e9}


def sweep_leg(count: int) -> dict:
    from torque_gb300 import workloads
    sites = workloads.peps_sweep(256)[:count]
    flops, t_all = 0.0, 0.0
    for s in sites:
        T = orc.HostBS(np.asarray(s.T.dimension), s.T.begin, s.T.end, s.t_data)
        E1 = orc.HostBS(np.asarray(s.E1.dimension), s.E1.begin, s.E1.end, s.e1_data)
        E2 = orc.HostBS(np.asarray(s.E2.dimension), s.E2.begin, s.E2.end, s.e2_data)
        t0 = time.perf_counter()
        xb, xe, xo, xd = ref.contract(E1, T, s.pairs1, variant="fixed")
        X = orc.HostBS(np.concatenate([[s.E1.dimension[0], s.E1.dimension[3]],
                                       np.asarray(s.T.dimension)[2:]]), xb, xe, xd, offsets=xo)
        ref.contract(X, E2, s.pairs2, variant="fixed")
        t_all += time.perf_counter() - t0
        flops += workloads.useful_flops(s.E1, s.T, s.pairs1)
        flops += _pair_flops(X, E2, s.pairs2)
    return {"instances": len(sites), "s": t_all, "useful_flop": flops,
            "gflops": flops / t_all / 1e9}


def _pair_flops(A: orc.HostBS, B: orc.HostBS, pairs) -> float:
    """Useful flops of a reference-layout contraction: 2 m n k per matched pair
    with k the size of the pair's contracted intersection."""
    pa, pb = orc.match(A, B, pairs)
    pairs = np.asarray(pairs).reshape(-1, 2)
    al, bl = pairs[:, 0], pairs[:, 1]
    fa = [l for l in range(A.rank) if l not in set(al.tolist())]
    fb = [l for l in range(B.rank) if l not in set(bl.tolist())]
    da, db = A.block_dims, B.block_dims
    m = np.prod(da[pa][:, fa], axis=1).astype(float)
    n = np.prod(db[pb][:, fb], axis=1).astype(float)
    lo = np.maximum(A.begin[pa][:, al], B.begin[pb][:, bl])
    hi = np.minimum(A.end[pa][:, al], B.end[pb][:, bl])
    k = np.prod(hi - lo + 1, axis=1).astype(float)
    return float((2.0 * m * n * k).sum())


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--samples", type=int, default=8)
    ap.add_argument("--index-samples", type=int, default=64)
    ap.add_argument("--sweep", type=int, default=256)
    args = ap.parse_args()
    if build_ref.build() is None:
        raise SystemExit("the reference's sources are not here")
    blas = ref.use_blas(1, "fixed")
    ref.use_blas(1, "asis")
    out = {"cores": 1, "blas": blas or "loop", "small": small_leg()}
    if args.sweep:
        out["sweep"] = sweep_leg(args.sweep)
    if args.samples:
        out["uneven"] = uneven_legs(args.samples, args.index_samples)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
