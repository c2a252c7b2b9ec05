#!/usr/bin/env python3
"""Block-sparse contraction throughput on GB300 (useful TFLOP/s).

Workload (default): the uneven U(1) pair A[a,b,c,d] x B[c,d,e,f] contracted over
(c,d); every leg has 33 charge sectors q = -16..16 of sizes
max(1, round(48 exp(-q^2/32))) (488 per leg): 23,969 blocks per tensor
(2.69e9 float64 each, 21.5 GB), 593,505 matched block pairs, block GEMMs from
1x1x1 to 2304x2304x2304, 7.129e13 useful flop.  Entries N(0,1) float64 from
torch's CUDA generator, seed 2 (A then B).  Reduced layout (pairs landing in the
same output block summed), FP64-level Ozaki form with 5 slices.

A step is one full contraction through the public plan/execute API (symbolic
index stage + slicing + block GEMM).  Inputs (43 GB) are far larger than L2,
so no flush is needed between steps.  Useful flops = sum over matched pairs of
2*m*n*k (no padding, no slice products).

--impl reference times the reference's CPU algorithm (the oracle port,
OpenMP over pairs on all host cores) on a bounded sample of pairs of the same
workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "block-sparse contract TFLOP/s: mixed-prec+batched vs plain FP64, rel err<=1e-10"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--precision", default="ozaki", choices=["ozaki", "bf16x3", "native"])
    p.add_argument("--slices", type=int, default=5)
    p.add_argument("--peak", type=float, default=48.0, help="sector size peak (48: full size)")
    p.add_argument("--qmax", type=int, default=16,
                   help="charges -qmax..qmax per leg (16: full size; smaller keeps only the "
                        "central, largest sectors)")
    p.add_argument("--cpu-seconds", type=float, default=10.0)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-fp64", action="store_true")
    p.add_argument("--no-sweep", action="store_true")
    p.add_argument("--no-peps", action="store_true")
    p.add_argument("--no-tune", action="store_true")
    p.add_argument("--no-hbm", action="store_true")
    p.add_argument("--no-costmodel", action="store_true")
    return p.parse_args()


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return {"hbm_gbs": d["hbm_gbs"], "bf16": d["bf16_tflops"],
                "bf16_sustained": d.get("bf16_tflops_sustained", d["bf16_tflops"]),
                "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16": 1900.0, "bf16_sustained": 1700.0, "source": "fallback"}


class Clocks:
    """nvidia-smi sampler running during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(index), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.count(",") >= 8]
        os.unlink(self.f.name)
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4)
                          if r[5 + k].strip().lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


# ---------------------------------------------------------------- host placement
def bind_near_gpu(dev):
    """Run this process on the CPU cores attached to the GPU (its PCI device's
    local CPU list), so pinned host buffers are allocated next to it: on a
    multi-socket host a buffer on the far socket more than halves host-device
    copy bandwidth.  Returns the cores, or None where the topology is not
    readable."""
    import torch
    try:
        uuid = str(torch.cuda.get_device_properties(dev).uuid)
        q = subprocess.run(["nvidia-smi", "--query-gpu=pci.bus_id", "--format=csv,noheader",
                            "-i", uuid if uuid.startswith("GPU-") else "GPU-" + uuid],
                           capture_output=True, text=True, timeout=30)
        bus = q.stdout.strip().splitlines()[0].strip().lower()
        dom, rest = bus.split(":", 1)
        path = "/sys/bus/pci/devices/%s:%s/local_cpulist" % (dom[-4:], rest)
        with open(path) as f:
            spec = f.read().strip()
        cpus = set()
        for part in spec.split(","):
            lo, _, hi = part.partition("-")
            cpus.update(range(int(lo), int(hi or lo) + 1))
        if cpus:
            os.sched_setaffinity(0, cpus)
            return sorted(cpus)
    except Exception:
        pass
    return None


# ---------------------------------------------------------------- replicas
def max_over_ranks(ms, world, device):
    """The slowest replica's time (every rank gets it): the job's step time."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_tflops(world, flops_per_replica, ms):
    """Useful TFLOP/s of the whole job: every replica contracts the full
    workload (weak scaling), all of them within the slowest one's time."""
    return world * flops_per_replica / (ms / 1e3) / 1e12


# ---------------------------------------------------------------- workload
def structure(peak, qmax=16):
    from torque_gb300 import workloads
    return workloads.uneven_u1(peak=peak, qmax=qmax, data=False)


def block_offsets(bl):
    sizes = np.prod(bl.block_dims, axis=1)
    return np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64), sizes


def host_pairs(c):
    """All matched pairs (i, j), reference order, for sector-aligned boxes."""
    from collections import defaultdict
    al, bl = c.pairs[:, 0], c.pairs[:, 1]
    byk = defaultdict(list)
    for j in range(c.B.n_blocks):
        byk[tuple(c.B.begin[j, bl])].append(j)
    pa, pb = [], []
    for i in range(c.A.n_blocks):
        for j in byk.get(tuple(c.A.begin[i, al]), ()):
            pa.append(i)
            pb.append(j)
    return np.asarray(pa, np.int64), np.asarray(pb, np.int64)


def pair_flops(c, pa, pb):
    da, db = c.A.block_dims, c.B.block_dims
    return 2.0 * np.prod(da[pa][:, :2], 1) * np.prod(db[pb][:, 2:], 1) * np.prod(da[pa][:, 2:], 1)


def compact_host(bl, offs, sizes, dev, idx):
    """HostBS of the blocks idx (in that order), data copied from the device."""
    from oracle import oracle as orc
    parts = [dev[int(offs[i]):int(offs[i] + sizes[i])].cpu().numpy() for i in idx]
    data = np.concatenate(parts) if parts else np.zeros(0)
    return orc.HostBS(bl.dimension, bl.begin[idx], bl.end[idx], data)


def cpu_sample(c, a_dev, b_dev, seconds, seed=11):
    """Time the oracle port (reference CPU algorithm) on a seeded sample of pairs
    sized to about `seconds` of work.  Returns (tflops, threads, description)."""
    from oracle import oracle as orc
    pa, pb = host_pairs(c)
    fl = pair_flops(c, pa, pb)
    rng = np.random.default_rng(seed)
    order = rng.permutation(pa.size)
    oa, sa = block_offsets(c.A)
    ob, sb = block_offsets(c.B)

    def run(budget):
        sel, tot = [], 0.0
        for q in order:
            if tot >= budget:
                break
            sel.append(q)
            tot += fl[q]
        sel = np.asarray(sel)
        ia, ra = np.unique(pa[sel], return_inverse=True)
        ib, rb = np.unique(pb[sel], return_inverse=True)
        hA = compact_host(c.A, oa, sa, a_dev, ia)
        hB = compact_host(c.B, ob, sb, b_dev, ib)
        t = time.perf_counter()
        _, _, threads = orc.pairs_baseline(hA, hB, c.pairs, ra, rb)
        dt = time.perf_counter() - t
        return tot, dt, threads, sel.size

    tot, dt, threads, n = run(2e9)
    rate = tot / max(dt, 1e-9)
    tot, dt, threads, n = run(max(rate * seconds, 2e9))
    return tot / dt / 1e12, threads, "%d of %d matched pairs (%.3g useful flop, seed %d), %.1f s" % (
        n, pa.size, tot, seed, dt)


# ---------------------------------------------------------------- validation
def sampled_error(c, a_dev, b_dev, C, n_blocks=6, max_cost=3e9, seed=5):
    """Max |C - ref| / max|ref| over a seeded sample of output blocks, ref = the
    sum over the block's pairs of A_i (m x k) @ B_j (k x n) in numpy float64
    (A's blocks are [a,b | c,d] and B's [c,d | e,f], column-major, so each is
    that matrix as stored)."""
    pa, pb = host_pairs(c)
    fl = pair_flops(c, pa, pb)
    dim, b, e, t, off = C.metadata()
    keys = {tuple(b[:, q]): q for q in range(b.shape[1])}
    groups = {}
    for q in range(pa.size):
        k = tuple(c.A.begin[pa[q], :2]) + tuple(c.B.begin[pb[q], 2:])
        groups.setdefault(k, []).append(q)
    cand = [k for k, qs in groups.items() if sum(fl[x] for x in qs) <= max_cost]
    rng = np.random.default_rng(seed)
    pick = [cand[x] for x in rng.choice(len(cand), min(n_blocks, len(cand)), replace=False)]
    oa, sa = block_offsets(c.A)
    ob, sb = block_offsets(c.B)
    da, db = c.A.block_dims, c.B.block_dims
    worst = 0.0
    for k in pick:
        m = int(np.prod(e[:2, keys[k]] - b[:2, keys[k]] + 1))
        n = int(np.prod(e[2:, keys[k]] - b[2:, keys[k]] + 1))
        want = np.zeros((m, n))
        for q in groups[k]:
            i, j = int(pa[q]), int(pb[q])
            kk = int(np.prod(da[i, 2:]))
            am = a_dev[int(oa[i]):int(oa[i] + sa[i])].cpu().numpy().reshape((m, kk), order="F")
            bm = b_dev[int(ob[j]):int(ob[j] + sb[j])].cpu().numpy().reshape((kk, n), order="F")
            want += am @ bm
        want = want.ravel(order="F")
        got = block_data(C, int(off[keys[k]]), m * n)
        worst = max(worst, float(np.max(np.abs(got - want)) / np.max(np.abs(want))))
    return worst, len(pick)


def block_data(C, offset, n):
    """Host copy of n elements of C's device data starting at `offset`."""
    import torch
    torch.cuda.synchronize()
    return _ptr_tensor(C.device_ptr() + 8 * offset, n).cpu().numpy()


def _ptr_tensor(ptr, n):
    """A float64 CUDA tensor viewing n elements at device address ptr (no copy)."""
    import torch

    class _Holder:
        __cuda_array_interface__ = {"shape": (n,), "typestr": "<f8", "data": (ptr, False),
                                    "version": 2}
    return torch.as_tensor(_Holder(), device="cuda")


# ---------------------------------------------------------------- arms
def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import torch
    c = structure(args.peak, args.qmax)
    # inputs are generated on the device (same generator as our arm) and the
    # sampled blocks copied to the host
    torch.cuda.set_device(0)
    g = torch.Generator(device="cuda")
    g.manual_seed(2)
    a = torch.randn(c.A.n_elem, dtype=torch.float64, device="cuda", generator=g)
    b = torch.randn(c.B.n_elem, dtype=torch.float64, device="cuda", generator=g)
    per_step = max(1.0, 60.0 / max(args.steps + args.warmup, 1))
    vals, desc, threads = [], "", 1
    for s in range(args.warmup + args.steps):
        v, threads, desc = cpu_sample(c, a, b, per_step, seed=100 + s)
        if s >= args.warmup:
            vals.append(v)
    value = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "TFLOP/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config_dict(args, c),
            "cpu_baseline": {"value": value, "unit": "TFLOP/s", "cores": threads, "kind": "port",
                             "sample": "per step: " + desc},
            "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def config_dict(args, c):
    return {"workload": "u1-rank4 A[a,b,c,d]xB[c,d,e,f] over (c,d), %d sectors "
                        "s_q=max(1,round(%g*exp(-q^2/32))), %d per leg, %d blocks/tensor" %
                        (2 * args.qmax + 1, args.peak, int(c.A.dimension[0]), c.A.n_blocks),
            "pairs": None, "layout": "reduced", "precision": args.precision,
            "slices": args.slices if args.precision != "native" else None,
            "l2": "inputs (2 x %.1f GB) exceed L2; no flush" % (8 * c.A.n_elem / 1e9),
            "parallelism": "replicas" if args.gpus > 1 else "single"}


def run_ours(args):
    import torch
    import torch.distributed as dist
    import torque_gb300 as tq
    from torque_gb300 import _lib

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    near = bind_near_gpu(local)
    if world > 1:
        dist.init_process_group("nccl")
    lib = tq.load()
    c = structure(args.peak, args.qmax)
    g = torch.Generator(device="cuda")
    g.manual_seed(2)
    a = torch.randn(c.A.n_elem, dtype=torch.float64, device="cuda", generator=g)
    b = torch.randn(c.B.n_elem, dtype=torch.float64, device="cuda", generator=g)
    A = tq.BlockSparseTensor(c.A.dimension, a, c.A.begin.T, c.A.end.T)
    B = tq.BlockSparseTensor(c.B.dimension, b, c.B.begin.T, c.B.end.T)
    kw = dict(precision=args.precision, slices=args.slices if args.precision != "native" else 0,
              layout="reduced")
    tune = None
    if args.precision != "native" and not args.no_tune:
        # the autotuner picks tile width and block grouping for this slice count
        # (timing only: the slice count fixes the error, measured below)
        cands = [dict(precision=args.precision, slices=args.slices, tile_n=tn, native_fill=0)
                 for tn in (96, 64, 32)]
        P0 = tq.ContractionPlan(A, B, c.pairs, **kw)
        t = time.perf_counter()
        best, ent = P0.autotune(-1.0, cands, reps=1)
        tune = {"candidates": ["n%d/g%d" % (x["tile_n"], x["native_fill"]) for x in cands],
                "ms": [e[1] for e in ent], "best": tune_name(cands[best]),
                "tuning_s": time.perf_counter() - t}
        kw.update(tile_n=cands[best]["tile_n"], native_fill=cands[best]["native_fill"])
        del P0
        torch.cuda.synchronize()
        _lib.check(lib.tq_release_cached_memory())  # the candidates' scratch back to the driver

    def step(profile=False):
        P = tq.ContractionPlan(A, B, c.pairs, **kw)
        if profile:
            P.set_profiling(True)
        P.execute()
        P.check()
        t = P.last_timings() if profile else None
        return P, t

    for _ in range(args.warmup):
        P, _t = step()
        n_out = P.result.n_elem
        del P
    torch.cuda.synchronize()
    # the pinned host buffers of the end-to-end passes, taken while host memory
    # is fresh (pinned pages allocated late in a long process can sit scattered
    # and slow the host<->device copies)
    pinned = None
    if not args.no_e2e and rank == 0:
        pinned = tuple(torch.empty(n, dtype=torch.float64, pin_memory=True)
                       for n in (c.A.n_elem, c.B.n_elem, n_out))
    if world > 1:
        dist.barrier()
    clocks = Clocks(local)
    l0 = lib.tq_debug_kernel_launches()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record()
    gemm_ms, prep_ms = [], []
    for _ in range(args.steps):
        P, t = step(profile=True)
        prep_ms.append(t[0])
        gemm_ms.append(t[1])
        flops, n_pairs = P.flops, P.n_pairs
        del P
    ev1.record()
    torch.cuda.synchronize()
    launches = lib.tq_debug_kernel_launches() - l0
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1) / args.steps
    ms = max_over_ranks(ms, world, "cuda")
    value = whole_job_tflops(world, flops, ms)

    line = {"metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (N(0,1) f64, torch CUDA generator seed 2)",
            "config": config_dict(args, c), "clocks": clk, "gpu_launches": launches}
    line["config"]["pairs"] = n_pairs
    if tune:
        line["config"]["schedule"] = tune["best"]
        line["autotune"] = tune
    line["useful_flop_per_step"] = flops

    if rank == 0:
        pk = measured_peaks()
        nprod = args.slices * (args.slices + 1) // 2 if args.precision != "native" else 1
        g_ms = statistics.mean(gemm_ms)
        if args.precision == "native":
            roof = {"bound": "fp64", "achieved": flops / (g_ms / 1e3) / 1e12,
                    "peak": 1.25, "unit": "TFLOP/s", "peak_source": "nominal FP64"}
        else:
            ach = flops * nprod / (g_ms / 1e3) / 1e12
            roof = {"bound": "tensor", "achieved": ach, "peak": pk["bf16_sustained"],
                    "unit": "TFLOP/s", "peak_source": pk["source"] + " bf16 sustained",
                    "algorithmic": "useful flop x %d slice products per launch" % nprod}
        roof["frac"] = roof["achieved"] / roof["peak"]
        roof["kernel"] = "oz_gemm_kernel" if args.precision != "native" else "gemm_native_kernel"
        roof["kernel_ms"] = g_ms
        roof["prepare_ms"] = statistics.mean(prep_ms)
        tr = os.path.join(ROOT, "profiles", "traffic.json")
        roof["traffic"] = None
        if os.path.exists(tr):
            with open(tr) as f:
                td = json.load(f)
            ent = td.get(roof["kernel"])
            if ent and ent.get("peak") == args.peak and ent.get("slices") in (None, args.slices):
                roof["traffic"] = ent["bytes_per_launch"]
        line["roofline"] = roof

        # accuracy on sampled output blocks (outside the timed region)
        P, _ = step()
        err, nb = sampled_error(c, a, b, P.result)
        line["error"] = {"max_rel_err": err, "blocks": nb,
                         "vs": "numpy float64 block products on sampled output blocks (each "
                               "block's max |C| as the scale)"}
        del P

        if not args.no_fp64:
            line["plain_fp64"] = fp64_subset(tq, c, A, a, b, kw)
        if not args.no_hbm:
            line["hbm_kernels"] = hbm_kernels(tq, c, A, B)
        line["cpu_baseline"] = dict(zip(("value", "cores", "sample"),
                                        cpu_sample(c, a, b, args.cpu_seconds)))
        line["cpu_baseline"].update({"unit": "TFLOP/s", "kind": "port"})

        if not args.no_e2e:
            # right after the device-resident steps, in the same GPU state
            ah, bh, ch = pinned
            ah.copy_(a)
            bh.copy_(b)
            del A, B, a, b
            torch.cuda.empty_cache()
            _lib.check(lib.tq_release_cached_memory())  # a fresh pool for the e2e passes
            line["e2e"] = e2e(tq, c, ah, bh, kw, 3, ch)
            line["e2e"]["host_cores"] = ("%d cores local to the GPU" % len(near)) if near else \
                "unbound"
            del ah, bh, ch, pinned
        _lib.check(lib.tq_release_cached_memory())

        if not args.no_sweep:
            line["batched_sweep"] = sweep(tq)
        if not args.no_peps:
            line["peps_norm"] = peps_norm(tq)
        if not args.no_costmodel:
            line["cost_model"] = cost_model(tq)
        print(json.dumps(line))
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


def hbm_kernels(tq, c, A, B):
    """The bandwidth-bound kernels on the full tensors: hard_transpose of A
    (21.5 GB read + written) for a leg-0-moving and a leg-0-keeping permutation,
    as GB/s of algorithmic traffic (read + write of every element) against the
    measured copy bandwidth; and the symbolic stage (pair matching over
    23,969 x 23,969 blocks, output boxes, the reduced layout's sort) as time."""
    import torch
    pk = measured_peaks()
    out = {"hbm_peak_gbs": pk["hbm_gbs"], "peak_source": pk["source"] + " copy"}
    nbytes = 2 * 8 * c.A.n_elem
    for name, perm in (("transpose_1032", [1, 0, 3, 2]), ("transpose_0213", [0, 2, 1, 3])):
        T = A.hard_transpose(perm)  # warm-up (allocates)
        del T
        torch.cuda.synchronize()
        ts, ws = [], []
        for _ in range(3):
            t = time.perf_counter()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            T = A.hard_transpose(perm)
            e1.record()
            torch.cuda.synchronize()
            ws.append(time.perf_counter() - t)
            ts.append(e0.elapsed_time(e1) / 1e3)
            del T
        dt = min(ts)
        out[name] = {"ms": dt * 1e3, "gbs": nbytes / dt / 1e9, "frac": nbytes / dt / 1e9 / pk["hbm_gbs"],
                     "bytes": nbytes, "wall_ms": min(ws) * 1e3,
                     "timing": "CUDA events around tq_bs_hard_transpose on the default stream "
                               "(its device work; the host plans the tiles first), best of 3"}
    ts = []
    for _ in range(3):
        torch.cuda.synchronize()
        t = time.perf_counter()
        P = tq.ContractionPlan(A, B, c.pairs, layout="reduced")
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t)
        del P
    out["symbolic_stage_ms"] = min(ts) * 1e3
    out["interval_tests"] = float(c.A.n_blocks) * float(c.B.n_blocks)
    return out


def tune_name(c):
    return "s%d/n%d/g%d" % (c["slices"], c["tile_n"], c["native_fill"])


def fp64_subset(tq, c, A, a, b, kw):
    """Plain FP64 (native) and the chosen form on the same sub-workload: B
    restricted to every 8th output sector (e,f), so the block-size mix of the
    full case is kept."""
    import torch
    keys = sorted({tuple(x) for x in c.B.begin[:, 2:]})
    keep = set(keys[::8])
    sel = np.asarray([j for j in range(c.B.n_blocks) if tuple(c.B.begin[j, 2:]) in keep])
    ob, sb = block_offsets(c.B)
    parts = [b[int(ob[j]):int(ob[j] + sb[j])] for j in sel]
    bsub = torch.cat(parts)
    Bs = tq.BlockSparseTensor(c.B.dimension, bsub, c.B.begin[sel].T, c.B.end[sel].T)
    res = {}
    for name, opts in (("fp64", dict(precision="native", layout="reduced")), ("form", kw)):
        P = tq.ContractionPlan(A, Bs, c.pairs, **opts)
        P.execute()
        P.check()
        torch.cuda.synchronize()
        t = time.perf_counter()
        P = tq.ContractionPlan(A, Bs, c.pairs, **opts)
        P.execute()
        P.check()
        torch.cuda.synchronize()
        dt = time.perf_counter() - t
        res[name] = P.flops / dt / 1e12
        fl = P.flops
        # compared on the device (no multi-GB host copies)
        dev = _ptr_tensor(P.result.device_ptr(), P.result.n_elem)
        if name == "fp64":
            ref = dev.clone()
        else:
            res["form_vs_fp64_max_rel_diff"] = float(torch.max(torch.abs(dev - ref)) /
                                                     torch.max(torch.abs(ref)))
        del P, dev
    del ref, Bs, bsub
    return {"value": res["fp64"], "unit": "TFLOP/s", "form_value": res["form"],
            "speedup": res["form"] / res["fp64"],
            "form_vs_fp64_max_rel_diff": res["form_vs_fp64_max_rel_diff"],
            "sample": "B restricted to every 8th (e,f) sector: %d of %d blocks, %.3g useful flop, "
                      "one full contraction each" % (sel.size, c.B.n_blocks, fl)}


def sweep(tq, n=256, forms=(("ozaki", 5), ("bf16x3", 3)), replays=20):
    """PEPS-sweep site updates (E1 x T over (l,u), then X x E2 over (chi',r,d);
    D ~ U{4..10}, chi ~ U{16..64}, seed 3): n sequential plain-FP64 contract
    calls (symbolic + numeric each, as the reference runs them) against the same
    contractions planned once and run as one replayed CUDA graph of the batched
    sliced form (one persistent GEMM launch per wave), for the FP64-level
    (Ozaki) and the FP32-level (3 x bf16) forms."""
    import torch
    from torque_gb300 import workloads
    inst = workloads.peps_sweep(n, seed=3)
    ts = []
    for s in inst:
        ts.append(tuple(tq.BlockSparseTensor(bl.dimension, torch.from_numpy(d).cuda(),
                                             bl.begin.T, bl.end.T)
                        for bl, d in ((s.T, s.t_data), (s.E1, s.e1_data), (s.E2, s.e2_data))))
    torch.cuda.synchronize()

    def sequential():
        out = []
        for s, (T, E1, E2) in zip(inst, ts):
            X = E1.contract(T, s.pairs1, layout="reduced")
            out.append(X.contract(E2, s.pairs2, layout="reduced"))
        torch.cuda.synchronize()
        return out

    sequential()
    t = time.perf_counter()
    ref = sequential()
    t_seq = time.perf_counter() - t
    res = {"instances": n, "sequential_fp64_ms": t_seq * 1e3}
    for precision, slices in forms:
        # plans: the symbolic stage once
        t = time.perf_counter()
        p1 = [tq.ContractionPlan(E1, T, s.pairs1, precision=precision, slices=slices,
                                 layout="reduced") for s, (T, E1, E2) in zip(inst, ts)]
        p2 = [tq.ContractionPlan(a.result, E2, s.pairs2, precision=precision, slices=slices,
                                 layout="reduced") for a, s, (T, E1, E2) in zip(p1, inst, ts)]
        torch.cuda.synchronize()
        t_plan = time.perf_counter() - t
        flops = sum(p.flops for p in p1 + p2)
        batch = tq.Batch(p1 + p2, waves=[0] * n + [1] * n)
        batch.graph_launch()
        batch.check()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        for _ in range(replays):
            batch.graph_launch()
        ev1.record()
        torch.cuda.synchronize()
        batch.check()
        t_graph = ev0.elapsed_time(ev1) / 1e3 / replays
        err = 0.0
        for a, b in zip(p2, ref):
            x, y = a.result.data(), b.data()
            err = max(err, float(np.max(np.abs(x - y)) / np.max(np.abs(y))))
        res["useful_flop"] = flops
        res["sequential_fp64_tflops"] = flops / t_seq / 1e12
        res[precision] = {"slices": slices, "graph_ms": t_graph * 1e3,
                          "graph_tflops": flops / t_graph / 1e12, "speedup": t_seq / t_graph,
                          "plan_ms_once": t_plan * 1e3, "graph_kernels": batch.kernels,
                          "max_rel_err_vs_fp64": err}
        del batch, p1, p2
    return res


def peps_norm(tq):
    """<psi|psi> of the 4x4 open-boundary Z2 PEPS (d=2, D=6 as 3+3, seed 1),
    contracted exactly column by column, in each precision form; the error of
    each form is against the plain FP64 form (which the tests hold within 1e-12
    of the dense FP64 oracle)."""
    from torque_gb300 import peps
    out = {"config": "4x4 OBC PEPS, Z2, d=2 (1+1), D=6 (3+3), N(0,1)/sqrt(block size) seed 1; "
                     "double layer fused to D^2=36; exact column-by-column contraction"}
    forms = (("fp64", "native", 0), ("ozaki_s5", "ozaki", 5), ("ozaki_s7", "ozaki", 7),
             ("bf16x3", "bf16x3", 3))
    for name, prec, sl in forms:
        net = peps.network(tq, 4, 6, 2, 1, precision=prec, slices=sl)
        peps.contract_norm(tq, net, 4, precision=prec, slices=sl)  # warm-up
        ts = []
        for _ in range(3):
            norm, flops, secs = peps.contract_norm(tq, net, 4, precision=prec, slices=sl)
            ts.append(secs)
        secs = min(ts)
        out[name] = {"norm": norm, "ms": secs * 1e3, "tflops": flops / secs / 1e12}
        out["useful_flop"] = flops
    ref = out["fp64"]["norm"]
    for name, _, _ in forms:
        out[name]["rel_err_vs_fp64"] = abs(out[name]["norm"] - ref) / abs(ref)
    out["timing"] = "wall time of the 15 network contractions (plan + execute each), best of 3"
    return out


def cost_model(tq, n_live=24):
    """The learned cost model: trained on the GPU (library kernels) on the
    exhaustive tuner's measurements of 1,800 random contractions (seed 4),
    evaluated on the 200 held-out ones: regret against exhaustive tuning and gain
    over the default schedule, from the stored measurements; then live runs of
    the model's proposal at 1e-10 on n_live held-out contractions."""
    import torch
    from torque_gb300 import costmodel as cm, workloads
    recs = cm.load_records(cm.DATASET)
    train, test = cm.split(recs)
    t = time.perf_counter()
    net, curve = cm.train(train, steps=3000, log_every=1000)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t
    out = {"records": len(recs), "train": len(train), "held_out": len(test),
           "candidates": len(cm.CANDIDATES), "train_s": t_train, "loss_curve": curve,
           "mlp": "32 -> 64 -> 64 -> %d, ReLU, FP32, full-batch Adam, 3000 steps" %
                  len(cm.CANDIDATES)}
    rep = {}
    for eps in cm.TARGETS:
        m = cm.regret_report(test, cm.model_choices(net, test, eps), eps)
        d = cm.regret_report(test, [cm.default_choice(eps)] * len(test), eps)
        rep["%g" % eps] = {"model": m, "default": d,
                           "gain_over_default": d["ms_total"] / m["ms_total"]}
    out["held_out"] = rep
    # live: the proposal at 1e-10 run and checked against plain FP64 on the device
    specs = cm.held_out_specs()
    live_fl, live_ms, live_fp64, worst = 0.0, 0.0, 0.0, 0.0
    for sp in specs[:n_live]:
        rc = workloads.from_spec(sp)
        A, B, P = cm.plan_random(rc, 4)
        f = P.features(1e-10)
        pick = int(net.propose(f)[0])
        best, ent = P.autotune(1e-10, [cm.CANDIDATES[pick], dict(precision="native")], reps=3)
        if ent[0][2] > 1e-10 or ent[0][0] != 0:  # the tuner is the fallback
            best, ent2 = P.autotune(1e-10, cm.CANDIDATES, reps=1)
            ent[0] = ent2[best]
        live_fl += P.flops
        live_ms += ent[0][1]
        live_fp64 += ent[1][1]
        worst = max(worst, ent[0][2])
        del A, B, P
    out["live"] = {"contractions": min(n_live, len(specs)), "useful_flop": live_fl,
                   "tflops_model": live_fl / live_ms / 1e9, "tflops_fp64": live_fl / live_fp64 / 1e9,
                   "speedup_vs_fp64": live_fp64 / live_ms, "max_rel_err_vs_fp64": worst,
                   "timing": "numeric stage, fastest of 3 after a warm-up, CUDA events"}
    return out


def e2e(tq, c, ah, bh, kw, steps, ch=None):
    """The same contraction through the C ABI from pinned host buffers: H2D of
    both inputs, contraction, D2H of the whole result (into ch), every step."""
    import ctypes
    import torch
    from torque_gb300 import _lib
    an, bn = ah.numpy(), bh.numpy()
    times, phases = [], []
    for s in range(steps + 1):
        torch.cuda.synchronize()
        t = time.perf_counter()
        A = tq.BlockSparseTensor(c.A.dimension, an, c.A.begin.T, c.A.end.T)
        B = tq.BlockSparseTensor(c.B.dimension, bn, c.B.begin.T, c.B.end.T)
        t1 = time.perf_counter()  # creation from host memory returns after its copy
        P = tq.ContractionPlan(A, B, c.pairs, **kw)
        P.execute()
        P.check()
        C = P.result
        if ch is None:
            ch = torch.empty(C.n_elem, dtype=torch.float64, pin_memory=True)
        t2 = time.perf_counter()
        _lib.check(_lib.load().tq_bs_copy_data(C.handle, ctypes.c_void_p(ch.data_ptr()),
                                               _lib.TQ_MEM_HOST, None))
        t3 = time.perf_counter()
        dt = t3 - t
        fl = P.flops
        del P, C, A, B
        if s > 0:  # the first pass pins pages and warms the allocator
            times.append(dt)
            phases.append((t1 - t, t2 - t1, t3 - t2))
    dt = statistics.median(times)
    ph = phases[times.index(dt)] if dt in times else phases[0]
    return {"value": fl / dt / 1e12, "unit": "TFLOP/s", "ms_per_step": dt * 1e3,
            "phases_ms": {"h2d_create": ph[0] * 1e3, "plan_execute": ph[1] * 1e3,
                          "d2h": ph[2] * 1e3},
            "h2d_bytes_per_step": 8 * (ah.numel() + bh.numel()),
            "d2h_bytes_per_step": 8 * int(ch.numel()), "steps": steps,
            "path": "tq_bs_create(host) x2 + tq_plan_create/execute + tq_bs_copy_data(host)"}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
