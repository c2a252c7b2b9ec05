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
    p.add_argument("--no-sparse", action="store_true")
    p.add_argument("--no-half", action="store_true")
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
def sampled_error(c, a_dev, b_dev, C, n_largest=2, n_random=4, seed=5):
    """Accuracy on a seeded sample of output blocks: the n_largest blocks by
    useful work (the longest fused K and widest blocks, where the sliced
    accumulation is stressed most) and n_random others.  The reference is the
    sum over the block's pairs of A_i (m x k) @ B_j (k x n) in numpy float64 (A's
    blocks are [a,b | c,d] and B's [c,d | e,f], column-major, so each is that
    matrix as stored).  Reports, over the sampled blocks: the normwise error
    max|C - ref| / max|ref| per block, and the elementwise error against the
    product of magnitudes, max |C - ref| / (|A||B|) per element (the slicing
    bound itself scales with each row's and column's largest element, which
    is at least this)."""
    pa, pb = host_pairs(c)
    fl = pair_flops(c, pa, pb)
    dim, b, e, t, off = C.metadata()
    keys = {tuple(b[:, q]): q for q in range(b.shape[1])}
    groups = {}
    for q in range(pa.size):
        k = tuple(c.A.begin[pa[q], :2]) + tuple(c.B.begin[pb[q], 2:])
        groups.setdefault(k, []).append(q)
    cost = {k: sum(fl[x] for x in qs) for k, qs in groups.items()}
    order = sorted(cost, key=lambda k: -cost[k])
    pick = order[:n_largest]
    rest = order[n_largest:]
    rng = np.random.default_rng(seed)
    pick += [rest[x] for x in rng.choice(len(rest), min(n_random, len(rest)), replace=False)]
    oa, sa = block_offsets(c.A)
    ob, sb = block_offsets(c.B)
    da = c.A.block_dims
    worst, worst_elem, largest_k = 0.0, 0.0, 0
    for k in pick:
        m = int(np.prod(e[:2, keys[k]] - b[:2, keys[k]] + 1))
        n = int(np.prod(e[2:, keys[k]] - b[2:, keys[k]] + 1))
        want = np.zeros((m, n))
        mag = np.zeros((m, n))
        kf = 0
        for q in groups[k]:
            i, j = int(pa[q]), int(pb[q])
            kk = int(np.prod(da[i, 2:]))
            kf += kk
            am = a_dev[int(oa[i]):int(oa[i] + sa[i])].double().cpu().numpy().reshape((m, kk),
                                                                                     order="F")
            bm = b_dev[int(ob[j]):int(ob[j] + sb[j])].double().cpu().numpy().reshape((kk, n),
                                                                                     order="F")
            want += am @ bm
            mag += np.abs(am) @ np.abs(bm)
        largest_k = max(largest_k, kf)
        want = want.ravel(order="F")
        mag = mag.ravel(order="F")
        got = block_data(C, int(off[keys[k]]), m * n)
        d = np.abs(got - want)
        worst = max(worst, float(np.max(d) / np.max(np.abs(want))))
        worst_elem = max(worst_elem, float(np.max(d / np.maximum(mag, 1e-300))))
    return {"max_rel_err": worst, "max_elem_err_over_absAB": worst_elem, "blocks": len(pick),
            "largest_fused_k": largest_k,
            "vs": "numpy float64 block products: the %d largest output blocks by useful work and "
                  "%d random ones (seed %d); max_rel_err is max|C-ref|/max|ref| per block" %
                  (n_largest, len(pick) - n_largest, seed)}


def block_data(C, offset, n):
    """Host copy (float64) of n elements of C's device data starting at `offset`."""
    import torch
    torch.cuda.synchronize()
    dt = np.dtype(C.dtype)
    return _ptr_tensor(C.device_ptr() + dt.itemsize * offset, n, dt).cpu().double().numpy()


def _ptr_tensor(ptr, n, dtype=np.float64):
    """A CUDA tensor viewing n elements of `dtype` at device address ptr (no copy)."""
    import torch

    class _Holder:
        __cuda_array_interface__ = {"shape": (n,), "typestr": np.dtype(dtype).str,
                                    "data": (ptr, False), "version": 2}
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
    ref_config = config_dict(args, c)
    # the reference's CPU path computes in plain FP64 (no slicing)
    ref_config.update({"pairs": int(host_pairs(c)[0].size), "precision": "fp64 (host CPU)",
                       "slices": None})
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "TFLOP/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": ref_config,
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
                    "peak": fp64_peak(), "unit": "TFLOP/s",
                    "peak_source": "measured: cuBLAS DGEMM (torch.matmul float64 8192^3)"}
        else:
            ach = flops * nprod / (g_ms / 1e3) / 1e12
            roof = {"bound": "tensor", "achieved": ach, "peak": pk["bf16_sustained"],
                    "unit": "TFLOP/s", "peak_source": pk["source"] + " bf16 sustained",
                    "algorithmic": "useful flop x %d slice products per launch" % nprod}
        roof["frac"] = roof["achieved"] / roof["peak"]
        roof["kernel"] = "oz_gemm_kernel" if args.precision != "native" else "gemm_native_kernel"
        roof["kernel_ms"] = g_ms
        roof["prepare_ms"] = statistics.mean(prep_ms)
        # DRAM bytes of one launch from an ncu capture of the same workload
        tr = os.path.join(ROOT, "profiles", "dram_traffic_oz_gemm_kernel_uneven_u1.json")
        roof["traffic"] = None
        if os.path.exists(tr):
            with open(tr) as f:
                td = json.load(f)
            ent = td.get(roof["kernel"])
            if ent and ent.get("peak") == args.peak and ent.get("qmax") == args.qmax and \
                    ent.get("slices") in (None, args.slices) and args.precision == "ozaki":
                roof["traffic"] = ent["bytes_per_launch"]
                roof["traffic_source"] = "profiles/" + ent["source"]
        line["roofline"] = roof

        if not args.no_e2e:
            # right after the device-resident steps (the device-resident inputs
            # stay allocated for the legs below).  The pool's cached memory is
            # returned first: after the tile-width tuning has cycled tens of GB
            # through it, copies into buffers carved from that memory ran at a
            # quarter of the link's rate
            _lib.check(lib.tq_release_cached_memory())
            ah, bh, ch = pinned
            ah.copy_(a)
            bh.copy_(b)
            torch.cuda.synchronize()
            line["e2e"] = e2e(tq, c, ah, bh, kw, args.steps, ch)
            line["e2e"]["host_cores"] = ("%d cores local to the GPU" % len(near)) if near else \
                "unbound"
            del ah, bh, ch, pinned
            _lib.check(lib.tq_release_cached_memory())

        # accuracy on sampled output blocks (outside the timed region)
        P, _ = step()
        line["error"] = sampled_error(c, a, b, P.result)
        del P

        if not args.no_fp64:
            P, _ = step()
            line["plain_fp64"] = fp64_full(tq, c, A, B, P.result)
            # the whole sliced step (plan, operand slicing, GEMM) against the FP64
            # numeric stage alone
            line["plain_fp64"]["speedup_step_vs_fp64_numeric"] = \
                line["plain_fp64"]["numeric_ms"] / ms
            del P
        if not args.no_hbm:
            line["hbm_kernels"] = hbm_kernels(tq, c, A, B)
        if not args.no_half:
            line["half_tensor"] = half_tensor(tq, c, a, b)
        line["cpu_baseline"] = dict(zip(("value", "cores", "sample"),
                                        cpu_sample(c, a, b, args.cpu_seconds)))
        line["cpu_baseline"].update({"unit": "TFLOP/s", "kind": "port"})

        _lib.check(lib.tq_release_cached_memory())

        if not args.no_sweep:
            line["batched_sweep"] = sweep(tq)
        if not args.no_peps:
            line["peps_norm"] = peps_norm(tq)
        if not args.no_sparse:
            line["sparse_join"] = sparse_join(tq)
        if not args.no_costmodel:
            line["cost_model"] = cost_model(tq)
        print(json.dumps(line))
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


def half_tensor(tq, c, a, b, reps=3):
    """The headline contraction in half precision: the float64 inputs rounded
    to binary16, reduced layout; precision "tensor" (fp16 products on the
    tcgen05 tensor cores, fp32 accumulation, one rounding of each result) timed
    against the plain half path (FP32 SIMT accumulation) on the same tensors.
    Times: CUDA events around the numeric stage on the launching stream;
    accuracy: sampled output blocks against float64 products of the rounded
    inputs."""
    import torch
    a16, b16 = a.half(), b.half()
    A = tq.BlockSparseTensor(c.A.dimension, a16, c.A.begin.T, c.A.end.T, dtype=np.float16)
    B = tq.BlockSparseTensor(c.B.dimension, b16, c.B.begin.T, c.B.end.T, dtype=np.float16)
    out = {"dtype": "f16 operands and result, f32 accumulation"}
    for name, prec, n in (("tensor", "tensor", reps), ("native", "native", 1)):
        P = tq.ContractionPlan(A, B, c.pairs, precision=prec, layout="reduced")
        P.set_profiling(True)
        P.execute()
        P.check()
        ts, gm = [], []
        for _ in range(n):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            P.execute()
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
            gm.append(P.last_timings()[1])
        ms = statistics.median(ts)
        out[name] = {"ms": ms, "tflops": P.flops / (ms / 1e3) / 1e12,
                     "gemm_ms": statistics.median(gm)}
        if name == "tensor":
            out[name]["error"] = sampled_error(c, a16, b16, P.result)
        del P
    out["speedup_tensor_vs_native"] = out["native"]["ms"] / out["tensor"]["ms"]
    del A, B
    return out


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


def fp64_peak():
    """FP64 rate of this GPU as cuBLAS DGEMM delivers it (torch.matmul of two
    8192 x 8192 float64 matrices, best of 3, CUDA events): the roofline
    denominator of the plain FP64 form."""
    import torch
    n = 8192
    x = torch.randn(n, n, dtype=torch.float64, device="cuda")
    y = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(x, y)
    best = None
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(x, y)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    del x, y
    torch.cuda.empty_cache()
    return 2.0 * n ** 3 / (best / 1e3) / 1e12


def fp64_full(tq, c, A, B, form_result):
    """Plain FP64 (the native form) on the whole workload: the plan (symbolic
    stage) timed by wall clock, the numeric stage by CUDA events on the launching
    stream; its result compared on the device with the sliced form's."""
    import torch
    torch.cuda.synchronize()
    t = time.perf_counter()
    P = tq.ContractionPlan(A, B, c.pairs, precision="native", layout="reduced")
    torch.cuda.synchronize()
    plan_ms = (time.perf_counter() - t) * 1e3
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    P.execute()
    e1.record()
    P.check()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    ref = _ptr_tensor(P.result.device_ptr(), P.result.n_elem)
    got = _ptr_tensor(form_result.device_ptr(), form_result.n_elem)
    diff = float(torch.max(torch.abs(got - ref)) / torch.max(torch.abs(ref)))
    fl = P.flops
    del P, ref, got
    peak = fp64_peak()
    return {"value": fl / (ms / 1e3) / 1e12, "unit": "TFLOP/s", "numeric_ms": ms,
            "plan_ms": plan_ms, "useful_flop": fl, "form_vs_fp64_max_rel_diff": diff,
            "fp64_peak_tflops": peak, "frac_of_fp64_peak": fl / (ms / 1e3) / 1e12 / peak,
            "peak_source": "cuBLAS DGEMM via torch.matmul float64 8192^3, best of 3",
            "sample": "the whole workload, one contraction"}


def sweep(tq, n=256, forms=(("native", 0), ("ozaki", 5), ("bf16x3", 3)), replays=20):
    """PEPS-sweep site updates (E1 x T over (l,u), then X x E2 over (chi',r,d);
    D ~ U{4..10}, chi ~ U{16..64}, seed 3), every form run the same way: the 2n
    contractions planned once (symbolic stage, timed), then the numeric stage of
    all of them as one batch (tensor-core plans of a wave in one persistent
    launch) captured as a CUDA graph and replayed (timed with CUDA events); plus
    the reference's way for plain FP64, n sequential contract calls (symbolic +
    numeric each).  Errors of the sliced forms against the plain FP64 batch."""
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
    sequential()
    t_seq = time.perf_counter() - t
    res = {"instances": n, "sequential_fp64_ms": t_seq * 1e3}
    pk = measured_peaks()
    ref = None
    for precision, slices in forms:
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
        outs = [p.result.data().copy() for p in p2]
        ent = {"slices": slices or None, "plan_ms_once": t_plan * 1e3, "graph_ms": t_graph * 1e3,
               "graph_tflops": flops / t_graph / 1e12, "plan_plus_run_ms": (t_plan + t_graph) * 1e3,
               "graph_kernels": batch.kernels}
        if precision == "native":
            ref = outs
        else:
            nprod = slices * (slices + 1) // 2
            ent["slice_product_tflops"] = flops * nprod / t_graph / 1e12
            ent["frac_of_bf16_sustained"] = ent["slice_product_tflops"] / pk["bf16_sustained"]
            ent["max_rel_err_vs_fp64"] = max(float(np.max(np.abs(x - y)) / np.max(np.abs(y)))
                                              for x, y in zip(outs, ref))
            ent["speedup_vs_fp64_batched"] = res["native"]["graph_ms"] / (t_graph * 1e3)
            ent["speedup_plan_plus_run_vs_fp64"] = (res["native"]["plan_plus_run_ms"] /
                                                    ent["plan_plus_run_ms"])
            ent["speedup_vs_sequential_fp64"] = t_seq / t_graph
        res[precision] = ent
        res["useful_flop"] = flops
        del batch, p1, p2
    res["sequential_fp64_tflops"] = res["useful_flop"] / t_seq / 1e12
    return res


def sparse_join(tq, seed=29):
    """Element-sparse contraction (the reference's SparseTensor path): two
    random sparse tensors A[i,k,l] (4096 x 64 x 64) and B[k,l,j] (64 x 64 x
    4096), 1 % filled with N(0,1) entries (seed 29), contracted over (k,l).
    The sort-join (tq_bs_contract_elements) against the same contraction over
    one-element blocks through the block matcher (all nnz_A x nnz_B interval
    tests), both from the same device tensors, CUDA events, best of 3."""
    import torch
    from torque_gb300 import block_sparse as bs
    rng = np.random.default_rng(seed)
    da, db = (4096, 64, 64), (64, 64, 4096)
    na = int(0.01 * np.prod(da))
    nb = int(0.01 * np.prod(db))
    ia = np.sort(rng.choice(int(np.prod(da)), na, replace=False))
    ib = np.sort(rng.choice(int(np.prod(db)), nb, replace=False))
    pa = np.stack(np.unravel_index(ia, da, order="F"), 1)
    pb = np.stack(np.unravel_index(ib, db, order="F"), 1)
    A = tq.BlockSparseTensor(da, rng.standard_normal(na), pa.T, pa.T)
    B = tq.BlockSparseTensor(db, rng.standard_normal(nb), pb.T, pb.T)
    pairs = [[1, 0], [2, 1]]

    def timed(fn):
        fn()
        best = None
        for _ in range(3):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            C = fn()
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        return best, C
    t_join, S = timed(lambda: bs.contract_elements(A, B, pairs))
    t_all, R = timed(lambda: A.contract(B, pairs, layout="reduced"))
    x = _ptr_tensor(S.device_ptr(), S.n_elem)
    y = _ptr_tensor(R.device_ptr(), R.n_elem)
    diff = float(torch.max(torch.abs(x - y)) / torch.max(torch.abs(y))) \
        if S.n_elem == R.n_elem else None
    return {"nnz_a": na, "nnz_b": nb, "outputs": S.n_blocks,
            "sort_join_ms": t_join, "all_pairs_ms": t_all, "speedup": t_all / t_join,
            "max_rel_diff": diff,
            "timing": "CUDA events around the whole call (symbolic and numeric), best of 3"}


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


def cost_model(tq, n_live=200):
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
    # live: the model's proposals at 1e-10 for the held-out contractions, all of
    # them as one batch replayed as a CUDA graph, against the plain FP64 form
    # batched the same way; every result checked against its FP64 result
    specs = cm.held_out_specs()[:n_live]
    keep, prop, nat = [], [], []
    for sp in specs:
        rc = workloads.from_spec(sp)
        A, B, P = cm.plan_random(rc, 4)
        pick = cm.CANDIDATES[int(net.propose(P.features(1e-10))[0])]
        if pick["precision"] == "native":
            P.reschedule("native")
        else:
            P.reschedule(pick["precision"], slices=pick["slices"], tile_n=pick["tile_n"],
                         native_fill=pick["native_fill"])
        N = tq.ContractionPlan(A, B, rc.pairs, precision="native", layout="reduced")
        keep.append((A, B))
        prop.append(P)
        nat.append(N)

    def replay(plans, reps=10):
        b = tq.Batch(plans)
        b.graph_launch()
        b.check()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            b.graph_launch()
        e1.record()
        torch.cuda.synchronize()
        b.check()
        return e0.elapsed_time(e1) / reps, b.kernels

    ms_model, k_model = replay(prop)
    ms_fp64, k_fp64 = replay(nat)
    worst = 0.0
    for P, N in zip(prop, nat):
        x = _ptr_tensor(P.result.device_ptr(), P.result.n_elem)
        y = _ptr_tensor(N.result.device_ptr(), N.result.n_elem)
        if P.result.n_elem:
            worst = max(worst, float(torch.max(torch.abs(x - y)) / torch.max(torch.abs(y))))
    fl = sum(P.flops for P in prop)
    out["live"] = {"contractions": len(specs), "useful_flop": fl,
                   "tflops_model": fl / ms_model / 1e9, "tflops_fp64": fl / ms_fp64 / 1e9,
                   "speedup_vs_fp64": ms_fp64 / ms_model, "max_rel_err_vs_fp64": worst,
                   "graph_kernels_model": k_model, "graph_kernels_fp64": k_fp64,
                   "timing": "all held-out contractions as one batch (the model's proposals at "
                             "1e-10), CUDA-graph replay, CUDA events, mean of 10; plain FP64 "
                             "batched and replayed the same way"}
    del keep, prop, nat
    return out


def e2e(tq, c, ah, bh, kw, steps, ch=None):
    """The same contraction through the C ABI from pinned host buffers, as a
    serving loop: every step copies both inputs from the pinned host buffers
    into one of two operand buffer sets (tq_bs_set_data_async on a copy
    stream), plans, and runs tq_plan_execute_to into the pinned host result ch
    (the GEMM's epilogue writes the result over the link while it runs).  Step
    i+1's copies run on the copy engine during step i's GEMM; they are queued
    after step i's plan, whose small pageable uploads would otherwise wait
    behind them on the copy engine.  The timed region holds all `steps` steps
    and all of their copies (step 0's are exposed).  The first, untimed pass times the phases one after another.
    The last step's host result is compared bit for bit with the device
    result."""
    import torch
    an, bn = ah.numpy(), bh.numpy()
    # the link itself at this moment: torch's own copy of 4 GB of ah
    nprobe = min(ah.numel(), 1 << 29)
    probe = torch.empty(nprobe, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    tp = time.perf_counter()
    probe.copy_(ah[:nprobe], non_blocking=True)
    torch.cuda.synchronize()
    link_gbs = 8 * nprobe / (time.perf_counter() - tp) / 1e9
    del probe
    sets = [(tq.BlockSparseTensor(c.A.dimension, an, c.A.begin.T, c.A.end.T),
             tq.BlockSparseTensor(c.B.dimension, bn, c.B.begin.T, c.B.end.T)) for _ in range(2)]
    # two streams of their own: the legacy default stream would serialise the
    # copies with the contraction
    copy, comp = torch.cuda.Stream(), torch.cuda.Stream()
    ready = [torch.cuda.Event() for _ in range(2)]

    def issue_copies(k):
        sets[k][0].set_data(an, stream=copy, asynchronous=True)
        sets[k][1].set_data(bn, stream=copy, asynchronous=True)
        ready[k].record(copy)

    def plan_step(k):
        comp.wait_event(ready[k])
        return tq.ContractionPlan(sets[k][0], sets[k][1], c.pairs, stream=comp, **kw)

    def run_step(P):
        P.execute_to(ch, stream=comp)  # returns with the result in ch
        P.check(stream=comp)

    # untimed pass: the phases one after another
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    issue_copies(0)
    copy.synchronize()
    t1 = time.perf_counter()
    comp.wait_event(ready[0])
    P = tq.ContractionPlan(sets[0][0], sets[0][1], c.pairs, stream=comp, **kw)
    comp.synchronize()
    t2 = time.perf_counter()
    P.execute_to(ch, stream=comp)
    P.check(stream=comp)
    t3 = time.perf_counter()
    fl = P.flops
    del P
    # timed serving loop
    torch.cuda.synchronize()
    ts = time.perf_counter()
    issue_copies(0)
    for i in range(steps):
        # the plan first: its small pageable uploads would otherwise queue on
        # the copy engine behind the next step's 21.5 GB copies
        P = plan_step(i % 2)
        if i + 1 < steps:
            issue_copies((i + 1) % 2)  # the next step's inputs, during this step's GEMM
        run_step(P)
        if i + 1 < steps:
            del P
    torch.cuda.synchronize()
    dt = (time.perf_counter() - ts) / steps
    P.execute(stream=comp)
    comp.synchronize()
    dev = _ptr_tensor(P.result.device_ptr(), P.result.n_elem)
    same = bool(torch.equal(dev, ch[:P.result.n_elem].to("cuda", non_blocking=False)))
    del P, sets
    return {"value": fl / dt / 1e12, "unit": "TFLOP/s", "ms_per_step": dt * 1e3,
            "serial_phases_ms": {"h2d": (t1 - t0) * 1e3, "plan": (t2 - t1) * 1e3,
                                 "execute_to_host": (t3 - t2) * 1e3},
            "h2d_bytes_per_step": 8 * (ah.numel() + bh.numel()),
            "d2h_bytes_per_step": 8 * int(ch.numel()), "steps": steps,
            "host_result_equals_device_result": same,
            "h2d_link_probe_gbs": link_gbs,
            "path": "per step: tq_bs_set_data_async(pinned host) x2 on a copy stream (the "
                    "next step's during this step's GEMM) + tq_plan_create + "
                    "tq_plan_execute_to(pinned host buffer: the GEMM writes the result over "
                    "the link as it runs)"}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
