#!/usr/bin/env python
"""Benchmark: pobtaf + pobtasi throughput on one GB300 (TFLOP/s, matrices/s),
mixed precision against the FP64 form, at the stated relative error.

Workload (default): one SPD block-tridiagonal-with-arrowhead matrix, n=512
diagonal blocks of size b=512, arrowhead width a=64, float64, generated with
the seeded generator (seed 0, uniform[-1,1) blocks, diagonal-dominance
shift); total dimension 262,208.  Synthetic data of that shape stands in
for a dataset (the reference publishes none).

One step = restore the input stacks (device-to-device copy) + pobtaf +
pobtasi, in place.  The inputs (2.28 GB) are larger than L2 (129 MB), so no
L2 flush is needed between steps.  `value` is canonical TFLOP/s (LAPACK
flop conventions) over the timed K steps, with device-resident inputs, for
the headline form (`--precision`, default "mixed": FP64 storage, block
products as exact bf16 slice products on the tensor cores, 6 slices); the
FP64 drop-in is timed beside it (`compare`) and the mixed result's relative
error against the FP64 result is stated (`rel_err`).
`e2e` runs the same two calls through the public API on pinned NumPy host
arrays, host<->device copies included.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp64|mixed]
    python bench.py --impl reference     # the reference algorithm on host cores

Under torchrun each rank benchmarks an independent replica on its own GPU
(the sequential block chain does not shard): weak scaling, value summed.
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

# hardware queues for concurrent graph branches (the batch workload); must be
# set before CUDA initialises -- the library sets the same default on import
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from serinv_gb300.synthetic import flops, generate, nbytes_sweep  # noqa: E402

METRIC = "pobtaf+pobtasi TFLOP/s (n=512,b=512,a=64,FP64 storage)"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--precision", default="mixed",
                   help="fp64 | mixed | mixed:S (S = slice count 3..7); the headline form")
    p.add_argument("--compare", default="fp64,mixed:7:7",
                   help="comma-separated forms timed beside the headline (empty: none); mixed:7:7 is the "
                        "conditioning-robust form (7 slices everywhere)")
    p.add_argument("--n", type=int, default=512)
    p.add_argument("--b", type=int, default=512)
    p.add_argument("--a", type=int, default=64)
    p.add_argument("--nrhs", type=int, default=16)
    p.add_argument("--e2e-steps", type=int, default=2)
    p.add_argument("--cpu-sample-blocks", type=int, default=32)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--bare", action="store_true",
                   help="only the warm-up and timed steps (for profiler launch lists): no comparison form, "
                        "no accuracy run, no live FP64 peak, no e2e, no CPU baseline")
    p.add_argument("--workload", choices=["bta", "batched", "kappa", "autograd", "complex"], default="bta")
    p.add_argument("--cx-n", type=int, default=256)
    p.add_argument("--cx-b", type=int, default=256)
    p.add_argument("--cx-a", type=int, default=32)
    p.add_argument("--batch-count", type=int, default=256)
    p.add_argument("--batch-precision", choices=["native", "mixed"], default="native")
    p.add_argument("--ag-n", type=int, default=1024)
    p.add_argument("--ag-fd", type=int, default=64)
    return p.parse_args()


# ---------------------------------------------------------------- helpers

class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        loaded = [x for x in sm if x > 0.5 * (max(sm) if sm else 1)]
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peaks() -> dict:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


def fp64_peak_live(torch) -> float:
    """cuBLAS DGEMM 4096^3 TFLOP/s, measured now (the FP64 denominator)."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    for _ in range(2):
        a @ b
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = 1e30
    for _ in range(3):
        s.record()
        a @ b
        e.record()
        e.synchronize()
        best = min(best, s.elapsed_time(e) / 1e3)
    return 2 * n ** 3 / best / 1e12


def cpu_threads() -> int:
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)


def run_oracle_sample(n_s: int, b: int, a: int):
    """The reference algorithm (NumPy/SciPy port) on n_s blocks of the workload's shape."""
    import oracle
    m = generate(n_s, b, a, 0, seed=0)
    D, Lo, Ar, T = m.arrays()
    t0 = time.perf_counter()
    oracle.pobtaf(D, Lo, Ar, T)
    oracle.pobtasi(D, Lo, Ar, T)
    dt = time.perf_counter() - t0
    f = flops(n_s, b, a)
    return (f["pobtaf"] + f["pobtasi"]) / dt / 1e12, dt


# ---------------------------------------------------------------- reference arm

def bench_reference(args, rank: int, world: int):
    if rank != 0:
        return
    n_s = max(2, min(args.cpu_sample_blocks, args.n))
    for _ in range(args.warmup):
        run_oracle_sample(max(2, n_s // 4), args.b, args.a)
    vals, times = [], []
    for _ in range(args.steps):
        v, dt = run_oracle_sample(n_s, args.b, args.a)
        vals.append(v)
        times.append(dt)
    value = float(np.median(vals))
    cores = cpu_threads()
    sample = f"{n_s} of {args.n} diagonal blocks (b={args.b}, a={args.a}) per step, same generator"
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "TFLOP/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": float(np.median(times)) * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"BTA n={args.n} b={args.b} a={args.a} float64 (sampled {n_s} blocks)",
                   "n": args.n, "b": args.b, "a": args.a, "precision": "fp64",
                   "l2": "inputs larger than L2"},
        "cpu_baseline": {"value": value, "unit": "TFLOP/s", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- our arm

# Kernel classes bracketed by CUDA events inside the timed region: the
# FP64-pipe kernels (the roofline's subject).  The tensor-core and slicing
# kernels are launched as programmatic dependent launches; events between
# them would serialize what the timed region measures, so their breakdown
# comes from one extra profiled step after it.
TIMED_CLASSES = ("panel", "gemm")


def _timed_sweeps(torch, sg, _lib, A, A0, prec, steps, warmup, local, dist):
    """W warm-up + K timed steps (restore, pobtaf, pobtasi) with clocks and the
    FP64-pipe kernels' event times; then one step profiled in every class."""
    def step():
        for x, y in zip(A, A0):
            x.copy_(y)
        sg.pobtaf(*A, precision=prec, check_spd=False)
        sg.pobtasi(*A, precision=prec)

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = _lib.launch_count()
    _lib.profile_enable(True, classes=TIMED_CLASSES)
    stream = torch.cuda.current_stream()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(steps):
        step()
    ev1.record(stream)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    elapsed = ev0.elapsed_time(ev1) / 1e3
    launches = _lib.launch_count() - launches0
    prof = _lib.profile_read()
    _lib.profile_enable(False)
    clk = clocks.stop()
    _lib.profile_enable(True)
    step()
    torch.cuda.synchronize()
    prof_step = _lib.profile_read()
    _lib.profile_enable(False)
    if dist is not None:
        elapsed = max_over_ranks(dist, elapsed, "cuda")
    return elapsed / steps, launches, (prof, prof_step), clk


def _per_call_ms(torch, sg, A, A0, prec):
    """One extra step with CUDA events around each call: device ms of
    pobtaf and of pobtasi (median of three)."""
    s = torch.cuda.current_stream()
    out = {"pobtaf": [], "pobtasi": []}
    for _ in range(3):
        for x, y in zip(A, A0):
            x.copy_(y)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        ev[0].record(s)
        sg.pobtaf(*A, precision=prec, check_spd=False)
        ev[1].record(s)
        sg.pobtasi(*A, precision=prec)
        ev[2].record(s)
        ev[2].synchronize()
        out["pobtaf"].append(ev[0].elapsed_time(ev[1]))
        out["pobtasi"].append(ev[1].elapsed_time(ev[2]))
    return {k: float(np.median(v)) for k, v in out.items()}


def max_over_ranks(dist, value: float, device) -> float:
    """The largest of every rank's `value` (the job's time is its slowest
    replica's); every rank gets the result."""
    import torch

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(step_flops: float, world: int, per_step_s: float) -> float:
    """Whole-job TFLOP/s of `world` independent replicas, each doing one
    step of `step_flops` per `per_step_s` (the slowest replica's time)."""
    return step_flops * world / per_step_s / 1e12


# DRAM bytes (read + write) per launch of the dominant kernel, from one ncu
# capture of the same kernel at the same block sizes (the per-launch traffic
# of one block step does not depend on n): key (kernel class, precision, b, a).
# Source: profiles/launches_mixed_fp64_bench_n64_b512_a64.md (column-block
# kernel DRAM traffic, launches 70-72).
TRAFFIC_PER_LAUNCH = {
    ("panel", "mixed", 512, 64): 1.24e6 + 0.6e3,
}


def _roofline(torch, profs, prec="mixed", b=512, a=64):
    """Dominant kernel class of the profiled step; its achieved rate from the
    timed region's events when that class was timed there."""
    prof_timed, prof_step = profs
    dom = max(prof_step.items(), key=lambda kv: kv[1]["ms"]) if prof_step else (None, None)
    if dom[0] is None:
        return None
    peaks = measured_peaks()
    k, d = dom
    share = d["ms"] / sum(v["ms"] for v in prof_step.values())
    where = "one profiled step after the timed region"
    if k in prof_timed:
        d = prof_timed[k]
        where = "timed region"
    achieved = d["flops"] / (d["ms"] / 1e3) / 1e12
    if k == "gemm_tc":
        peak, src = peaks.get("bf16_tflops", 1900.0), "MEASURED_PEAKS.json bf16_tflops (of measured)"
    else:
        peak, src = fp64_peak_live(torch), "cuBLAS DGEMM 4096^3 measured live (of measured)"
    form = "mixed" if prec.startswith("mixed") else "fp64"
    traffic = TRAFFIC_PER_LAUNCH.get((k, form, b, a))
    out = {"bound": "tensor" if k == "gemm_tc" else "fp64-pipe", "kernel": k,
           "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
           "peak_source": src, "traffic": traffic,
           "traffic_note": ("DRAM bytes per launch, ncu capture of the same kernel at these block sizes "
                            "(profiles/launches_mixed_fp64_bench_n64_b512_a64.md)") if traffic else None,
           "algorithmic_bytes_per_launch": (8.0 * 3 * b * b) if k == "panel" and form == "mixed" else None,
           "avg_launch_ms": d["ms"] / d["launches"], "events_from": where,
           "share_of_device_time": share}
    # the tensor-core products: bf16 flops the MMA warps issue over their
    # event time in the profiled step, against the sustained bf16 peak
    tc = prof_step.get("gemm_tc")
    if tc and tc.get("issued"):
        pk = peaks.get("bf16_tflops_sustained", peaks.get("bf16_tflops", 1700.0))
        ach = tc["issued"] / (tc["ms"] / 1e3) / 1e12
        out["tensor"] = {"kernel": "gemm_tc", "bound": "tensor", "achieved": ach, "peak": pk,
                         "unit": "TFLOP/s (bf16 issued)", "frac": ach / pk,
                         "peak_source": "MEASURED_PEAKS.json bf16_tflops_sustained (of measured)",
                         "fp64_equivalent_tflops": tc["flops"] / (tc["ms"] / 1e3) / 1e12,
                         "launches": tc["launches"], "avg_launch_ms": tc["ms"] / tc["launches"],
                         "events_from": "one profiled step after the timed region (events around each launch)"}
    return out


def _dtype_label(prec: str) -> str:
    if prec.startswith("mixed"):
        S = int(prec.split(":")[1]) if ":" in prec else 6
        return f"f64 storage, products as {S} exact bf16 slices (tcgen05, fp32 accumulate)"
    return "f64"


def bench_ours(args, rank: int, world: int, dist):
    import torch

    import serinv_gb300 as sg
    from serinv_gb300 import _lib

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    _lib.load()
    n, b, a = args.n, args.b, args.a
    f = flops(n, b, a, args.nrhs)
    step_flops = f["pobtaf"] + f["pobtasi"]

    m = generate(n, b, a, args.nrhs, seed=0)
    A0 = [torch.from_numpy(x).cuda() for x in m.arrays()]
    A = [x.clone() for x in A0]
    prec = args.precision

    per_step, launches, prof, clk = _timed_sweeps(torch, sg, _lib, A, A0, prec, args.steps, args.warmup,
                                                  local, dist)
    value = replica_throughput(step_flops, world, per_step)

    # the comparison forms (e.g. the FP64 drop-in beside the mixed form)
    compare = {}
    if args.bare:
        args.compare, args.no_e2e, args.no_cpu_baseline = "", True, True
    for cp in [c for c in args.compare.split(",") if c and c != prec]:
        Ac = [x.clone() for x in A0]
        ps, _, pr, _ = _timed_sweeps(torch, sg, _lib, Ac, A0, cp, max(1, args.steps // 2), 1, local, dist)
        compare[cp] = {"value": step_flops * world / ps / 1e12, "unit": "TFLOP/s", "ms_per_step": ps * 1e3,
                       "kernel_profile_ms_one_step": {k: round(v["ms"], 2) for k, v in pr[1].items()}}
        del Ac

    # accuracy statement: a mixed form is compared with this GPU's FP64 path
    # (which the test suite pins to the reference at <= 1e-12)
    acc = {}
    if prec.startswith("mixed") and not args.bare:
        def rel(x, y):
            return float(torch.linalg.norm(x - y) / torch.linalg.norm(y))

        ref = [x.clone() for x in A0]
        sg.pobtaf(*ref)
        Lref = [x.clone() for x in ref]
        sg.pobtasi(*ref)
        for name, x, y in zip(("diag", "lower", "arrow", "tip"), A, ref):
            acc[name] = rel(x, y)
        acc["vs"] = "FP64 drop-in on the same inputs (relative Frobenius error per stack of the selected inverse)"
        # the factor L and the solution x of the benchmark's right-hand sides
        Lm = [x.clone() for x in A0]
        sg.pobtaf(*Lm, precision=prec)
        acc["factor"] = {nm: rel(x, y) for nm, x, y in zip(("diag", "lower", "arrow", "tip"), Lm, Lref)}
        Bh = torch.from_numpy(m.B).cuda()
        xr = Bh.clone()
        sg.pobtas(*Lref, xr, trans="N")
        sg.pobtas(*Lref, xr, trans="T")
        xm = Bh.clone()
        sg.pobtas(*Lm, xm, trans="N")
        sg.pobtas(*Lm, xm, trans="T")
        xf = Bh.clone()
        sg.pobtas_refine(*A0, *Lm, xf, iters=1)
        acc["solution"] = {"nrhs": int(Bh.shape[1]), "mixed_factor": rel(xm, xr),
                           "mixed_factor_refined_once": rel(xf, xr)}
        del ref, Lref, Lm
    else:
        acc = {"note": "FP64 path; parity with the reference pinned at <=1e-12 by the test suite"}

    roof = None if args.bare else _roofline(torch, prof, prec, b, a)
    per_call = None if args.bare else _per_call_ms(torch, sg, A, A0, prec)

    # end to end through the public API with pinned host arrays
    e2e = None
    if not args.no_e2e:
        pinned = [torch.empty(x.shape, dtype=torch.float64, pin_memory=True).numpy() for x in m.arrays()]
        work = [torch.empty(x.shape, dtype=torch.float64, pin_memory=True).numpy() for x in m.arrays()]
        for p, x in zip(pinned, m.arrays()):
            np.copyto(p, x)
        tot = 0.0
        for i in range(args.e2e_steps + 1):
            for w, p in zip(work, pinned):
                np.copyto(w, p)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            sg.pobtaf(*work, precision=prec, check_spd=False)
            sg.pobtasi(*work, precision=prec)
            dt = time.perf_counter() - t0
            if i > 0:  # first pass warms the host path
                tot += dt
        nbytes = sum(x.nbytes for x in m.arrays())
        e2e = {"value": step_flops / (tot / args.e2e_steps) / 1e12, "unit": "TFLOP/s",
               "h2d_bytes_per_step": 2 * nbytes, "d2h_bytes_per_step": 2 * nbytes,
               "ms_per_step": tot / args.e2e_steps * 1e3}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        n_s = max(2, min(args.cpu_sample_blocks, n))  # the reference arm's sample
        v, dt = run_oracle_sample(n_s, b, a)
        cpu = {"value": v, "unit": "TFLOP/s", "cores": cpu_threads(), "kind": "port",
               "sample": f"{n_s} of {n} diagonal blocks (b={b}, a={a}), {dt:.1f} s, OpenBLAS all threads"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_step * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": _dtype_label(prec), "data": "synthetic (seeded generator, seed 0)",
            "config": {"workload": f"BTA n={n} b={b} a={a} float64, pobtaf+pobtasi",
                       "n": n, "b": b, "a": a, "precision": prec,
                       "l2": "inputs larger than L2 (2.28 GB), no flush",
                       "parallelism": f"replicas x{world}"},
            "matrices_per_s": world / per_step,
            "rel_err": acc,
            "compare": compare,
            "roofline": roof,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": launches,
            "kernel_profile_one_step": prof[1],
            "per_call_ms": per_call,
            "clocks": clk,
            "hbm_bytes_algorithmic_per_step": 2 * nbytes_sweep(n, b, a),
        }
        # whole-step canonical TFLOP/s against the FP64 and bf16 tensor peaks
        pk = measured_peaks()
        line["peak_fractions"] = {
            "of_fp64_dgemm_live": value / roof["peak"] if roof and roof.get("bound") == "fp64-pipe" else None,
            "of_bf16_tensor": value / pk["bf16_tflops"] if pk.get("bf16_tflops") else None,
            "note": "canonical pobtaf+pobtasi flops per second over cuBLAS DGEMM measured live, and over the "
                    "bf16 dense tensor peak of MEASURED_PEAKS.json (of measured)"}
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- other workloads

def bench_batched(args):
    """256 uneven matrices (n ~ U{16..256}, b in {32,64,128,256}, a in {0,4,16}),
    half float32 / half float64, 4 RHS each, in one graph launch per step:
    pobtaf -> pobtas N/T -> pobtasi for every matrix.  Inputs from the NumPy
    generator (``batch_shapes``; matrix i from ``generate(..., seed=i)``).
    Stream count from the autotuner.  Value: matrices/s.  Every item's
    outputs are compared with the single-matrix FP64 GPU path on the same
    inputs (float32 items: their inputs promoted to float64)."""
    import torch

    import serinv_gb300 as sg
    from serinv_gb300 import _lib
    from serinv_gb300.batched import BatchPlan, autotune
    from serinv_gb300.synthetic import batch_shapes, generate

    torch.cuda.set_device(0)
    _lib.load()
    count = args.batch_count
    shapes = batch_shapes(count, 0)
    src, rhs0 = [], []
    tot_flops = 0.0
    for i, (n, b, a, dt) in enumerate(shapes):
        m = generate(n, b, a, 4, seed=i, dtype=dt)
        src.append(tuple(torch.from_numpy(x).cuda() for x in m.arrays()))
        rhs0.append(torch.from_numpy(m.B).cuda())
        f = flops(n, b, a, 4)
        tot_flops += f["pobtaf"] + f["pobtasi"] + f["pobtas"]
    work = [tuple(x.clone() for x in m) for m in src]
    rhs = [r.clone() for r in rhs0]
    prec = ["mixed" if args.batch_precision == "mixed" else "fp64"] * count
    t0 = time.perf_counter()
    ns, panel, split = autotune(work, rhs, precisions=prec, candidates=(16, 32, 64, 128), reps=1)
    tune_s = time.perf_counter() - t0
    k0 = _lib.launch_count()
    plan = BatchPlan(work, rhs, precisions=prec, nstreams=ns, panel_ctas=panel, tc_ksplit=split)
    kernels_per_graph = _lib.launch_count() - k0  # launches captured into the plan's graph

    def restore():
        for d, s_ in zip(work, src):
            for x, y in zip(d, s_):
                x.copy_(y)
        for d, s_ in zip(rhs, rhs0):
            d.copy_(s_)

    for _ in range(args.warmup):
        restore()
        plan.run()
    torch.cuda.synchronize()
    times = []
    for _ in range(args.steps):
        restore()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        plan.run()
        e1.record()
        e1.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    t = float(np.median(times))
    bad = int((plan.info() != 0).sum())

    # accuracy: the last replay's outputs against the single-matrix FP64 path
    worst = {"float32": 0.0, "float64": 0.0}
    for (d, x), m_src, r_src in zip(zip(work, rhs), src, rhs0):
        ref = [y.to(torch.float64).clone() for y in m_src]
        xr = r_src.to(torch.float64).clone()
        sg.pobtaf(*ref)
        L = [y.clone() for y in ref]
        sg.pobtas(*L, xr, trans="N")
        sg.pobtas(*L, xr, trans="T")
        sg.pobtasi(*ref)
        e = 0.0
        for g, r_ in list(zip(d, ref)) + [(x, xr)]:
            if r_.numel():
                nr = float(torch.linalg.norm(r_))
                e = max(e, float(torch.linalg.norm(g.to(torch.float64) - r_)) / max(nr, 1e-300))
        key = "float32" if d[0].dtype == torch.float32 else "float64"
        worst[key] = max(worst[key], e)
    line = {"metric": "batched BTA matrices/s (256 uneven, f32+f64, pobtaf+pobtas+pobtasi, 1 graph launch)",
            "value": count / t, "unit": "matrices/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t * 1e3, "higher_is_better": True, "tflops": tot_flops / t / 1e12,
            "dtype": "half f32, half " + ("f64 mixed" if args.batch_precision == "mixed" else "f64"),
            "data": "synthetic (NumPy generator, seed i for matrix i)",
            "config": {"workload": "batch of 256 uneven BTA matrices", "nstreams": ns,
                       "panel_ctas": panel or 24, "tc_ksplit": split, "autotune_s": tune_s, "not_spd": bad,
                       "hardware_queues": os.environ.get("CUDA_DEVICE_MAX_CONNECTIONS")},
            "max_rel_err_vs_single_fp64": {**worst, "vs": "single-matrix FP64 GPU path on the same inputs, "
                                                         "max over items of the relative Frobenius error of "
                                                         "each output stack and the solution"},
            "gpu_launches": kernels_per_graph}
    print(json.dumps(line), flush=True)


def bench_kappa(args):
    """Mixed vs FP64 at targeted condition numbers (kappa in 1e2, 1e5, 1e8):
    A = A0 + sigma I with sigma from Lanczos extremes of A0; the achieved
    kappa is measured (lambda_min through the FP64 factor)."""
    import torch

    import serinv_gb300 as sg
    from serinv_gb300 import _lib
    from bench_conditioning import bta_matvec, kappa_of, lanczos_extremes, shift_for_kappa
    from serinv_gb300.synthetic import generate_torch

    torch.cuda.set_device(0)
    _lib.load()
    n, b, a = args.n, args.b, args.a
    D0, Lo, Ar, T0, _ = generate_torch(n, b, a, 1, seed=0, shift=0.0)
    N = n * b + a
    lmin0, lmax0 = lanczos_extremes(lambda v: bta_matvec(D0, Lo, Ar, T0, v), N, steps=120)
    out = []
    f = flops(n, b, a)
    for kappa in (1e2, 1e5, 1e8):
        sigma = shift_for_kappa(lmin0, lmax0, kappa)
        idx = torch.arange(b, device="cuda")
        D = D0.clone()
        D[:, idx, idx] += sigma
        T = T0.clone()
        if a:
            ti = torch.arange(a, device="cuda")
            T[ti, ti] += sigma
        achieved, lmin, lmax = kappa_of(D, Lo, Ar, T)
        res = {"kappa_target": kappa, "kappa_achieved": achieved, "sigma": sigma}
        ref = [x.clone() for x in (D, Lo, Ar, T)]
        sg.pobtaf(*ref)
        # the solve: FP64 factor, and the mixed factor unrefined / refined
        # against A (16 right-hand sides, torch generator seed 1)
        g = torch.Generator(device="cuda").manual_seed(1)
        B = torch.rand((N, 16), generator=g, device="cuda", dtype=torch.float64) * 2 - 1
        A = (D, Lo, Ar, T)

        def solve(L, iters):
            x = B.clone()
            sg.pobtas_refine(*A, *L, x, iters=iters)
            r = sg.bta_matvec(*A, x, alpha=-1.0, beta=1.0, y=B.clone())
            return x, float(torch.linalg.norm(r) / torch.linalg.norm(B))

        x64, res64 = solve(ref, 0)
        Lm = [x.clone() for x in A]
        sg.pobtaf(*Lm, precision=args.precision, check_spd=False)
        sol = {"fp64": {"rel_residual": res64}}
        for iters in (0, 1, 2):
            xm, rm = solve(Lm, iters)
            sol[f"{args.precision}_refine{iters}"] = {
                "rel_residual": rm, "rel_diff_vs_fp64": float(torch.linalg.norm(xm - x64) / torch.linalg.norm(x64))}
        res["solve"] = sol
        del Lm
        sg.pobtasi(*ref)
        for prec in [p for p in args.compare.split(",") if p] + [args.precision]:
            if prec == "fp64":
                continue
            X = [x.clone() for x in (D, Lo, Ar, T)]
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            sg.pobtaf(*X, precision=prec, check_spd=False)
            sg.pobtasi(*X, precision=prec)
            e1.record()
            e1.synchronize()
            dt = e0.elapsed_time(e1) / 1e3
            res[prec] = {"tflops": (f["pobtaf"] + f["pobtasi"]) / dt / 1e12,
                         "rel_err": {nm: float(torch.linalg.norm(x - y) / torch.linalg.norm(y))
                                     for nm, x, y in zip(("diag", "lower", "arrow", "tip"), X, ref)}}
        out.append(res)
        del ref
    line = {"metric": "mixed-precision error vs conditioning (pobtaf+pobtasi against FP64; solve refined against A)",
            "config": {"n": n, "b": b, "a": a, "lanczos_A0": [lmin0, lmax0]}, "results": out}
    print(json.dumps(line), flush=True)


def bench_autograd(args):
    """logdet(A) + y^T A^{-1} y with its selected-inversion backward at
    n=1024, b=256, a=32 (FP64): forward+backward time, central finite
    differences (h=1e-6) on 64 seeded entries, and dense torch autograd at n=16."""
    import torch

    from serinv_gb300 import _lib
    from serinv_gb300.autograd import bta_logdet_quad
    from serinv_gb300.synthetic import generate_torch

    torch.cuda.set_device(0)
    _lib.load()
    n, b, a = args.ag_n, 256, 32
    D, Lo, Ar, T, y = generate_torch(n, b, a, 1, seed=0)
    params = [x.clone().requires_grad_(True) for x in (D, Lo, Ar, T)]
    yy = y[:, 0].clone().requires_grad_(True)
    for _ in range(2):
        for p in params + [yy]:
            p.grad = None
        bta_logdet_quad(*params, yy).backward()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    reps = 3
    for _ in range(reps):
        for p in params + [yy]:
            p.grad = None
        loss = bta_logdet_quad(*params, yy)
        loss.backward()
    torch.cuda.synchronize()
    t_fb = (time.perf_counter() - t0) / reps
    rng = np.random.default_rng(0)
    h = 1e-6
    worst = 0.0
    for _ in range(args.ag_fd):
        w = int(rng.integers(0, 4))
        t = params[w]
        idx = tuple(int(rng.integers(0, s_)) for s_ in t.shape)
        if w in (0, 3) and idx[-1] > idx[-2]:
            idx = idx[:-2] + (idx[-1], idx[-2])
        with torch.no_grad():
            pl = [x.detach().clone() for x in params]
            mi = [x.detach().clone() for x in params]
            pl[w][idx] += h
            mi[w][idx] -= h
            fd = (float(bta_logdet_quad(*pl, yy.detach())) - float(bta_logdet_quad(*mi, yy.detach()))) / (2 * h)
        g = float(t.grad[idx])
        worst = max(worst, abs(fd - g) / max(1.0, abs(g)))
    line = {"metric": "logdet+quadratic-form forward+backward time (selected-inversion backward)",
            "value": t_fb * 1e3, "unit": "ms", "higher_is_better": False,
            "config": {"n": n, "b": b, "a": a, "dtype": "f64"},
            "finite_difference": {"entries": args.ag_fd, "h": h, "max_rel_dev": worst}}
    print(json.dumps(line), flush=True)


def bench_complex(args):
    """complex128 Hermitian pobtaf + pobtasi (default n=256, b=256, a=32)
    through the real embedding, mixed and FP64 forms.  The metric counts the
    canonical complex flops (4x the real count); the real sweeps run on the
    embedded (n, 2b, 2a) matrix, twice those flops.  Device-resident inputs,
    CUDA events around each pobtaf+pobtasi on torch's current stream (the
    library's stream), a fresh copy of the inputs before each timed step
    (outside the events; the stacks exceed L2 after embedding)."""
    import torch

    from serinv_gb300 import _lib, pobtaf, pobtasi
    from serinv_gb300.synthetic import flops, generate_torch

    torch.cuda.set_device(0)
    _lib.load()
    n, b, a = args.cx_n, args.cx_b, args.cx_a
    src = generate_torch(n, b, a, 0, seed=0, dtype=torch.complex128)[:4]
    fl = flops(n, b, a)
    cflops = 4.0 * (fl["pobtaf"] + fl["pobtasi"])
    fr = flops(n, 2 * b, 2 * a)
    out = {}
    for prec in ("mixed", "fp64"):
        work = [x.clone() for x in src]
        times = []
        for it in range(args.warmup + args.steps):
            for w, x in zip(work, src):
                w.copy_(x)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            pobtaf(*work, precision=prec)
            pobtasi(*work, precision=prec)
            e1.record()
            torch.cuda.synchronize()
            if it >= args.warmup:
                times.append(e0.elapsed_time(e1))
        ms = float(np.median(times))
        out[prec] = {"ms": ms, "value": cflops / (ms * 1e-3) / 1e12,
                     "embedded_real_tflops": (fr["pobtaf"] + fr["pobtasi"]) / (ms * 1e-3) / 1e12,
                     "X": [x.clone() for x in work]}
    errs = {}
    for name, g, r in zip(("diag", "lower", "arrow", "tip"), out["mixed"]["X"], out["fp64"]["X"]):
        errs[name] = float(torch.linalg.vector_norm(g - r) / torch.linalg.vector_norm(r))
    line = {"metric": "complex128 pobtaf+pobtasi throughput (canonical complex flops)",
            "value": out["mixed"]["value"], "unit": "TFLOP/s", "higher_is_better": True,
            "ms_per_step": out["mixed"]["ms"], "steps": args.steps, "warmup": args.warmup,
            "dtype": "c128 (real embedding, FP64 storage; tensor-core slice products)",
            "config": {"workload": f"complex128 Hermitian BTA n={n} b={b} a={a}", "n": n, "b": b, "a": a,
                       "flops_complex": cflops, "flops_embedded_real": fr["pobtaf"] + fr["pobtasi"]},
            "embedded_real_tflops": out["mixed"]["embedded_real_tflops"],
            "compare": {"fp64": {"value": out["fp64"]["value"], "ms_per_step": out["fp64"]["ms"],
                                 "embedded_real_tflops": out["fp64"]["embedded_real_tflops"]}},
            "rel_err_mixed_vs_fp64": errs}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        bench_reference(args, rank, world)
        return
    if args.workload != "bta":
        {"batched": bench_batched, "kappa": bench_kappa, "autograd": bench_autograd,
         "complex": bench_complex}[args.workload](args)
        return
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    bench_ours(args, rank, world, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
