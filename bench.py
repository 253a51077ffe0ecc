"""Benchmark of the execute hot path: batched fftwf c2c, N = 4096 x 65536.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload c2c4096|c2c1024d|r2c16384|c2c1m|c3d512|r2c2d8192]

One step = one fftwf_execute_dft of the whole batch (65536 transforms of 4096
complex64 points, 2 GiB in, 2 GiB out, both larger than the 129 MB L2 so
every step streams from HBM).  Reported on one JSON line:

  value      Gflop/s, 5 N log2 N per transform (libbench2/mflops.c:21-27),
             device-resident arrays, CUDA events around K steps on the
             launching stream
  e2e        the same metric through fftwf_execute_dft on page-locked HOST
             arrays (fftwf_malloc): host->device copy, passes, device->host
             copy all inside the timed region
  roofline   HBM: algorithmic bytes (one read + one write of the batch) per
             launch / average launch time, against MEASURED_PEAKS.json
  cpu_baseline  the reference algorithm on the host cores (bounded sample)

--impl reference times the reference's CPU implementation on the host cores:
oracle/_ref (the reference FFTW, codelet-free) when it was built here, else
the oracle's C restatement; all host threads; a bounded sample per step.
Under torchrun, every rank runs the whole batch on its own GPU (weak
scaling, no collective: the transforms are independent) and rank 0 prints.
"""
from __future__ import annotations

import argparse
import datetime
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (kind, shape, howmany, prec, inplace)
    "c2c4096": ("c2c", [4096], 65536, "f", False),
    "c2c256": ("c2c", [256], 1 << 20, "f", False),
    "c2c65536": ("c2c", [65536], 4096, "f", False),
    "c2c1024d": ("c2c", [1024], 4096, "d", False),
    "r2c16384": ("r2c", [16384], 16384, "f", False),
    "c2c1m": ("c2c", [1 << 20], 64, "f", False),
    "c3d512": ("c2c", [512, 512, 512], 1, "f", True),
    "r2c2d8192": ("r2c", [8192, 8192], 1, "f", False),
    "r2r4096": ("r2r", [4096], 65536, "f", False),     # REDFT10 (DCT-II)
}
R2R_KIND = 5   # fftw_r2r_kind REDFT10 of the r2r workloads
METRIC = "FFT Gflop/s (5N log2N/t) & HBM %peak: split-FP16 TC vs FP32, rel err<=1e-6"


def smooth_set(lo=60, hi=60000):
    """{2^a 3^b 5^c 7^d} within [lo, hi]."""
    out = set()
    a = 1
    while a <= hi:
        b = a
        while b <= hi:
            c = b
            while c <= hi:
                d = c
                while d <= hi:
                    if d >= lo:
                        out.add(d)
                    d *= 7
                c *= 5
            b *= 3
        a *= 2
    return sorted(out)


def primes_in(lo, hi):
    return [p for p in range(max(2, lo), hi + 1) if all(p % q for q in range(2, int(p ** 0.5) + 1))]


def uneven_lengths(rng, count, max_pow2=16, max_smooth=60000, max_prime=4093):
    """Seeded uneven batch: 60% powers of two 2^6..2^max_pow2 (log-uniform),
    30% smooth composites 2^a3^b5^c7^d in [60, max_smooth], 10% primes in
    [17, max_prime]."""
    sm = smooth_set(60, max_smooth)
    pr = primes_in(17, max_prime)
    out = []
    for u in rng.random(count):
        if u < 0.6:
            out.append(1 << int(rng.integers(6, max_pow2 + 1)))
        elif u < 0.9:
            out.append(int(sm[int(rng.integers(0, len(sm)))]))
        else:
            out.append(int(pr[int(rng.integers(0, len(pr)))]))
    return out


def flops_per_step(kind, shape, howmany):
    n = math.prod(shape)
    f = 5.0 * n * math.log2(n) * howmany
    return f / 2 if kind in ("r2c", "c2r", "r2r") else f


def bytes_per_step(kind, shape, howmany, prec):
    n = math.prod(shape)
    cs = 8 if prec == "f" else 16
    if kind == "c2c":
        return 2 * n * cs * howmany
    if kind == "r2r":
        return n * cs * howmany
    nc = n // shape[-1] * (shape[-1] // 2 + 1)
    return (n * cs // 2 + nc * cs) * howmany


def aggregate(ms_local, ws, flops_per_rank, device):
    """Whole-job throughput: the slowest rank's time (max over ranks, the
    only collective; the transforms themselves never cross ranks) and the
    flops of all ranks over it.  Returns (ms_max, Gflop/s)."""
    ms = float(ms_local)
    if ws > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, flops_per_rank * ws / (ms * 1e-3) / 1e9


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples (every 20 ms) of the SM clock and throttle reasons
    around the timed region.  The sampler is running before the region starts;
    the summary uses the samples whose timestamps fall inside the region, or
    the two nearest ones when the region is shorter than the interval."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        fd, self.path = tempfile.mkstemp(prefix="fftw_gb300_clocks_", suffix=".csv")
        os.close(fd)
        self.t0 = self.t1 = None

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=timestamp,clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "20"], stdout=self.f, stderr=subprocess.DEVNULL)
            deadline = time.time() + 3.0
            while time.time() < deadline and os.path.getsize(self.path) == 0:
                time.sleep(0.01)
        except Exception:
            self.proc = None
        self.t0 = datetime.datetime.now()
        return self

    def __exit__(self, *a):
        self.t1 = datetime.datetime.now()
        if self.proc:
            time.sleep(0.05)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        try:
            rows = []
            for r in open(self.path).read().strip().splitlines():
                f = [x.strip() for x in r.split(",")]
                if len(f) < 7:
                    continue
                rows.append((datetime.datetime.strptime(f[0], "%Y/%m/%d %H:%M:%S.%f"), f))
            inside = [f for t, f in rows if self.t0 <= t <= self.t1]
            nearest = not inside
            if nearest:
                mid = self.t0 + (self.t1 - self.t0) / 2
                inside = [f for _, f in sorted(rows, key=lambda tf: abs((tf[0] - mid).total_seconds()))[:2]]
            sm = [float(f[1]) for f in inside]
            mx = [float(f[2]) for f in inside]
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            reasons = sorted({names[i] for f in inside for i in range(4) if f[3 + i] == "Active"})
            return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": reasons,
                    "samples": len(inside), "window_ms": round((self.t1 - self.t0).total_seconds() * 1e3, 1),
                    "samples_are": "nearest to the timed region (shorter than the 20 ms interval)" if nearest
                    else "inside the timed region"}
        except Exception:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        finally:
            try:
                os.unlink(self.path)
            except OSError:
                pass


def committed_traffic(workload):
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", f"{workload}_traffic.json")
    try:
        with open(path) as f:
            return json.load(f).get("dram_bytes_per_launch")
    except Exception:
        return None


def cpu_sample(workload, nthreads, budget_s=10.0, prefer_ref=True):
    """Time the reference algorithm on the host: oracle/_ref (reference FFTW)
    if it was built on this machine, else the oracle's C restatement."""
    import numpy as np
    from oracle.oracle import Reference, Restatement, ref_available
    kind, shape, howmany, prec, _ = WORKLOADS[workload]
    n = math.prod(shape)
    per = max(1, min(howmany, int(2 ** 22 // n)))   # ~32 MB of complex64 per call
    rng = np.random.default_rng(0)
    cdt = np.complex64 if prec == "f" else np.complex128
    use_ref = prefer_ref and ref_available()
    if kind == "c2c":
        x = (rng.standard_normal(per * n) + 1j * rng.standard_normal(per * n)).astype(cdt)
    else:
        x = rng.standard_normal(per * n).astype(np.float32 if prec == "f" else np.float64)
    if kind == "r2r":
        # the codelet-free reference plans no even-length r2r: the oracle's
        # O(n log n) restatement (real DFT of the symmetric extension)
        use_ref = False
    if use_ref:
        R = Reference(prec)
        fn = (lambda: R.c2c(x, shape, -1, nthreads=nthreads)) if kind == "c2c" else (lambda: R.r2c(x, shape, nthreads=nthreads))
        kind_s = "reference"
    else:
        R = Restatement()
        if kind == "c2c":
            fn = lambda: R.c2c(x, shape, -1, prec, nthreads)
        elif kind == "r2r":
            fn = lambda: R.r2r_fast(x, n, R2R_KIND, prec, nthreads)
        else:
            fn = lambda: R.r2c(x, shape, prec, nthreads)
        kind_s = "port"
    fn()
    t0 = time.perf_counter()
    calls = 0
    while True:
        fn()
        calls += 1
        if time.perf_counter() - t0 >= budget_s:
            break
    dt = time.perf_counter() - t0
    val = flops_per_step(kind, shape, per) * calls / dt / 1e9
    return {"value": round(val, 3), "unit": "Gflop/s", "cores": nthreads, "kind": kind_s,
            "sample": f"{calls} calls x {per} transforms of {'x'.join(map(str, shape))} ({'reference FFTW, codelet-free build' if use_ref else 'oracle C restatement'}), {dt:.1f} s"}


def run_reference_arm(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    kind, shape, howmany, prec, _ = WORKLOADS[args.workload]
    nthreads = os.cpu_count() or 1
    vals = []
    base = None
    for i in range(args.warmup + args.steps):
        r = cpu_sample(args.workload, nthreads, budget_s=max(2.0, 20.0 / max(1, args.steps)))
        if i >= args.warmup:
            vals.append(r["value"])
            base = r
    v = statistics.mean(vals)
    n = math.prod(shape)
    out = {
        "metric": METRIC, "value": round(v, 3), "unit": "Gflop/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(flops_per_step(kind, shape, howmany) / (v * 1e9) * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if prec == "f" else "f64", "data": "synthetic",
        "config": {"workload": f"{args.workload}: {kind} {'x'.join(map(str, shape))} x {howmany} ({'float' if prec == 'f' else 'double'})",
                   "sample_per_step": base["sample"]},
        "cpu_baseline": dict(base, value=round(v, 3)),
        "e2e": {"value": round(v, 3), "unit": "Gflop/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def run_ours(args):
    import numpy as np
    import torch
    import fftw3_gb300 as g
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    from fftw3_gb300 import build as b
    b.build()
    lib = g.load()
    kind, shape, howmany, prec, inplace = WORKLOADS[args.workload]
    if args.howmany:
        howmany = args.howmany
    n = math.prod(shape)
    cdt = torch.complex64 if prec == "f" else torch.complex128
    rdt = torch.float32 if prec == "f" else torch.float64
    gen = torch.Generator(device="cuda").manual_seed(1234 + rank)
    nc = n // shape[-1] * (shape[-1] // 2 + 1)
    if kind == "c2c":
        xin = torch.randn(howmany * n, dtype=cdt, device="cuda", generator=gen)
        yout = xin if inplace else torch.empty_like(xin)
        p = g.plan_many_dft(shape, howmany, xin.data_ptr(), yout.data_ptr(), -1, g.FFTW_ESTIMATE, prec)
    elif kind == "r2r":
        xin = torch.randn(howmany * n, dtype=rdt, device="cuda", generator=gen)
        yout = torch.empty_like(xin)
        p = g.plan_many_r2r(shape, howmany, xin.data_ptr(), yout.data_ptr(), [R2R_KIND] * len(shape),
                            g.FFTW_ESTIMATE, prec)
    else:
        xin = torch.randn(howmany * n, dtype=rdt, device="cuda", generator=gen)
        yout = torch.empty(howmany * nc, dtype=cdt, device="cuda")
        p = g.plan_many_dft_r2c(shape, howmany, xin.data_ptr(), yout.data_ptr(), g.FFTW_ESTIMATE, prec)
    stream = torch.cuda.current_stream()
    p.set_stream(stream.cuda_stream)
    p.set_async(True)

    def step():
        if kind == "c2c":
            p.execute_dft(xin.data_ptr(), yout.data_ptr())
        elif kind == "r2r":
            p.execute_r2r(xin.data_ptr(), yout.data_ptr())
        else:
            p.execute_dft_r2c(xin.data_ptr(), yout.data_ptr())

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    l0 = g.launch_count()
    # one event between consecutive steps: the total over K steps is the
    # reported time; the per-step spread (min, median) is reported beside it
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        evs[0].record(stream)
        for i in range(args.steps):
            step()
            evs[i + 1].record(stream)
        torch.cuda.synchronize()
    ms = evs[0].elapsed_time(evs[-1])
    per_step = sorted(evs[i].elapsed_time(evs[i + 1]) for i in range(args.steps))
    launches = g.launch_count() - l0
    fl = flops_per_step(kind, shape, howmany)
    ms, value = aggregate(ms, ws, fl * args.steps, "cuda")
    ms_step = ms / args.steps

    # accuracy of this run on a sample of transforms, against the oracle
    # (in-place or very long single transforms: forward/backward round trip)
    from oracle.oracle import Restatement, rel_l2
    k = min(howmany, 64) if n <= 65536 else 1
    rt_err = None
    if kind == "c2c" and (inplace or n > (1 << 20)):
        x0 = torch.randn(howmany * n, dtype=cdt, device="cuda", generator=gen)
        xin.copy_(x0)
        pb = g.plan_many_dft(shape, howmany, yout.data_ptr(), xin.data_ptr(), 1, g.FFTW_ESTIMATE, prec)
        pb.set_stream(stream.cuda_stream)
        step()
        torch.cuda.synchronize()
        if inplace and prec == "f" and howmany * n <= (1 << 28):
            # the forward transform of the whole array against the oracle
            # (a round trip alone cannot see errors that cancel, such as a
            # wrong axis order or a twiddle conjugated on both sides)
            yf = yout.cpu().numpy()
            ref = Restatement().c2c(x0.cpu().numpy().astype(np.complex128), shape, -1, "d", os.cpu_count() or 1)
            err = float(np.linalg.norm((yf.astype(np.complex128) - ref.ravel())) / np.linalg.norm(ref))
            k = howmany
            del yf, ref
        else:
            k = 0
        pb.execute_dft(yout.data_ptr(), xin.data_ptr())
        torch.cuda.synchronize()
        rt_err = float(torch.linalg.vector_norm(xin / n - x0) / torch.linalg.vector_norm(x0))
        if not k:
            err = rt_err
    else:
        # k transforms spread evenly over the batch (every CTA of a persistent
        # kernel walks many tiles: the sample covers late tiles too)
        sel = torch.from_numpy(np.linspace(0, howmany - 1, k).astype(np.int64)).cuda()
        xs = xin.view(howmany, n)[sel].cpu().numpy()
        step()
        torch.cuda.synchronize()
        no = nc if kind == "r2c" else n
        ys = yout.view(howmany, no)[sel].cpu().numpy()
        rdt, cdt_ = (np.float64, np.complex128) if prec == "f" else (np.longdouble, np.clongdouble)
        if kind == "r2r":
            ref = Restatement().r2r_fast(xs.astype(rdt), n, R2R_KIND, "d" if prec == "f" else "l",
                                         os.cpu_count() or 1)
        elif kind == "c2c":
            ref = Restatement().c2c(xs.astype(cdt_), shape, -1, "d" if prec == "f" else "l", os.cpu_count() or 1)
        else:
            ref = Restatement().r2c(xs.astype(rdt), shape, "d" if prec == "f" else "l", os.cpu_count() or 1)
        err = rel_l2(ys, ref)

    # the split-FP16 tensor-core form on the same batch, beside the FP32 form
    tc = None
    if kind == "c2c" and prec == "f" and not args.no_tc:
        tc = run_tc_form(g, shape, howmany, xin, yout, stream, args, fl, ws, gen)

    # dominant kernel: per-launch time from the events (one pass per step for
    # single-pass plans; per-pass share otherwise is taken from the ncu list)
    npass = len(p.passes())
    hbm, src = peaks()
    alg = bytes_per_step(kind, shape, howmany, prec)
    achieved = alg / (ms_step * 1e-3) / 1e9
    roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
            "frac": round(achieved / hbm, 4), "traffic": committed_traffic(args.workload),
            "peak_source": src, "passes_per_step": npass,
            "note": "achieved = algorithmic bytes per step (one read + one write) / step time"}

    # e2e: host arrays through the public API
    e2e = None
    if not args.no_e2e and rank == 0:
        e2e = run_e2e(lib, g, kind, shape, howmany, prec, inplace, args)

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        cpu = cpu_sample(args.workload, os.cpu_count() or 1, budget_s=12.0, prefer_ref=True)

    if rank == 0:
        out = {
            "metric": METRIC, "value": round(value, 2), "unit": "Gflop/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 4),
            "ms_step_min": round(per_step[0], 4), "ms_step_median": round(statistics.median(per_step), 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if prec == "f" else "f64", "data": "synthetic",
            "config": {"workload": f"{args.workload}: fftw{'f' if prec == 'f' else ''}_plan_many_"
                                   f"{'r2r REDFT10' if kind == 'r2r' else 'dft_r2c' if kind == 'r2c' else 'dft'} "
                                   f"{'x'.join(map(str, shape))} x {howmany}, {'in place' if inplace else 'out of place'}, FFTW_ESTIMATE",
                       "inputs": "N(0,1) from torch.Generator seed 1234+rank; batch larger than L2 (no flush needed)",
                       "form": "plain FP32 CUDA-core" if prec == "f" else "FP64",
                       ("rel_l2_vs_fp64_oracle" if k else "roundtrip_rel_l2"): err, "oracle_sample_transforms": k,
                       **({"roundtrip_rel_l2": rt_err} if rt_err is not None and k else {})},
            "gbs": round(achieved, 1),
            "roofline": roof,
            "gpu_launches": launches,
            "clocks": clk.summary(),
            "e2e": e2e,
            "cpu_baseline": cpu,
            "tc_form": tc,
        }
        if prec == "d":
            # double precision is bound by the FP64 units, not HBM: the rate of
            # this run (5 N log2 N convention) against the measured FP64 FMA peak
            fp64 = lib.fftw_gb300_fp64_fma_gflops()
            out["fp64_roofline"] = {"bound": "fp64", "achieved": round(value, 1), "peak": round(fp64, 1),
                                    "unit": "GFLOP/s", "frac": round(value / fp64, 4) if fp64 > 0 else None,
                                    "peak_source": "measured in this run (FP64 FMA loop, CUDA events)",
                                    "note": "achieved counts 5 N log2 N flops per transform, not the FP64 "
                                            "instructions the kernel executes"}
        print(json.dumps(out))
    if ws > 1:
        torch.distributed.destroy_process_group()


def run_uneven(args):
    """10,000 independent fftwf c2c forward transforms of seeded uneven
    lengths as one plan set: one work-queue kernel in one CUDA graph launch
    per step, the set planned with FFTW_MEASURE (the set tuner picks each
    length's item body, radix order, prime algorithm and long split and keeps
    them in wisdom); beside it the set with the planner's defaults and the
    same plans executed one after another."""
    import ctypes
    import numpy as np
    import torch
    import fftw3_gb300 as g
    from fftw3_gb300 import build as b
    from oracle.oracle import Restatement, rel_l2
    b.build()
    lib = g.load()
    torch.cuda.set_device(0)
    count = args.howmany or 10000
    lengths = uneven_lengths(np.random.default_rng(2024), count)
    offs = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64)
    gen = torch.Generator(device="cuda").manual_seed(1234)
    xin = torch.randn(int(offs[-1]), dtype=torch.complex64, device="cuda", generator=gen)
    yout = torch.zeros_like(xin)
    es = xin.element_size()
    t0 = time.perf_counter()
    plans = [g.plan_many_dft([int(n)], 1, xin.data_ptr() + int(offs[i]) * es, yout.data_ptr() + int(offs[i]) * es,
                             -1, g.FFTW_ESTIMATE, "f") for i, n in enumerate(lengths)]
    plan_s = time.perf_counter() - t0
    arr = (ctypes.c_void_p * len(plans))(*[p.ptr for p in plans])
    lib.fftwf_gb300_plan_set.restype = ctypes.c_void_p
    lib.fftwf_gb300_plan_set.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_uint]
    lib.fftwf_gb300_execute_set.argtypes = [ctypes.c_void_p]
    lib.fftwf_gb300_set_stream_set.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    lib.fftwf_gb300_set_info.argtypes = [ctypes.c_void_p] + [ctypes.POINTER(ctypes.c_int)] * 5
    stream = torch.cuda.current_stream()
    fl = sum(5.0 * n * math.log2(n) for n in lengths if n > 1)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def make_set(flags):
        t0 = time.perf_counter()
        s = lib.fftwf_gb300_plan_set(len(plans), arr, flags)
        if not s:
            raise RuntimeError("plan set failed: " + g.last_error())
        lib.fftwf_gb300_set_stream_set(s, stream.cuda_stream, 1)
        return s, time.perf_counter() - t0

    def time_set(s):
        for _ in range(args.warmup):
            lib.fftwf_gb300_execute_set(s)
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            lib.fftwf_gb300_execute_set(s)
        ev1.record(stream)
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1) / args.steps

    # the planner's defaults, then the set tuner's choices (every length
    # timed on scratch arrays within a 120 s limit, kept in wisdom)
    s_est, est_build_s = make_set(g.FFTW_ESTIMATE)
    if args.no_tune:
        s, set_s, ms_est = s_est, est_build_s, None
    else:
        ms_est = time_set(s_est)
        lib.fftwf_gb300_destroy_set.argtypes = [ctypes.c_void_p]
        lib.fftwf_gb300_destroy_set(s_est)
        lib.fftwf_set_timelimit(120.0)
        s, set_s = make_set(g.FFTW_MEASURE)
        lib.fftwf_set_timelimit(-1.0)
    info = [ctypes.c_int() for _ in range(5)]
    lib.fftwf_gb300_set_info(s, *[ctypes.byref(v) for v in info])
    # queue kernels a graph launch runs: the last item in queue order is in
    # the large-tile queue when the set has one
    it = [ctypes.c_int() for _ in range(6)]
    lib.fftwf_gb300_set_item_info.argtypes = [ctypes.c_void_p, ctypes.c_int] + [ctypes.POINTER(ctypes.c_int)] * 6
    lib.fftwf_gb300_set_item_info(s, info[0].value - 1, *[ctypes.byref(v) for v in it])
    kernels_per_step = 2 if it[4].value == 1 else 1
    wis = ctypes.string_at(lib.fftwf_export_wisdom_to_string()).decode()
    tuned = wis.count('"set p4 n')
    # what the set tuner chose: fields variant tb load store n1 groups order
    choices = {"register_body": 0, "rader": 0, "bluestein": 0, "other_split": 0, "radix_order": 0, "tile": 0}
    for line in wis.splitlines():
        if '"set p4 n' not in line:
            continue
        f = [int(v, 16) for v in line.split('"')[2].replace(")", "").replace("#x", "").split()]
        f = [v - (1 << 32) if v >= 1 << 31 else v for v in f]
        choices["register_body"] += f[0] == 0
        choices["rader"] += f[0] == 5
        choices["bluestein"] += f[0] == 3
        choices["other_split"] += f[4] != 0
        choices["radix_order"] += f[6] != 0
        choices["tile"] += f[1] != 0
    with ClockSampler(0) as clk:
        ms = time_set(s)
    # the same plans one after another (async, one launch or more each)
    for p in plans:
        p.set_stream(stream.cuda_stream)
        p.set_async(True)
    for p in plans:
        p.execute()
    torch.cuda.synchronize()
    l0 = g.launch_count()
    ev0.record(stream)
    for _ in range(max(1, args.steps // 4)):
        for p in plans:
            p.execute()
    ev1.record(stream)
    torch.cuda.synchronize()
    ms_loop = ev0.elapsed_time(ev1) / max(1, args.steps // 4)
    loop_launches = (g.launch_count() - l0) // max(1, args.steps // 4)
    lib.fftwf_gb300_execute_set(s)
    torch.cuda.synchronize()
    # per-transform error against the FP64 oracle on a sample
    R = Restatement()
    xh, yh = xin.cpu().numpy(), yout.cpu().numpy()
    rng = np.random.default_rng(5)
    sample = sorted(set(rng.integers(0, len(lengths), 200).tolist()))
    errs = []
    for i in sample:
        a, c = int(offs[i]), int(offs[i + 1])
        errs.append(rel_l2(yh[a:c], R.c2c(xh[a:c].astype(np.complex128), [c - a], -1, "d")))
    alg = 2 * int(offs[-1]) * 8
    hbm, src = peaks()
    out = {
        "metric": METRIC, "value": round(fl / (ms * 1e-3) / 1e9, 2), "unit": "Gflop/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"uneven{count}: {count} fftwf c2c forward plans, seeded lengths (60% 2^6..2^16, 30% 2^a3^b5^c7^d in [60,60000], 10% primes in [17,4093]) as one plan set",
                   "distinct_lengths": len(set(lengths)), "points": int(offs[-1]),
                   "queue_items": info[0].value, "long_transforms": info[2].value, "grid": info[3].value,
                   "smem": info[4].value, "plan_s": round(plan_s, 2), "set_tune_and_build_s": round(set_s, 2),
                   "tuned_lengths": tuned, "tuner_choices": choices,
                   "set_planning": "FFTW_ESTIMATE" if args.no_tune else "FFTW_MEASURE (the set tuner), 120 s limit",
                   "estimate_set": None if ms_est is None else {
                       "ms_per_step": round(ms_est, 4), "value": round(fl / (ms_est * 1e-3) / 1e9, 2),
                       "build_s": round(est_build_s, 2)},
                   "rel_l2_max_sample": max(errs), "rel_l2_median_sample": float(np.median(errs)),
                   "sampled_transforms": len(sample)},
        "gbs": round(alg / (ms * 1e-3) / 1e9, 1),
        "roofline": {"bound": "hbm", "achieved": round(alg / (ms * 1e-3) / 1e9, 1), "peak": hbm, "unit": "GB/s",
                     "frac": round(alg / (ms * 1e-3) / 1e9 / hbm, 4), "traffic": None, "peak_source": src},
        "gpu_launches": args.steps * kernels_per_step,
        "launch_note": "one CUDA graph launch per step: the small-tile work-queue kernel, and the large-tile one "
                       "beside it when the set has items that need 8192-point tiles",
        "loop_baseline": {"value": round(fl / (ms_loop * 1e-3) / 1e9, 2), "ms_per_step": round(ms_loop, 3),
                          "kernel_launches_per_step": loop_launches},
        "clocks": clk.summary(), "e2e": None, "cpu_baseline": None,
    }
    print(json.dumps(out))


def run_tc_form(g, shape, howmany, xin, yout, stream, args, fl, ws, gen):
    """Time the FFTW_GB300_TENSOR_CORE plan (radix-16 stages as split-FP16
    tcgen05 GEMMs) on the same arrays and report it beside the FP32 form,
    with its error against the FP64 oracle: on fresh N(0,1) input and on the
    log-uniform variant (magnitudes 10^U[-3,3), random signs), transforms
    spread over the batch (or the whole array of a single transform)."""
    import numpy as np
    import torch
    from oracle.oracle import Restatement
    n = math.prod(shape)
    p = g.plan_many_dft(shape, howmany, xin.data_ptr(), yout.data_ptr(), -1, g.FFTW_ESTIMATE | (1 << 28), "f")
    if "tc-split-fp16" not in p.describe():
        return None
    p.set_stream(stream.cuda_stream)
    p.set_async(True)
    for _ in range(args.warmup):
        p.execute()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        p.execute()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    k = min(howmany, 16)
    sel = torch.from_numpy(np.linspace(0, howmany - 1, k).astype(np.int64)).cuda()
    errs = {}
    for dist in ("normal", "loguniform"):
        if dist == "normal":
            x0 = torch.randn(howmany * n, dtype=torch.complex64, device="cuda", generator=gen)
        else:
            def mag():
                m = torch.pow(10.0, torch.rand(howmany * n, device="cuda", generator=gen) * 6 - 3)
                return m * (torch.randint(0, 2, (howmany * n,), device="cuda", generator=gen) * 2 - 1)
            x0 = torch.complex(mag(), mag())
        xs = x0.view(howmany, n)[sel].cpu().numpy()
        xin.copy_(x0)
        del x0
        p.execute()
        torch.cuda.synchronize()
        ys = yout.view(howmany, n)[sel].cpu().numpy().astype(np.complex128)
        ref = Restatement().c2c(xs.astype(np.complex128), shape, -1, "d", os.cpu_count() or 1).reshape(ys.shape)
        errs[dist] = float(np.linalg.norm(ys - ref) / np.linalg.norm(ref))
    hbm, _ = peaks()
    alg = 2 * n * 8 * howmany
    return {"value": round(fl * ws / (ms * 1e-3) / 1e9, 2), "unit": "Gflop/s", "ms_per_step": round(ms, 4),
            "hbm_frac": round(alg / (ms * 1e-3) / 1e9 / hbm, 4), "rel_l2_vs_fp64_oracle": errs["normal"],
            "rel_l2_loguniform_vs_fp64_oracle": errs["loguniform"], "oracle_sample_transforms": k,
            "passes": len(p.passes()),
            "form": "radix-16 stages as tcgen05 kind::f16 GEMMs, operands split FP16 hi+lo (3 products), FP32 accumulate"}


def run_e2e(lib, g, kind, shape, howmany, prec, inplace, args):
    """fftwf_execute_dft on page-locked host arrays: H2D + passes + D2H timed."""
    import ctypes
    n = math.prod(shape)
    cs = 8 if prec == "f" else 16
    nc = n // shape[-1] * (shape[-1] // 2 + 1)
    in_bytes = howmany * n * (cs if kind == "c2c" else cs // 2)
    out_bytes = howmany * n * cs // 2 if kind == "r2r" else howmany * (n if kind == "c2c" else nc) * cs
    pfx = "fftwf_" if prec == "f" else "fftw_"
    hin = getattr(lib, pfx + "malloc")(in_bytes)
    hout = hin if inplace else getattr(lib, pfx + "malloc")(out_bytes)
    ctypes.memset(hin, 0, in_bytes)
    if not inplace:
        ctypes.memset(hout, 0, out_bytes)
    if kind == "c2c":
        p = g.plan_many_dft(shape, howmany, hin, hout, -1, g.FFTW_ESTIMATE, prec)
        ex = lambda: p.execute_dft(hin, hout)
    elif kind == "r2r":
        p = g.plan_many_r2r(shape, howmany, hin, hout, [R2R_KIND] * len(shape), g.FFTW_ESTIMATE, prec)
        ex = lambda: p.execute_r2r(hin, hout)
    else:
        p = g.plan_many_dft_r2c(shape, howmany, hin, hout, g.FFTW_ESTIMATE, prec)
        ex = lambda: p.execute_dft_r2c(hin, hout)
    fails0 = lib.fftw_gb300_failures()
    ex()
    steps = max(2, min(args.steps, 5))
    each = []
    for _ in range(steps):
        t0 = time.perf_counter()
        ex()
        each.append(time.perf_counter() - t0)
    dt = sum(each) / steps
    if lib.fftw_gb300_failures() != fails0:
        raise RuntimeError("e2e: fftw execute failed: " + g.last_error())
    path = ("direct host access" if len(p.passes()) == 1 else
            "pipelined chunk staging" if howmany >= 2 else "staged copies around the passes")
    p.destroy()
    getattr(lib, pfx + "free")(hin)
    if not inplace:
        getattr(lib, pfx + "free")(hout)
    v = flops_per_step(kind, shape, howmany) / dt / 1e9
    return {"value": round(v, 2), "unit": "Gflop/s", "h2d_bytes_per_step": in_bytes, "d2h_bytes_per_step": out_bytes,
            "ms_per_step": round(dt * 1e3, 3), "ms_min": round(min(each) * 1e3, 3), "ms_max": round(max(each) * 1e3, 3),
            "path": path,
            "timer": "host wall clock around the execute call (synchronous)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2c4096", choices=sorted(WORKLOADS) + ["uneven10k"])
    ap.add_argument("--howmany", type=int, default=0, help="override the batch (profiling runs only)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-tc", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="uneven10k: the planner's defaults only (profiling runs)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference_arm(args)
    elif args.workload == "uneven10k":
        run_uneven(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
