"""Benchmark of the GB300 RNS interval-evaluation path.

Headline workload (one "step"): division of 2^18 (dividend, divisor) pairs
plus power-of-two scaling of 2^18 numbers with the n = 32 greedy moduli set
(M ~ 2^960): dividends uniform in [0, M), divisor bit length uniform in
[1, 959], scaling exponents uniform in [1, 900].  Metric: RNS numbers per
second (a division pair counts as one number), whole job.

Extra lines in the same JSON record: eval+cmp at n = 32 and n = 8 (2^20
pairs), the reference-layout (AoS) form of the same calls, and the
dominant kernel's roofline.  Inputs are generated on the device by the
seeded generator; the timed region starts with them resident in HBM.  L2
is flushed (256 MiB write) between timed steps, outside the events.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N32 = 32
PAIRS = 1 << 18
CMP_PAIRS = 1 << 20
DMAX = 900
SEED = 20260101


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region"""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu, self.proc, self.lines = gpu, None, []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        if not self.lines:
            return None
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(ngpus):
    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    return rank, world, local


def barrier_max(value, world):
    import torch
    if world == 1:
        return value
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_baseline(threads=None, sample=4096):
    """the reference's CPU path (host rns_div + host rns_scale2pow, restated in
    oracle/) on the host cores; returns (Mnum/s, cores, description)"""
    import numpy as np
    from grns_gb300 import workload as W
    from oracle import oracle as O
    moduli = O.greedy_moduli(N32)
    orc = O.Oracle(moduli)
    threads = threads or O.lib().oracle_max_threads()
    x = W.uniform_residues(moduli, sample, SEED, W.S_X, layout="aos")
    d, _ = W.divisors(moduli, orc.log2M, sample, SEED, layout="aos")
    xs = W.uniform_residues(moduli, sample, SEED, W.S_Y, layout="aos")
    D = W.shifts(sample, DMAX, SEED)
    t0 = time.perf_counter()
    orc.div(x, d, path=O.PATH_HOST, fast=0, threads=threads)
    t1 = time.perf_counter()
    orc.scale2pow(xs, D, path=O.PATH_HOST, threads=threads)
    t2 = time.perf_counter()
    rate = 2 * sample / (t2 - t0) / 1e6
    return rate, threads, (f"{sample} div pairs + {sample} scale2pow numbers (n=32, same generator), host path "
                           f"(rns_div, rns_scale2pow) restated in oracle/, {threads} threads: "
                           f"div {1e6 * (t1 - t0) / sample * threads:.0f} us/pair/core, "
                           f"scale {1e6 * (t2 - t1) / sample * threads:.1f} us/num/core")


def run_reference(args):
    rank, world, _ = (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), 0)
    if rank != 0:
        return
    vals = []
    for i in range(args.warmup + args.steps):
        v, cores, desc = cpu_baseline(sample=2048)
        if i >= args.warmup:
            vals.append(v)
    v = statistics.median(vals)
    line = {"impl": "reference", "metric": "RNS Mnum/s div+scale2pow (960-bit, n=32)", "value": v,
            "unit": "Mnum/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32+f64",
            "data": "synthetic (seeded splitmix64 generator)",
            "config": {"workload": "div 2^18 pairs + scale2pow 2^18 numbers, n=32 greedy moduli from 2^30-1",
                       "sample_per_step": "2048 div pairs + 2048 scale2pow numbers"},
            "cpu_baseline": {"value": v, "unit": "Mnum/s", "cores": cores, "kind": "port", "sample": desc},
            "e2e": {"value": v, "unit": "Mnum/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def greedy(n):
    from math import gcd
    out, c = [], 2 ** 30 - 1
    while len(out) < n:
        if c % 2 and all(gcd(c, m) == 1 for m in out):
            out.append(c)
        c -= 1
    return out


def run_only(args):
    """one op on a seeded case, timed per call with CUDA events (also the
    command line for ncu captures)"""
    import ctypes
    import torch
    import grns_gb300 as G
    from grns_gb300 import native
    from grns_gb300.workload import S_X, S_Y
    L = native.lib(build_if_missing=True)
    n = {"div": 32, "scale": 32, "cmp32": 32, "cmp8": 8, "max64": 64, "eval32": 32, "mpint64": 64}[args.only]
    ctx = G.RNSContext(greedy(n))
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    cnt = args.pairs
    x = torch.empty((n, cnt), dtype=torch.int32, device="cuda")
    y = torch.empty_like(x)
    native.check(L.grns_gen_uniform(ctx.handle, SEED, S_X, cnt, 0, P(x), sp))
    if args.only == "div":
        native.check(L.grns_gen_divisors(ctx.handle, SEED, cnt, 0, P(y), sp))
    else:
        native.check(L.grns_gen_uniform(ctx.handle, SEED, S_Y, cnt, 0, P(y), sp))
    D = torch.empty(cnt, dtype=torch.int32, device="cuda")
    native.check(L.grns_gen_shifts(SEED, cnt, DMAX, P(D), sp))
    a, b = torch.empty_like(x), torch.empty_like(x)
    out = torch.empty(cnt * 32, dtype=torch.uint8, device="cuda")
    val = torch.empty(n, dtype=torch.int32, device="cuda")
    idx = torch.empty(1, dtype=torch.int64, device="cuda")
    mb = G.mpint_bytes(n)
    if args.only == "mpint64":
        from grns_gb300.workload import mpint_values  # operands: residues of random ints below 2^950
        ma = torch.zeros(cnt * mb, dtype=torch.uint8, device="cuda")
        mc = torch.zeros_like(ma)
        mo = torch.zeros_like(ma)
    def call():
        if args.only == "div":
            native.check(L.grns_div(ctx.handle, P(x), P(y), cnt, 0, P(a), P(b), None, sp))
        elif args.only == "scale":
            native.check(L.grns_scale2pow(ctx.handle, P(x), P(D), 0, cnt, 0, P(a), None, sp))
        elif args.only in ("cmp32", "cmp8"):
            native.check(L.grns_cmp(ctx.handle, P(x), P(y), cnt, 0, P(D), None, sp))
        elif args.only == "max64":
            native.check(L.grns_max(ctx.handle, P(x), cnt, 0, P(val), P(idx), None, 0, sp))
        elif args.only == "eval32":
            native.check(L.grns_eval(ctx.handle, P(x), cnt, 0, P(out), None, sp))
        elif args.only == "mpint64":
            native.check(L.grns_mpint_mul(ctx.handle, P(ma), P(mc), cnt, P(mo), None, sp))

    for _ in range(args.warmup):
        call()
    times = []
    stream = torch.cuda.current_stream()
    flush = torch.empty(64 << 20, dtype=torch.int32, device="cuda") if args.flush else None
    for _ in range(args.steps):
        if flush is not None:
            flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        call()
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    ms = statistics.median(times) if times else 0.0
    print(json.dumps({"only": args.only, "count": cnt, "flush": bool(args.flush), "calls": args.warmup + args.steps,
                      "ms_median": ms,
                      "Mnum_s": cnt / (ms * 1e-3) / 1e6 if ms else None}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="grns_gb300")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--pairs", type=int, default=PAIRS, help="numbers per op (profiling cases use fewer)")
    ap.add_argument("--flush", action="store_true", help="profiling mode: flush L2 (256 MiB write) before each call")
    ap.add_argument("--only", choices=["div", "scale", "cmp32", "cmp8", "max64", "eval32", "mpint64"], default=None,
                    help="profiling: run just this op --warmup + --steps times on --pairs numbers, no JSON line")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup) if args.only is None else args.warmup
    if args.impl == "reference":
        return run_reference(args)
    if args.only:
        return run_only(args)

    import torch
    import grns_gb300 as G
    from grns_gb300 import native
    rank, world, local = dist_setup(args.gpus)
    L = native.lib(build_if_missing=True)
    from grns_gb300.workload import S_X, S_Y
    import ctypes

    ctx = G.RNSContext(greedy(N32))
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    seed = SEED + rank

    # ---- inputs resident in HBM (SoA) ----
    x = torch.empty((N32, PAIRS), dtype=torch.int32, device=dev)
    d = torch.empty_like(x)
    xs = torch.empty_like(x)
    D = torch.empty(PAIRS, dtype=torch.int32, device=dev)
    native.check(L.grns_gen_uniform(ctx.handle, seed, S_X, PAIRS, 0, P(x), sp))
    native.check(L.grns_gen_divisors(ctx.handle, seed, PAIRS, 0, P(d), sp))
    native.check(L.grns_gen_uniform(ctx.handle, seed, S_Y, PAIRS, 0, P(xs), sp))
    native.check(L.grns_gen_shifts(seed, PAIRS, DMAX, P(D), sp))
    q, r, so = torch.empty_like(x), torch.empty_like(x), torch.empty_like(x)
    flush = torch.empty(64 << 20, dtype=torch.int32, device=dev)  # 256 MiB > L2

    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731

    def step(timers=None):
        e0, e1, e2 = (timers or (None, None, None))
        if e0: e0.record(stream)
        native.check(L.grns_div(ctx.handle, P(x), P(d), PAIRS, 0, P(q), P(r), None, sp))
        if e1: e1.record(stream)
        native.check(L.grns_scale2pow(ctx.handle, P(xs), P(D), 0, PAIRS, 0, P(so), None, sp))
        if e2: e2.record(stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    step_ms, div_ms, scale_ms = [], [], []
    with Clocks(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            t = (ev(), ev(), ev())
            step(t)
            torch.cuda.synchronize()
            div_ms.append(t[0].elapsed_time(t[1]))
            scale_ms.append(t[1].elapsed_time(t[2]))
            step_ms.append(t[0].elapsed_time(t[2]))
    total_ms = barrier_max(sum(step_ms), world)
    ms = total_ms / args.steps
    value = world * 2 * PAIRS / (ms * 1e-3) / 1e6

    # ---- end to end through the C ABI with host buffers (pinned), copies inside the timed region ----
    hx = x.cpu().pin_memory(); hd = d.cpu().pin_memory(); hxs = xs.cpu().pin_memory(); hD = D.cpu().pin_memory()
    hq = torch.empty_like(hx).pin_memory(); hr = torch.empty_like(hx).pin_memory(); hso = torch.empty_like(hx).pin_memory()
    e2e_ms = []
    for i in range(args.warmup + args.steps):
        flush.zero_()
        a, b = ev(), ev()
        a.record(stream)
        x.copy_(hx, non_blocking=True); d.copy_(hd, non_blocking=True)
        xs.copy_(hxs, non_blocking=True); D.copy_(hD, non_blocking=True)
        step()
        hq.copy_(q, non_blocking=True); hr.copy_(r, non_blocking=True); hso.copy_(so, non_blocking=True)
        b.record(stream)
        torch.cuda.synchronize()
        if i >= args.warmup:
            e2e_ms.append(a.elapsed_time(b))
    e2e = world * 2 * PAIRS / (barrier_max(sum(e2e_ms), world) / args.steps * 1e-3) / 1e6
    h2d = 4 * (x.numel() * 3 + D.numel())
    d2h = 4 * x.numel() * 3

    # ---- extra lines: eval+cmp (960-bit and 240-bit), SoA and the reference AoS layout ----
    extra = {}
    for n in (32, 8):
        c2 = G.RNSContext(greedy(n))
        a = torch.empty((n, CMP_PAIRS), dtype=torch.int32, device=dev)
        bb = torch.empty_like(a)
        native.check(L.grns_gen_uniform(c2.handle, seed, S_X, CMP_PAIRS, 0, P(a), sp))
        native.check(L.grns_gen_uniform(c2.handle, seed, S_Y, CMP_PAIRS, 0, P(bb), sp))
        out = torch.empty(CMP_PAIRS, dtype=torch.int32, device=dev)
        for layout, lname in ((0, "soa"), (1, "aos")):
            A = a if layout == 0 else a.t().contiguous()
            B = bb if layout == 0 else bb.t().contiguous()
            for _ in range(3):
                native.check(L.grns_cmp(c2.handle, P(A), P(B), CMP_PAIRS, layout, P(out), None, sp))
            tt = []
            for _ in range(max(3, args.steps)):
                flush.zero_()
                s0, s1 = ev(), ev()
                s0.record(stream)
                native.check(L.grns_cmp(c2.handle, P(A), P(B), CMP_PAIRS, layout, P(out), None, sp))
                s1.record(stream)
                torch.cuda.synchronize()
                tt.append(s0.elapsed_time(s1))
            m = statistics.median(tt)
            extra[f"eval_cmp_n{n}_{lname}_Mnum_s"] = CMP_PAIRS / (m * 1e-3) / 1e6
            if lname == "soa":
                bytes_pair = 8 * n + 4
                extra[f"eval_cmp_n{n}_soa_GBps"] = bytes_pair * CMP_PAIRS / (m * 1e-3) / 1e9
        c2.close()

    peak, peak_kind = load_peaks()
    div_avg = statistics.mean(div_ms)
    alg_bytes = 16 * N32 * PAIRS
    achieved = alg_bytes / (div_avg * 1e-3) / 1e9
    line = {
        "metric": "RNS Mnum/s div+scale2pow (960-bit, n=32)", "value": value, "unit": "Mnum/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32+f64",
        "data": "synthetic (seeded splitmix64 generator, device-generated)",
        "config": {"workload": "div 2^18 pairs (divisor bits uniform in [1,959]) + scale2pow 2^18 numbers "
                               "(D uniform in [1,900]), n=32 greedy moduli from 2^30-1, SoA",
                   "l2": "flushed (256 MiB write) between timed steps", "parallelism": f"replicas x{world}"},
        "roofline": {"bound": "hbm", "kernel": "k_div<32>", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind, "traffic": None,
                     "note": "division is compute-bound (FP64/INT pipes), not HBM-bound"},
        "kernels_ms": {"k_div": div_avg, "k_scale": statistics.mean(scale_ms)},
        "e2e": {"value": e2e, "unit": "Mnum/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": 2 * args.steps,
        "extra": extra,
    }
    line["clocks"] = clk.summary()
    if rank == 0 and not args.no_cpu:
        v, cores, desc = cpu_baseline()
        line["cpu_baseline"] = {"value": v, "unit": "Mnum/s", "cores": cores, "kind": "port", "sample": desc}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
