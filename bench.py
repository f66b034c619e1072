"""Benchmark of the GB300 RNS interval-evaluation path.

Headline workload (one "step"): division of 2^18 (dividend, divisor) pairs
plus power-of-two scaling of 2^18 numbers with the n = 32 greedy moduli set
(M ~ 2^960): dividends uniform in [0, M), divisor bit length uniform in
[1, 959], scaling exponents uniform in [1, 900].  Metric: RNS numbers per
second (a division pair counts as one number), whole job.

The same JSON record carries the other workloads (skipped with --quick):
  extra:      eval+cmp at n = 8 and n = 32 (2^20 pairs, SoA and the
              reference's AoS layout), rns_eval_compute alone (n = 32, 2^22),
              mp_int add/sub/mul at n = 64 (2^22 pairs, magnitudes < 2^950),
              the maximum over 2^24 numbers at n = 64 -- each with its HBM
              roofline fraction;
  workloads:  4096 uneven jobs (log-uniform lengths in [1e2, 1e6]) in one
              persistent launch captured as a CUDA graph vs one plain call per
              job; a served request stream (n = 32 and n = 64 contexts,
              log-uniform lengths in [1e3, 1e7], Poisson arrivals at swept
              rates) with p50/p99 latency vs per-request plain calls.
Inputs are generated on the device by the seeded generator; timed regions
start with them resident in HBM.  L2 is flushed (256 MiB write) between timed
calls, outside the events.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--quick] [--impl reference]
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
DIV_TRAFFIC_BYTES = 447.1e6  # DRAM bytes of one 2^18-pair division call (ncu, five launches, each cold)
CONV_COUNT = 1 << 22  # numbers per binary <-> RNS conversion call
CMP_PAIRS = 1 << 20
EVAL_COUNT = 1 << 22
MP_PAIRS = 1 << 22          # mp_int pairs at n = 64
MP_BITS = 950               # mp_int magnitudes uniform in [0, 2^950)
MAX_COUNT = 1 << 24         # maximum over 2^24 numbers at n = 64
BATCH_JOBS = 4096
BATCH_LEN = (1e2, 1e6)      # log-uniform job lengths
SERVE_REQS = 64
SERVE_LEN = (1e3, 1e7)      # log-uniform request lengths
SERVE_POOL = 10 ** 7        # device-resident operand pools
SERVE_BUDGET = 48 << 30     # server HBM budget for outputs
SERVE_LOADS = (0.5, 0.9)    # offered load as a fraction of the all-at-once throughput
SERVE_GATHER_US = 500       # gathering window of the second all-at-once run (the server's gather_us)
DMAX = 900
SEED = 20260101
WARMUP_SECONDS = 0.25       # minimum warm-up time before the timed steps


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
    """the maximum of `value` over the ranks (NCCL on GPUs; gloo on the CPU)"""
    import torch
    if world == 1:
        return value
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate(per_rank_ms, count_per_rank, world):
    """(ms per step, whole-job Mnum/s): every rank processed count_per_rank
    numbers per step (weak scaling); the job takes the slowest rank's time"""
    ms = barrier_max(per_rank_ms, world)
    return ms, world * count_per_rank / (ms * 1e-3) / 1e6


HEADLINE_OPS = ("div_n32", "div_fast_n32", "scale2pow_n32")


def cpu_ops(threads=None, scale=1.0, which=None):
    """the reference's CPU path op by op (host rns_eval_compute, rns_cmp,
    rns_div, rns_div_fast, rns_scale2pow, mpint_add/sub/mul, restated in
    oracle/ and pinned bit for bit to the reference compiled for the CPU), on
    the workloads' own seeded inputs: each op on all host threads (OpenMP)
    and on one.  Returns {op: {"Mnum_s", "Mnum_s_1core", "sample", ...}} and
    the thread count.  `scale` shrinks the samples (the reference arm's
    per-step samples); `which` limits the ops timed."""
    from grns_gb300 import workload as W
    from oracle import oracle as O
    threads = threads or O.lib().oracle_max_threads()
    H = O.PATH_HOST

    def timed(fn, count, cores):
        t0 = time.perf_counter()
        fn(cores)
        return count / (time.perf_counter() - t0) / 1e6

    def run(name, call, count, count1, **info):
        if which is not None and name not in which:
            return
        all_c = timed(call(count), count, threads)
        one_c = timed(call(count1), count1, 1)
        res[name] = dict(Mnum_s=all_c, Mnum_s_1core=one_c, sample=count, sample_1core=count1, **info)

    res = {}
    k = lambda c: max(64, int(c * scale))  # noqa: E731
    # n = 32 (960 bits): division, scaling, evaluation, comparison
    m32 = O.greedy_moduli(N32)
    o32 = O.Oracle(m32)
    nd = k(8192)
    ne = k(1 << 18)
    x = W.uniform_residues(m32, max(ne, nd), SEED, W.S_X, layout="aos")
    y = W.uniform_residues(m32, max(ne, nd), SEED, W.S_Y, layout="aos")
    d, _ = W.divisors(m32, o32.log2M, nd, SEED, layout="aos")
    D = W.shifts(nd, DMAX, SEED)
    run("div_n32", lambda c: lambda t: o32.div(x[:c], d[:c], path=H, fast=0, threads=t), nd, max(16, nd // 64),
        ref="rns_div (src/rnsdiv.cuh:19), one quotient bit per iteration")
    run("div_fast_n32", lambda c: lambda t: o32.div(x[:c], d[:c], path=H, fast=1, threads=t), nd, max(64, nd // 8),
        ref="rns_div_fast (src/rnsdiv.cuh:67)")
    run("scale2pow_n32", lambda c: lambda t: o32.scale2pow(y[:c], D[:c], path=H, threads=t), nd, max(64, nd // 8),
        ref="rns_scale2pow (src/rnsscal.cuh:93)")
    run("eval_n32", lambda c: lambda t: o32.eval(x[:c], path=H, threads=t), ne, max(256, ne // 8),
        ref="rns_eval_compute (src/rnseval.cuh:29)")
    run("eval_cmp_n32", lambda c: lambda t: o32.cmp(x[:c], y[:c], path=H, threads=t), ne, max(256, ne // 8),
        ref="rns_cmp (src/rnscmp.cuh:20), two evaluations per pair")
    if which is not None and not any(w.endswith(("_n8", "_n64")) for w in which):
        return res, threads
    # n = 8 (240 bits): comparison
    m8 = O.greedy_moduli(8)
    o8 = O.Oracle(m8)
    x8 = W.uniform_residues(m8, ne, SEED, W.S_X, layout="aos")
    y8 = W.uniform_residues(m8, ne, SEED, W.S_Y, layout="aos")
    run("eval_cmp_n8", lambda c: lambda t: o8.cmp(x8[:c], y8[:c], path=H, threads=t), ne, max(256, ne // 8),
        ref="rns_cmp (src/rnscmp.cuh:20)")
    # n = 64 (1920 bits): mp_int add / sub / mul, magnitudes below 2^950
    m64 = O.greedy_moduli(64)
    o64 = O.Oracle(m64)
    nm = k(1 << 16)
    ma = o64.mpint_from_ints(W.mpint_values(nm, MP_BITS, SEED), path=H)
    mc = o64.mpint_from_ints(W.mpint_values(nm, MP_BITS, SEED + 1), path=H)
    for op in ("add", "sub", "mul"):
        run(f"mpint_{op}_n64", lambda c, op=op: lambda t: o64.mpint(op, ma[:c], mc[:c], path=H, threads=t), nm,
            max(256, nm // 8), ref=f"mpint_{op} (src/mpint.cuh:{ {'add': 160, 'sub': 215, 'mul': 270}[op] })")
    return res, threads


def cpu_baseline(threads=None, scale=1.0, every_op=True):
    """the headline's CPU figure: division (the faster of host rns_div and
    rns_div_fast, which give the same q and r) plus power-of-two scaling at
    n = 32, as numbers per second over the two ops; and each op's figure
    (every op of the path, or the headline's three)"""
    ops, threads = cpu_ops(threads, scale, None if every_op else HEADLINE_OPS)
    div = max(ops["div_n32"]["Mnum_s"], ops["div_fast_n32"]["Mnum_s"])
    div1 = max(ops["div_n32"]["Mnum_s_1core"], ops["div_fast_n32"]["Mnum_s_1core"])
    sc, sc1 = ops["scale2pow_n32"]["Mnum_s"], ops["scale2pow_n32"]["Mnum_s_1core"]
    rate = 2.0 / (1.0 / div + 1.0 / sc)
    rate1 = 2.0 / (1.0 / div1 + 1.0 / sc1)
    desc = (f"{ops['div_fast_n32']['sample']} div pairs + {ops['scale2pow_n32']['sample']} scale2pow numbers "
            f"(n=32, the workload's generators); host path restated in oracle/ (bit-identical to the reference "
            f"compiled for the CPU), {threads} threads; division = the faster of rns_div "
            f"({ops['div_n32']['Mnum_s'] * 1e6:.0f}/s) and rns_div_fast ({ops['div_fast_n32']['Mnum_s'] * 1e6:.0f}/s); "
            f"one core: {rate1:.4f} Mnum/s")
    return rate, threads, desc, ops


def run_reference(args):
    rank, world, _ = (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), 0)
    if rank != 0:
        return
    vals = []
    for i in range(args.warmup + args.steps):  # a step: the headline's ops on a bounded sample
        v, cores, desc, ops = cpu_baseline(scale=0.5, every_op=False)
        if i >= args.warmup:
            vals.append(v)
    v = statistics.median(vals)
    ops, _ = cpu_ops(cores)  # every op of the path once, for the record
    line = {"impl": "reference", "metric": "RNS Mnum/s div+scale2pow (960-bit, n=32)", "value": v,
            "unit": "Mnum/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32+f64",
            "data": "synthetic (seeded splitmix64 generator)",
            "config": {"workload": "div 2^18 pairs + scale2pow 2^18 numbers, n=32 greedy moduli from 2^30-1",
                       "sample_per_step": desc.split(";")[0]},
            "cpu_baseline": {"value": v, "unit": "Mnum/s", "cores": cores, "kind": "port", "sample": desc,
                             "ops": ops},
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
    n = args.n or {"div": 32, "scale": 32, "cmp32": 32, "cmp8": 8, "max64": 64, "eval32": 32, "evtight32": 32,
                   "mpint64": 64, "mpdiv32": 32, "tobin32": 32, "frombin32": 32, "tobin64": 64, "mrc32": 32}[args.only]
    ctx = G.RNSContext(greedy(n))
    if args.eval_split is not None:
        native.check(L.grns_ctx_set_eval_split(ctx.handle, args.eval_split))
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
    if args.only in ("mpint64", "mpdiv32"):
        ma = torch.zeros(cnt * mb, dtype=torch.uint8, device="cuda")
        mc = torch.zeros_like(ma)
        mo = torch.zeros_like(ma)
    if args.only in ("tobin32", "frombin32", "tobin64"):  # integers below M as 32-bit limbs
        LM = L.grns_ctx_binary_limbs(ctx.handle)
        words = torch.empty((cnt, LM), dtype=torch.int32, device="cuda")
        native.check(L.grns_to_binary(ctx.handle, P(x), cnt, 0, P(words), LM, None, sp))
    if args.only == "mpdiv32":  # signed dividends below 2^900, divisors below 2^450
        native.check(L.grns_gen_mpint(ctx.handle, SEED, cnt, 900, P(ma), sp))
        native.check(L.grns_gen_mpint(ctx.handle, SEED + 1, cnt, 450, P(mc), sp))
    if args.only == "mpint64":  # the workload's operands: random signs, magnitudes below 2^950
        native.check(L.grns_gen_mpint(ctx.handle, SEED, cnt, MP_BITS, P(ma), sp))
        native.check(L.grns_gen_mpint(ctx.handle, SEED + 1, cnt, MP_BITS, P(mc), sp))
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
        elif args.only == "evtight32":
            native.check(L.grns_eval_tight(ctx.handle, P(x), cnt, 0, P(out), None, sp))
        elif args.only == "mpint64":
            native.check(getattr(L, f"grns_mpint_{args.mp_op}")(ctx.handle, P(ma), P(mc), cnt, P(mo), None, sp))
        elif args.only == "mpdiv32":
            native.check(L.grns_mpint_div(ctx.handle, P(ma), P(mc), cnt, P(mo), None, sp))
        elif args.only in ("tobin32", "tobin64"):
            native.check(L.grns_to_binary(ctx.handle, P(x), cnt, 0, P(words), LM, None, sp))
        elif args.only == "frombin32":
            native.check(L.grns_from_binary(ctx.handle, P(words), LM, cnt, 0, P(a), sp))
        elif args.only == "mrc32":
            native.check(L.grns_mrc(ctx.handle, P(x), cnt, 0, P(a), None, sp))

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
    print(json.dumps({"only": args.only, "n": n, "count": cnt, "flush": bool(args.flush),
                      "calls": args.warmup + args.steps,
                      "eval_split": L.grns_ctx_get_eval_split(ctx.handle),
                      "ms_median": ms,
                      "Mnum_s": cnt / (ms * 1e-3) / 1e6 if ms else None}))


# ---------------------------------------------------------------------------
# timing helpers

def _ev():
    import torch
    return torch.cuda.Event(enable_timing=True)


def time_calls(fn, steps, stream, flush=None):
    """per-call device time (ms) of fn() on `stream`, L2 flushed before each call"""
    import torch
    out = []
    for _ in range(steps):
        if flush is not None:
            flush.zero_()
        a, b = _ev(), _ev()
        a.record(stream)
        fn()
        b.record(stream)
        torch.cuda.synchronize()
        out.append(a.elapsed_time(b))
    return out


def log_uniform_lengths(rng, count, lo, hi):
    import math
    return [int(round(math.exp(rng.uniform(math.log(lo), math.log(hi))))) for _ in range(count)]


# ---------------------------------------------------------------------------
# eval + cmp (n = 8 and n = 32), eval alone, mp_int and max (n = 64)

def bench_eval_cmp(ctx_for, L, dev, stream, sp, P, seed, steps, flush, peak):
    import torch
    from grns_gb300 import native
    from grns_gb300.workload import S_X, S_Y
    res = {}
    for n in (8, 32):
        c2 = ctx_for(n)
        a = torch.empty((n, CMP_PAIRS), dtype=torch.int32, device=dev)
        bb = torch.empty_like(a)
        native.check(L.grns_gen_uniform(c2.handle, seed, S_X, CMP_PAIRS, 0, P(a), sp))
        native.check(L.grns_gen_uniform(c2.handle, seed, S_Y, CMP_PAIRS, 0, P(bb), sp))
        out = torch.empty(CMP_PAIRS, dtype=torch.int32, device=dev)
        for layout, lname in ((0, "soa"), (1, "aos")):
            A = a if layout == 0 else a.t().contiguous()
            B = bb if layout == 0 else bb.t().contiguous()
            f = lambda: native.check(L.grns_cmp(c2.handle, P(A), P(B), CMP_PAIRS, layout, P(out), None, sp))  # noqa
            time_calls(f, 3, stream)
            m = statistics.median(time_calls(f, max(3, steps), stream, flush))
            rate = CMP_PAIRS / (m * 1e-3)
            gbs = (8 * n + 4) * rate / 1e9
            res[f"eval_cmp_n{n}_{lname}"] = {"Mnum_s": rate / 1e6, "GBps": gbs, "frac_hbm": gbs / peak,
                                             "ms": m, "pairs": CMP_PAIRS}
    # rns_eval_compute alone at n = 32: reads 128 B, writes one interval (32 B) per number
    c32 = ctx_for(32)
    cnt = EVAL_COUNT
    x = torch.empty((32, cnt), dtype=torch.int32, device=dev)
    native.check(L.grns_gen_uniform(c32.handle, seed, S_X, cnt, 0, P(x), sp))
    iv = torch.empty(cnt * 32, dtype=torch.uint8, device=dev)
    f = lambda: native.check(L.grns_eval(c32.handle, P(x), cnt, 0, P(iv), None, sp))  # noqa
    time_calls(f, 3, stream)
    m = statistics.median(time_calls(f, max(3, steps), stream, flush))
    gbs = (4 * 32 + 32) * cnt / (m * 1e-3) / 1e9
    res["eval_n32_soa"] = {"Mnum_s": cnt / (m * 1e-3) / 1e6, "GBps": gbs, "frac_hbm": gbs / peak, "ms": m,
                           "count": cnt, "bytes_per_number": 160, "kernel": "k_eval (bit-identical intervals)"}
    f = lambda: native.check(L.grns_eval_tight(c32.handle, P(x), cnt, 0, P(iv), None, sp))  # noqa
    time_calls(f, 3, stream)
    m = statistics.median(time_calls(f, max(3, steps), stream, flush))
    gbs = (4 * 32 + 32) * cnt / (m * 1e-3) / 1e9
    res["eval_tight_n32_soa"] = {"Mnum_s": cnt / (m * 1e-3) / 1e6, "GBps": gbs, "frac_hbm": gbs / peak, "ms": m,
                                 "count": cnt, "bytes_per_number": 160,
                                 "kernel": "k_eval_tight_soa4 (one-ulp intervals, never wider than the reference's)"}
    return res


def bench_mpint_max(ctx_for, L, dev, stream, sp, P, seed, steps, flush, peak):
    """mp_int add / sub / mul at n = 64 (2^22 pairs, magnitudes below 2^950, random
    signs) and the maximum over 2^24 uniform numbers at n = 64"""
    import torch
    import grns_gb300 as G
    from grns_gb300 import native
    from grns_gb300.workload import S_X
    c64 = ctx_for(64)
    mb = G.mpint_bytes(64)
    cnt = MP_PAIRS
    ma = torch.empty(cnt * mb, dtype=torch.uint8, device=dev)
    mc = torch.empty_like(ma)
    mo = torch.empty_like(ma)
    native.check(L.grns_gen_mpint(c64.handle, seed, cnt, MP_BITS, P(ma), sp))
    native.check(L.grns_gen_mpint(c64.handle, seed + 1, cnt, MP_BITS, P(mc), sp))
    res = {}
    for op in ("add", "sub", "mul"):
        fn = getattr(L, f"grns_mpint_{op}")
        f = lambda: native.check(fn(c64.handle, P(ma), P(mc), cnt, P(mo), None, sp))  # noqa
        time_calls(f, 3, stream)
        m = statistics.median(time_calls(f, max(3, steps), stream, flush))
        gbs = 3 * mb * cnt / (m * 1e-3) / 1e9
        res[f"mpint_{op}_n64"] = {"Mnum_s": cnt / (m * 1e-3) / 1e6, "GBps": gbs, "frac_hbm": gbs / peak, "ms": m,
                                  "pairs": cnt, "bytes_per_pair": 3 * mb}
    del ma, mc, mo
    cnt = MAX_COUNT
    x = torch.empty((64, cnt), dtype=torch.int32, device=dev)
    native.check(L.grns_gen_uniform(c64.handle, seed, S_X, cnt, 0, P(x), sp))
    val = torch.empty(64, dtype=torch.int32, device=dev)
    idx = torch.empty(1, dtype=torch.int64, device=dev)
    scratch = torch.empty(c64.max_scratch_size(cnt), dtype=torch.uint8, device=dev)
    f = lambda: native.check(L.grns_max(c64.handle, P(x), cnt, 0, P(val), P(idx), P(scratch),  # noqa
                                        scratch.numel(), sp))
    time_calls(f, 3, stream)
    m = statistics.median(time_calls(f, max(3, steps), stream, flush))
    gbs = 4 * 64 * cnt / (m * 1e-3) / 1e9
    res["max_n64_soa"] = {"Mnum_s": cnt / (m * 1e-3) / 1e6, "GBps": gbs, "frac_hbm": gbs / peak, "ms": m,
                          "count": cnt, "bytes_per_number": 256}
    return res


def bench_next_ops(ctx_for, L, dev, stream, sp, P, seed, steps, flush, peak):
    """the operations next to the path: mp_int division (n = 32, 2^18 pairs,
    900-bit dividends, 450-bit divisors), binary <-> RNS conversion (n = 32
    and 64, 2^22 numbers below M) and mixed-radix conversion (n = 32, 2^22)"""
    import torch
    import grns_gb300 as G
    from grns_gb300 import native
    from grns_gb300.workload import S_X
    res = {}
    c32 = ctx_for(32)
    mb = G.mpint_bytes(32)
    cnt = PAIRS
    ma = torch.empty(cnt * mb, dtype=torch.uint8, device=dev)
    mc, mo = torch.empty_like(ma), torch.empty_like(ma)
    native.check(L.grns_gen_mpint(c32.handle, seed, cnt, 900, P(ma), sp))
    native.check(L.grns_gen_mpint(c32.handle, seed + 1, cnt, 450, P(mc), sp))
    f = lambda: native.check(L.grns_mpint_div(c32.handle, P(ma), P(mc), cnt, P(mo), None, sp))  # noqa
    time_calls(f, 3, stream)
    m = statistics.median(time_calls(f, max(3, steps), stream, flush))
    res["mpint_div_n32"] = {"Mnum_s": cnt / (m * 1e-3) / 1e6, "ms": m, "pairs": cnt,
                            "operands": "900-bit dividends, 450-bit divisors, random signs"}
    del ma, mc, mo
    for n in (32, 64):
        c = ctx_for(n)
        cnt = CONV_COUNT
        LM = L.grns_ctx_binary_limbs(c.handle)
        x = torch.empty((n, cnt), dtype=torch.int32, device=dev)
        y = torch.empty_like(x)
        w = torch.empty((cnt, LM), dtype=torch.int32, device=dev)
        native.check(L.grns_gen_uniform(c.handle, seed, S_X, cnt, 0, P(x), sp))
        f = lambda: native.check(L.grns_to_binary(c.handle, P(x), cnt, 0, P(w), LM, None, sp))  # noqa
        time_calls(f, 3, stream)
        m = statistics.median(time_calls(f, max(3, steps), stream, flush))
        b = (4 * n + 4 * LM) * cnt
        res[f"to_binary_n{n}"] = {"Mnum_s": cnt / (m * 1e-3) / 1e6, "GBps": b / (m * 1e-3) / 1e9,
                                  "frac_hbm": b / (m * 1e-3) / 1e9 / peak, "ms": m, "count": cnt, "limbs": LM}
        f = lambda: native.check(L.grns_from_binary(c.handle, P(w), LM, cnt, 0, P(y), sp))  # noqa
        time_calls(f, 3, stream)
        m = statistics.median(time_calls(f, max(3, steps), stream, flush))
        res[f"from_binary_n{n}"] = {"Mnum_s": cnt / (m * 1e-3) / 1e6, "GBps": b / (m * 1e-3) / 1e9,
                                    "frac_hbm": b / (m * 1e-3) / 1e9 / peak, "ms": m, "count": cnt, "limbs": LM}
        if n == 32:
            f = lambda: native.check(L.grns_mrc(c.handle, P(x), cnt, 0, P(y), None, sp))  # noqa
            time_calls(f, 3, stream)
            m = statistics.median(time_calls(f, max(3, steps), stream, flush))
            res["mrc_n32"] = {"Mnum_s": cnt / (m * 1e-3) / 1e6, "ms": m, "count": cnt,
                              "note": "n (n - 1) / 2 = 496 subtract-and-multiply steps per number"}
        del x, y, w
    return res


# ---------------------------------------------------------------------------
# batched uneven workload (n = 32): one persistent launch (CUDA graph) vs one plain call per job

def bench_batched(ctx_for, L, dev, stream, sp, P, seed, steps, flush):
    """three uneven job sets at n = 32 (4096 jobs, log-uniform lengths): the
    mixed one (eval+cmp, div, scale2pow, max), eval+cmp only and div only --
    each as one persistent launch (CUDA graph) and as one plain call per job"""
    import ctypes
    from grns_gb300 import native
    c = ctx_for(32)
    tuned = {}
    for op in (native.OP_CMP, native.OP_DIV, native.OP_SCALE2POW, native.OP_MAX):
        sc, ms = native.Schedule(), ctypes.c_double()
        native.check(L.grns_autotune(c.handle, op, 1 << 18, None, ctypes.byref(sc), ctypes.byref(ms)))
        tuned[str(op)] = {"coop": sc.coop, "chunk": sc.chunk}
    out = {"schedules": tuned}
    sets = (("mixed", (native.OP_CMP, native.OP_DIV, native.OP_SCALE2POW, native.OP_MAX)),
            ("eval_cmp_only", (native.OP_CMP,)), ("div_only", (native.OP_DIV,)))
    for k, (name, ops) in enumerate(sets):
        out[name] = batched_job_set(c, L, dev, stream, sp, P, seed + k, steps, flush, ops)
    return out


def batched_job_set(c, L, dev, stream, sp, P, seed, steps, flush, op_choices):
    import random
    import ctypes
    import torch
    from grns_gb300 import native
    from grns_gb300.workload import S_X, S_Y
    n = 32
    rng = random.Random(seed)
    lens = log_uniform_lengths(rng, BATCH_JOBS, *BATCH_LEN)
    ops = [rng.choice(op_choices) for _ in lens]
    pool = max(lens)
    # operand pools in the reference's AoS layout: a job is a window [o, o + len) of them
    X = torch.empty((pool, n), dtype=torch.int32, device=dev)
    Y = torch.empty_like(X)
    Dv = torch.empty_like(X)
    Sh = torch.empty(pool, dtype=torch.int32, device=dev)
    native.check(L.grns_gen_uniform(c.handle, seed, S_X, pool, 1, P(X), sp))
    native.check(L.grns_gen_uniform(c.handle, seed, S_Y, pool, 1, P(Y), sp))
    native.check(L.grns_gen_divisors(c.handle, seed, pool, 1, P(Dv), sp))
    native.check(L.grns_gen_shifts(seed, pool, DMAX, P(Sh), sp))
    offs = [rng.randrange(pool - ln + 1) for ln in lens]
    # outputs: one region per kind, carved per job (every job writes its own outputs)
    tot = {op: sum(ln for ln, o in zip(lens, ops) if o == op) for op in set(ops)}
    q_all = torch.empty(max(1, tot.get(native.OP_DIV, 0)) * n, dtype=torch.int32, device=dev)
    r_all = torch.empty_like(q_all)
    s_all = torch.empty(max(1, tot.get(native.OP_SCALE2POW, 0)) * n, dtype=torch.int32, device=dev)
    c_all = torch.empty(max(1, tot.get(native.OP_CMP, 0)), dtype=torch.int32, device=dev)
    nmax = sum(1 for o in ops if o == native.OP_MAX)
    mv_all = torch.empty(max(1, nmax) * n, dtype=torch.int32, device=dev)
    mi_all = torch.empty(max(1, nmax), dtype=torch.int64, device=dev)
    jobs = (native.Job * BATCH_JOBS)()
    calls = []
    cur = {native.OP_DIV: 0, native.OP_SCALE2POW: 0, native.OP_CMP: 0, native.OP_MAX: 0}
    for t, (ln, op, o) in enumerate(zip(lens, ops, offs)):
        j = jobs[t]
        j.op, j.layout, j.count, j.ld = op, 1, ln, 0
        a = X.data_ptr() + 4 * n * o
        j.a = a
        k = cur[op]
        if op == native.OP_CMP:
            b, o0 = Y.data_ptr() + 4 * n * o, c_all.data_ptr() + 4 * k
            j.b, j.out0 = b, o0
            cur[op] += ln
            calls.append((L.grns_cmp, (c.handle, a, b, ln, 1, o0, None, sp)))
        elif op == native.OP_DIV:
            b, o0, o1 = Dv.data_ptr() + 4 * n * o, q_all.data_ptr() + 4 * n * k, r_all.data_ptr() + 4 * n * k
            j.b, j.out0, j.out1 = b, o0, o1
            cur[op] += ln
            calls.append((L.grns_div, (c.handle, a, b, ln, 1, o0, o1, None, sp)))
        elif op == native.OP_SCALE2POW:
            b, o0 = Sh.data_ptr() + 4 * o, s_all.data_ptr() + 4 * n * k
            j.b, j.out0 = b, o0
            cur[op] += ln
            calls.append((L.grns_scale2pow, (c.handle, a, b, 0, ln, 1, o0, None, sp)))
        else:
            o0, o1 = mv_all.data_ptr() + 4 * n * k, mi_all.data_ptr() + 8 * k
            j.out0, j.out1 = o0, o1
            cur[op] += 1
            calls.append((L.grns_max, (c.handle, a, ln, 1, o0, o1, None, 0, sp)))
    total = sum(lens)

    def per_call():
        for fn, args in calls:
            native.check(fn(*args))

    # plain per-call form (integer fast path), one call per job
    per_call()
    torch.cuda.synchronize()
    t_call = statistics.median(time_calls(per_call, max(2, steps // 2), stream, flush))
    # one persistent launch of every job, captured as a CUDA graph
    h = ctypes.c_void_p()
    native.check(L.grns_batch_create(c.handle, jobs, BATCH_JOBS, 1, ctypes.byref(h)))
    launch = lambda: native.check(L.grns_batch_launch(h, sp))  # noqa
    for _ in range(2):
        launch()
    torch.cuda.synchronize()
    t_batch = statistics.median(time_calls(launch, max(3, steps), stream, flush))
    L.grns_batch_destroy(h)
    names = {native.OP_CMP: "eval+cmp", native.OP_DIV: "div", native.OP_SCALE2POW: "scale2pow",
             native.OP_MAX: "max"}
    res = {
        "jobs": BATCH_JOBS, "numbers": total, "lengths": f"log-uniform [{BATCH_LEN[0]:g}, {BATCH_LEN[1]:g}]",
        "ops": "uniform over " + ", ".join(names[o] for o in op_choices) + "; AoS operand windows",
        "batched_Mnum_s": total / (t_batch * 1e-3) / 1e6, "batched_ms": t_batch,
        "per_call_Mnum_s": total / (t_call * 1e-3) / 1e6, "per_call_ms": t_call,
        "batched_vs_per_call": t_call / t_batch, "graph": True,
    }
    del X, Y, Dv, Sh, q_all, r_all, s_all, c_all, mv_all, mi_all
    torch.cuda.empty_cache()
    return res


# ---------------------------------------------------------------------------
# served stream: n = 32 and n = 64 contexts, Poisson arrivals, continuous batching

def bench_served(ctx_for, L, dev, stream, sp, P, seed):
    import random
    import torch
    import grns_gb300 as G
    from grns_gb300 import native
    from grns_gb300.serve import Server
    from grns_gb300.workload import S_X, S_Y
    c32, c64 = ctx_for(32), ctx_for(64)
    pool = SERVE_POOL
    X = torch.empty((32, pool), dtype=torch.int32, device=dev)
    Y = torch.empty_like(X)
    Dv = torch.empty_like(X)
    Sh = torch.empty(pool, dtype=torch.int32, device=dev)
    native.check(L.grns_gen_uniform(c32.handle, seed, S_X, pool, 0, P(X), sp))
    native.check(L.grns_gen_uniform(c32.handle, seed, S_Y, pool, 0, P(Y), sp))
    native.check(L.grns_gen_divisors(c32.handle, seed, pool, 0, P(Dv), sp))
    native.check(L.grns_gen_shifts(seed, pool, DMAX, P(Sh), sp))
    mb = G.mpint_bytes(64)
    MA = torch.empty(pool * mb, dtype=torch.uint8, device=dev)
    MC = torch.empty_like(MA)
    native.check(L.grns_gen_mpint(c64.handle, seed, pool, MP_BITS, P(MA), sp))
    native.check(L.grns_gen_mpint(c64.handle, seed + 1, pool, MP_BITS, P(MC), sp))
    X64 = torch.empty((64, pool), dtype=torch.int32, device=dev)
    native.check(L.grns_gen_uniform(c64.handle, seed, S_X, pool, 0, P(X64), sp))
    torch.cuda.synchronize()
    sv = Server(budget_bytes=SERVE_BUDGET, slots=4, max_jobs=256, admission_timeout_ms=0)
    i32, i64 = sv.add_context(c32), sv.add_context(c64)
    hX = sv.put(i32, X)
    hY = sv.put(i32, Y)
    hD = sv.put(i32, Dv)
    hS = sv.put(i32, Sh, kind=native.ARRAY_U32, count=pool)
    hMA = sv.put(i64, MA, kind=native.ARRAY_MPINT, count=pool)
    hMC = sv.put(i64, MC, kind=native.ARRAY_MPINT, count=pool)
    hX64 = sv.put(i64, X64)
    rng = random.Random(seed + 7)
    lens = log_uniform_lengths(rng, SERVE_REQS, *SERVE_LEN)
    kinds = [rng.choice(("cmp", "div", "scale2pow", "mpint_mul", "max")) for _ in lens]
    spec = {"cmp": (i32, hX, hY), "div": (i32, hX, hD), "scale2pow": (i32, hX, hS),
            "mpint_mul": (i64, hMA, hMC), "max": (i64, hX64, 0)}

    def run(rate):
        """submit the request list at Poisson times (rate requests/s, 0: all at once), wait for all"""
        sv.reset_stats()
        gaps = [rng.expovariate(rate) if rate else 0.0 for _ in lens]
        ids = []
        t0 = time.perf_counter()
        due = t0
        for ln, kd, g in zip(lens, kinds, gaps):
            due += g
            now = time.perf_counter()
            if due > now:
                time.sleep(due - now)
            ci, a, b = spec[kd]
            ids.append(sv.submit(kd, ci, a, b, count=ln))
        outs = []
        for rid in ids:
            st, o0, o1 = sv.wait(rid)
            if st != 0:
                raise RuntimeError(f"served request failed with status {st}")
            outs.append((o0, o1))
        wall = time.perf_counter() - t0
        stats = sv.stats()
        for o0, o1 in outs:
            for hnd in (o0, o1):
                if hnd:
                    sv.free(hnd)
        return wall, stats

    run(0)  # warm-up
    wall_all, st_all = run(0)
    # the same burst with a gathering window: free slots wait while requests keep arriving
    sv.set_gather_us(SERVE_GATHER_US)
    wall_g, st_g = run(0)
    sv.set_gather_us(0)
    total = sum(lens)
    cap_rps = len(lens) / wall_all
    sweeps = []
    for frac in SERVE_LOADS:
        wall, st = run(frac * cap_rps)
        sweeps.append({"offered_load": frac, "rate_req_s": frac * cap_rps, "Mnum_s": total / wall / 1e6,
                       "p50_ms": st["p50_us"] / 1e3, "p99_ms": st["p99_us"] / 1e3,
                       "mean_jobs_per_launch": st["mean_jobs_per_launch"], "launches": st["launches"]})
    sv.close()
    # the same requests as plain per-request calls, one after another
    outs = {"cmp": torch.empty(pool, dtype=torch.int32, device=dev), "q": torch.empty_like(X),
            "r": torch.empty_like(X), "s": torch.empty_like(X), "m": torch.empty_like(MA),
            "mv": torch.empty(64, dtype=torch.int32, device=dev), "mi": torch.empty(1, dtype=torch.int64, device=dev)}
    svc = []
    for ln, kd in zip(lens, kinds):
        if kd == "cmp":
            xs, ys = X[:, :ln].contiguous(), Y[:, :ln].contiguous()
            f = lambda: native.check(L.grns_cmp(c32.handle, P(xs), P(ys), ln, 0, P(outs["cmp"]), None, sp))  # noqa
        elif kd == "div":
            xs, ys = X[:, :ln].contiguous(), Dv[:, :ln].contiguous()
            f = lambda: native.check(L.grns_div(c32.handle, P(xs), P(ys), ln, 0, P(outs["q"]), P(outs["r"]),  # noqa
                                                None, sp))
        elif kd == "scale2pow":
            xs = X[:, :ln].contiguous()
            f = lambda: native.check(L.grns_scale2pow(c32.handle, P(xs), P(Sh), 0, ln, 0, P(outs["s"]),  # noqa
                                                      None, sp))
        elif kd == "mpint_mul":
            f = lambda: native.check(L.grns_mpint_mul(c64.handle, P(MA), P(MC), ln, P(outs["m"]), None, sp))  # noqa
        else:
            xs = X64[:, :ln].contiguous()
            f = lambda: native.check(L.grns_max(c64.handle, P(xs), ln, 0, P(outs["mv"]), P(outs["mi"]),  # noqa
                                                None, 0, sp))
        f()
        svc.append(time_calls(f, 1, stream)[0])
    svc_sorted = sorted(svc)
    t_plain = sum(svc)
    return {
        "requests": len(lens), "numbers": total, "lengths": f"log-uniform [{SERVE_LEN[0]:g}, {SERVE_LEN[1]:g}]",
        "ops": "uniform over eval+cmp, div, scale2pow (n=32), mp_int mul, max (n=64)",
        "all_at_once": {"Mnum_s": total / wall_all / 1e6, "p50_ms": st_all["p50_us"] / 1e3,
                        "p99_ms": st_all["p99_us"] / 1e3, "mean_jobs_per_launch": st_all["mean_jobs_per_launch"]},
        "all_at_once_gathered": {"gather_us": SERVE_GATHER_US, "Mnum_s": total / wall_g / 1e6,
                                 "p50_ms": st_g["p50_us"] / 1e3, "p99_ms": st_g["p99_us"] / 1e3,
                                 "mean_jobs_per_launch": st_g["mean_jobs_per_launch"]},
        "poisson": sweeps,
        "per_request_plain": {"Mnum_s": total / (t_plain * 1e-3) / 1e6,
                              "p50_ms": svc_sorted[len(svc) // 2],
                              "p99_ms": svc_sorted[min(len(svc) - 1, int(0.99 * len(svc)))],
                              "note": "service time of each call alone (no queueing), device events"},
    }


# ---------------------------------------------------------------------------

def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="grns_gb300")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--quick", action="store_true", help="headline workload only")
    ap.add_argument("--pairs", type=int, default=PAIRS, help="numbers per op (profiling cases use fewer)")
    ap.add_argument("--flush", action="store_true", help="profiling mode: flush L2 (256 MiB write) before each call")
    ap.add_argument("--n", type=int, default=None,
                    help="profiling: moduli count of the --only case (greedy 30-bit moduli), e.g. 128 or 256")
    ap.add_argument("--mp-op", default="mul", choices=["add", "sub", "mul"], help="profiling: the mpint64 operation")
    ap.add_argument("--eval-split", type=int, default=None,
                    help="profiling: eighths of the evaluation's warps on the FP64 pipe (grns_ctx_set_eval_split)")
    ap.add_argument("--only", choices=["div", "scale", "cmp32", "cmp8", "max64", "eval32", "evtight32", "mpint64",
                                           "mpdiv32", "tobin32", "frombin32", "tobin64", "mrc32"], default=None,
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

    ctxs = {}

    def ctx_for(n):
        if n not in ctxs:
            ctxs[n] = G.RNSContext(greedy(n))
        return ctxs[n]

    ctx = ctx_for(N32)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    seed = SEED + rank
    peak, peak_kind = load_peaks()

    # ---- headline: div + scale2pow at n = 32, inputs resident in HBM (SoA) ----
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

    # the two operations of a step are independent: the scaling runs on a second
    # stream beside the division, so it fills the SMs the division leaves idle
    # (its tails, the sort between its passes); the step ends when both have
    # finished
    s_scale = torch.cuda.Stream()
    sp_scale = ctypes.c_void_p(s_scale.cuda_stream)
    fork, join = torch.cuda.Event(), torch.cuda.Event()

    def step(timers=None):
        e0, e1, e2, e3, e4, e5 = (timers or (None,) * 6)
        if e0: e0.record(stream)
        fork.record(stream)
        s_scale.wait_event(fork)
        if e3: e3.record(s_scale)
        native.check(L.grns_scale2pow(ctx.handle, P(xs), P(D), 0, PAIRS, 0, P(so), None, sp_scale))
        if e4: e4.record(s_scale)
        join.record(s_scale)
        if e1: e1.record(stream)
        native.check(L.grns_div(ctx.handle, P(x), P(d), PAIRS, 0, P(q), P(r), None, sp))
        if e2: e2.record(stream)
        stream.wait_event(join)
        if e5: e5.record(stream)

    step_ms, div_ms, scale_ms = [], [], []
    with Clocks(local) as clk:
        # warm-up: at least W steps and at least WARMUP_SECONDS, so the timed steps start
        # after the clock sampler has started and the GPU has settled
        t0 = time.perf_counter()
        done = 0
        while done < args.warmup or time.perf_counter() - t0 < WARMUP_SECONDS:
            step()
            torch.cuda.synchronize()
            done += 1
        for _ in range(args.steps):
            flush.zero_()
            t = tuple(_ev() for _ in range(6))
            step(t)
            torch.cuda.synchronize()
            div_ms.append(t[1].elapsed_time(t[2]))     # division, on its stream (sharing the GPU)
            scale_ms.append(t[3].elapsed_time(t[4]))   # scaling, on its stream
            step_ms.append(t[0].elapsed_time(t[5]))    # the whole step
        # ---- end to end through the C ABI's host-buffer forms (pinned host arrays), every
        # copy inside the timed region: grns_div_host and grns_scale2pow_host pipeline their
        # chunks' copies with their kernels; the two operations run on two streams, so one's
        # transfers also overlap the other's kernels ----
        hx = x.cpu().pin_memory(); hd = d.cpu().pin_memory(); hxs = xs.cpu().pin_memory(); hD = D.cpu().pin_memory()
        hq = torch.empty_like(hx).pin_memory(); hr = torch.empty_like(hx).pin_memory()
        hso = torch.empty_like(hx).pin_memory()
        s2 = torch.cuda.Stream()
        sp2 = ctypes.c_void_p(s2.cuda_stream)
        e2e_ms = []
        for i in range(args.warmup + args.steps):
            flush.zero_()
            a, b, c2 = _ev(), _ev(), _ev()
            a.record(stream)
            s2.wait_event(a)
            native.check(L.grns_div_host(ctx.handle, P(hx), P(hd), PAIRS, 0, P(hq), P(hr), None, 0, sp))
            native.check(L.grns_scale2pow_host(ctx.handle, P(hxs), P(hD), 0, PAIRS, 0, P(hso), None, 0, sp2))
            c2.record(s2)
            stream.wait_event(c2)
            b.record(stream)
            torch.cuda.synchronize()
            if i >= args.warmup:
                e2e_ms.append(a.elapsed_time(b))
        e2e_ok = torch.equal(hq, q.cpu()) and torch.equal(hr, r.cpu()) and torch.equal(hso, so.cpu())
    ms, value = aggregate(sum(step_ms) / args.steps, 2 * PAIRS, world)
    _, e2e = aggregate(sum(e2e_ms) / args.steps, 2 * PAIRS, world)
    h2d = 4 * (x.numel() * 3 + D.numel())
    d2h = 4 * x.numel() * 3
    del hx, hd, hxs, hD, hq, hr, hso

    # ---- the other workloads (rank 0 measurements, in the same JSON record) ----
    extra, workloads = {}, {}
    if not args.quick and rank == 0:
        with Clocks(local) as clk2:
            extra.update(bench_eval_cmp(ctx_for, L, dev, stream, sp, P, seed, args.steps, flush, peak))
            torch.cuda.empty_cache()
            extra.update(bench_mpint_max(ctx_for, L, dev, stream, sp, P, seed, args.steps, flush, peak))
            torch.cuda.empty_cache()
            extra.update(bench_next_ops(ctx_for, L, dev, stream, sp, P, seed, args.steps, flush, peak))
            torch.cuda.empty_cache()
            workloads["batched_uneven_n32"] = bench_batched(ctx_for, L, dev, stream, sp, P, seed, args.steps, flush)
            torch.cuda.empty_cache()
            workloads["served_stream_n32_n64"] = bench_served(ctx_for, L, dev, stream, sp, P, seed)
            torch.cuda.empty_cache()
        extra["clocks_other_workloads"] = clk2.summary()

    div_avg = statistics.mean(div_ms)
    alg_bytes = (4 * 4 * N32) * PAIRS  # x, d read; q, r written
    achieved = alg_bytes / (div_avg * 1e-3) / 1e9
    line = {
        "metric": "RNS Mnum/s div+scale2pow (960-bit, n=32)", "value": value, "unit": "Mnum/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32+u64",
        "data": "synthetic (seeded splitmix64 generator, device-generated)",
        "config": {"workload": "div 2^18 pairs (divisor bits uniform in [1,959]) + scale2pow 2^18 numbers "
                               "(D uniform in [1,900]), n=32 greedy moduli from 2^30-1, SoA",
                   "streams": "the division and the scaling of a step on two streams at once (independent); "
                              "kernels_ms are each one's span on its stream while they share the GPU",
                   "l2": "flushed (256 MiB write) between timed steps", "parallelism": f"replicas x{world}"},
        "roofline": {"bound": "hbm", "kernel": "k_div_a<32> + k_div_rows<32> + k_div_place + k_div_b<32> + k_div_out<32> "
                                               "(one division call)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "traffic": DIV_TRAFFIC_BYTES,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of the five launches of "
                                       "one call, each captured cold, profiles/k_div_n32_262144pairs.md",
                     "note": "division is integer-pipe bound (48-bit digit steps); the HBM-bound kernels "
                             "(eval, cmp, max, mp_int) carry their own fractions in extra"},
        "kernels_ms": {"division": div_avg, "k_scale_warp": statistics.mean(scale_ms),
                       "division_steps": [round(v, 4) for v in div_ms],
                       "k_scale_warp_steps": [round(v, 4) for v in scale_ms]},
        "e2e": {"value": e2e, "unit": "Mnum/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "api": "grns_div_host + grns_scale2pow_host (pinned host arrays, chunked copy/compute "
                       "overlap), the two on two streams", "matches_device_results": e2e_ok},
        "gpu_launches": 6 * args.steps,  # per step: k_div_a, k_div_rows, k_div_place, k_div_b, k_div_out, k_scale_warp
        "extra": extra,
        "workloads": workloads,
    }
    line["clocks"] = clk.summary()
    if rank == 0 and not args.no_cpu:
        v, cores, desc, ops = cpu_baseline()
        line["cpu_baseline"] = {"value": v, "unit": "Mnum/s", "cores": cores, "kind": "port", "sample": desc,
                                "ops": ops}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
