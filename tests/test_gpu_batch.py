"""GPU: batched execution (one persistent launch for many uneven jobs, CUDA
graph replay, n-threaded vs serial schedules, autotuner).  Every job's
outputs must equal the per-call entry points' outputs bit for bit, and a
seeded sample of every job's outputs must equal the oracle's (intervals,
mp_int records) and exact big-integer arithmetic (signs, quotients and
remainders, scaled values, the maximum and its index) -- tests/jobcheck.py."""
import ctypes
import random

import pytest

from oracle.oracle import Oracle, greedy_moduli
from tests.jobcheck import check_job

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def L():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from grns_gb300 import native
    return native.lib(build_if_missing=True)


def P(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def make_jobs(ctx, n, rng, njobs, stream):
    """random ops and lengths (including empty and tiny jobs), device-generated inputs"""
    from grns_gb300 import native
    from grns_gb300 import mpint_bytes
    L = native.lib()
    jobs, bufs = [], []
    for t in range(njobs):
        op = rng.choice([0, 1, 2, 3, 4, 5, 6, 7, 8])
        count = rng.choice([0, 1, 3, 31, 100, 1000, 5000, 20000 if op not in (2, 3, 8) else 2000])
        layout = rng.choice([0, 1]) if op < 5 else 0
        j = native.Job()
        j.op, j.layout, j.count = op, layout, count
        if op >= 5:
            nb = mpint_bytes(n)
            a = torch.zeros(max(1, count) * nb, dtype=torch.uint8, device="cuda")
            b = torch.zeros_like(a)
            if count:  # signed operands whose products stay below M, evaluations from the device path;
                # division: dividends of nearly the full range, divisors of half of it
                lg = L.grns_ctx_log2(ctx)
                bits_a, bits_b = (lg - 8, lg // 2) if op == 8 else (lg // 2 - 10, lg // 2 - 10)
                native.check(L.grns_gen_mpint(ctx, 70 + t, count, bits_a, P(a), stream))
                native.check(L.grns_gen_mpint(ctx, 170 + t, count, bits_b, P(b), stream))
            o0 = torch.zeros_like(a)
            j.a, j.b, j.out0 = a.data_ptr(), b.data_ptr(), o0.data_ptr()
            bufs.append((op, count, layout, a, b, o0, None))
        else:
            shape = (n, max(1, count)) if layout == 0 else (max(1, count), n)
            x = torch.empty(shape, dtype=torch.int32, device="cuda")
            y = torch.empty_like(x)
            if count:
                tmp = torch.empty((n, count), dtype=torch.int32, device="cuda")
                native.check(L.grns_gen_uniform(ctx, 7 + t, 1, count, 0, P(tmp), stream))
                x.copy_(tmp if layout == 0 else tmp.t())
                if op == 2:
                    native.check(L.grns_gen_divisors(ctx, 7 + t, count, 0, P(tmp), stream))
                else:
                    native.check(L.grns_gen_uniform(ctx, 7 + t, 2, count, 0, P(tmp), stream))
                y.copy_(tmp if layout == 0 else tmp.t())
            D = None
            if op == 3:
                D = torch.randint(1, 900, (max(1, count),), dtype=torch.int32, device="cuda")
            if op == 0:
                o0 = torch.zeros(max(1, count) * 32, dtype=torch.uint8, device="cuda")
                o1 = None
            elif op == 1:
                o0 = torch.zeros(max(1, count), dtype=torch.int32, device="cuda")
                o1 = None
            elif op == 4:
                o0 = torch.zeros(n, dtype=torch.int32, device="cuda")
                o1 = torch.zeros(1, dtype=torch.int64, device="cuda")
            else:
                o0 = torch.zeros_like(x)
                o1 = torch.zeros_like(x) if op == 2 else None
            j.a = x.data_ptr()
            j.b = D.data_ptr() if op == 3 else (y.data_ptr() if op in (1, 2) else None)
            j.out0 = o0.data_ptr()
            j.out1 = o1.data_ptr() if o1 is not None else None
            bufs.append((op, count, layout, x, y if op != 3 else D, o0, o1))
        jobs.append(j)
    arr = (native.Job * len(jobs))(*jobs)
    return arr, bufs


def reference_outputs(L, ctx, n, bufs, stream):
    """the same jobs through the per-call entry points"""
    from grns_gb300 import native
    outs = []
    for op, count, layout, a, b, o0, o1 in bufs:
        r0 = torch.zeros_like(o0)
        r1 = torch.zeros_like(o1) if o1 is not None else None
        if count:
            if op == 0:
                native.check(L.grns_eval(ctx, P(a), count, layout, P(r0), None, stream))
            elif op == 1:
                native.check(L.grns_cmp(ctx, P(a), P(b), count, layout, P(r0), None, stream))
            elif op == 2:
                native.check(L.grns_div(ctx, P(a), P(b), count, layout, P(r0), P(r1), None, stream))
            elif op == 3:
                native.check(L.grns_scale2pow(ctx, P(a), P(b), 0, count, layout, P(r0), None, stream))
            elif op == 4:
                native.check(L.grns_max(ctx, P(a), count, layout, P(r0), P(r1), None, 0, stream))
            else:
                fn = {5: L.grns_mpint_add, 6: L.grns_mpint_sub, 7: L.grns_mpint_mul, 8: L.grns_mpint_div}[op]
                native.check(fn(ctx, P(a), P(b), count, P(r0), None, stream))
        elif op == 4:
            r1.fill_(-1)
        outs.append((r0, r1))
    return outs


@pytest.mark.parametrize("n", [8, 32])
@pytest.mark.parametrize("coop", [0, 1])
@pytest.mark.parametrize("graph", [0, 1])
def test_batch_matches_per_call(L, n, coop, graph):
    from grns_gb300 import native
    ctx = ctypes.c_void_p()
    mods = (ctypes.c_int32 * n)(*greedy_moduli(n))
    native.check(L.grns_ctx_create(mods, n, ctypes.byref(ctx)))
    s = torch.cuda.Stream()
    sp = ctypes.c_void_p(s.cuda_stream)
    orc = Oracle(greedy_moduli(n))
    try:
        for op in (1, 4):
            sc = native.Schedule(coop, 256 if n == 8 else 1024)
            native.check(L.grns_ctx_set_schedule(ctx, op, ctypes.byref(sc)))
        rng = random.Random(n * 10 + coop * 2 + graph)
        with torch.cuda.stream(s):
            jobs, bufs = make_jobs(ctx, n, rng, 36, sp)
            want = reference_outputs(L, ctx, n, bufs, sp)
        b = ctypes.c_void_p()
        native.check(L.grns_batch_create(ctx, jobs, len(jobs), graph, ctypes.byref(b)))
        try:
            for rep in range(2):  # second launch replays the graph and must reset the counters
                for (_, count, _, _, _, o0, o1) in bufs:
                    o0.zero_()
                    if o1 is not None:
                        o1.zero_()
                native.check(L.grns_batch_launch(b, sp))
                s.synchronize()
                for t, ((op, count, layout, a, bb, o0, o1), (r0, r1)) in enumerate(zip(bufs, want)):
                    if count == 0 and op != 4:
                        continue
                    assert torch.equal(o0, r0), (t, op, count, layout)
                    if o1 is not None:
                        assert torch.equal(o1, r1), (t, op, count, layout)
                    if rep == 0:
                        check_job(orc, op, count, layout, a, bb, o0, o1, seed=t)
        finally:
            L.grns_batch_destroy(b)
    finally:
        L.grns_ctx_destroy(ctx)


def test_batch_update_replays_graph_on_new_data(L):
    from grns_gb300 import native
    n = 8
    ctx = ctypes.c_void_p()
    mods = (ctypes.c_int32 * n)(*greedy_moduli(n))
    native.check(L.grns_ctx_create(mods, n, ctypes.byref(ctx)))
    s = torch.cuda.Stream()
    sp = ctypes.c_void_p(s.cuda_stream)
    try:
        cnt = 10000
        xs = [torch.empty((n, cnt), dtype=torch.int32, device="cuda") for _ in range(4)]
        for i, x in enumerate(xs):
            native.check(L.grns_gen_uniform(ctx, 100 + i, 1, cnt, 0, P(x), sp))
        out = torch.zeros(cnt, dtype=torch.int32, device="cuda")
        j = native.Job(op=1, layout=0, count=cnt, a=xs[0].data_ptr(), b=xs[1].data_ptr(), out0=out.data_ptr())
        arr = (native.Job * 1)(j)
        b = ctypes.c_void_p()
        native.check(L.grns_batch_create(ctx, arr, 1, 1, ctypes.byref(b)))
        ref = torch.zeros_like(out)
        for pair in ((0, 1), (2, 3)):
            arr[0].a, arr[0].b = xs[pair[0]].data_ptr(), xs[pair[1]].data_ptr()
            native.check(L.grns_batch_update(b, arr, 1))
            native.check(L.grns_batch_launch(b, sp))
            native.check(L.grns_cmp(ctx, P(xs[pair[0]]), P(xs[pair[1]]), cnt, 0, P(ref), None, sp))
            s.synchronize()
            assert torch.equal(out, ref)
        bad = native.Job(op=2, layout=0, count=cnt, a=xs[0].data_ptr(), b=xs[1].data_ptr(), out0=out.data_ptr())
        assert L.grns_batch_update(b, (native.Job * 1)(bad), 1) == 1  # shape change refused
        L.grns_batch_destroy(b)
    finally:
        L.grns_ctx_destroy(ctx)


def test_autotune_and_cache(L, tmp_path):
    from grns_gb300 import native
    n = 32
    ctx = ctypes.c_void_p()
    mods = (ctypes.c_int32 * n)(*greedy_moduli(n))
    native.check(L.grns_ctx_create(mods, n, ctypes.byref(ctx)))
    try:
        cache = str(tmp_path / "tune.txt").encode()
        for op in (1, 4, 2):
            sc = native.Schedule()
            ms = ctypes.c_double()
            native.check(L.grns_autotune(ctx, op, 20000 if op != 2 else 4000, cache, ctypes.byref(sc), ctypes.byref(ms)))
            assert sc.chunk >= 32 and ms.value > 0
            got = native.Schedule()
            native.check(L.grns_ctx_get_schedule(ctx, op, ctypes.byref(got)))
            assert (got.coop, got.chunk) == (sc.coop, sc.chunk)
        ctx2 = ctypes.c_void_p()
        native.check(L.grns_ctx_create(mods, n, ctypes.byref(ctx2)))
        applied = ctypes.c_int()
        native.check(L.grns_autotune_load(ctx2, cache, ctypes.byref(applied)))
        assert applied.value == 3
        L.grns_ctx_destroy(ctx2)
    finally:
        L.grns_ctx_destroy(ctx)
