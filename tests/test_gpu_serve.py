"""GPU: serving -- device-resident arrays, continuous batching of a request
stream over two resident moduli sets (n = 32 and n = 64), admission by HBM
footprint, cached evaluations, latency stats.  Every request's result must be
the same alone (through the per-call entry points, and alone through the
server) and inside the mix, and a seeded sample of it must equal the oracle's
and exact big-integer arithmetic (tests/jobcheck.py)."""
import ctypes
import random

import numpy as np
import pytest

from oracle.oracle import Oracle, greedy_moduli
from tests.jobcheck import check_job

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def env():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import grns_gb300 as G
    from grns_gb300 import native
    native.lib(build_if_missing=True)
    ctxs = {n: G.RNSContext(greedy_moduli(n)) for n in (32, 64)}
    return G, native, ctxs


def P(t):
    return ctypes.c_void_p(t.data_ptr())


def gen(native, ctx, count, stream_id, seed, divisors=False):
    x = torch.empty((ctx.n, count), dtype=torch.int32, device="cuda")
    fn = native.lib().grns_gen_divisors if divisors else None
    if divisors:
        native.check(fn(ctx.handle, seed, count, 0, P(x), None))
    else:
        native.check(native.lib().grns_gen_uniform(ctx.handle, seed, stream_id, count, 0, P(x), None))
    torch.cuda.synchronize()
    return x


def per_call(native, ctx, op, x, y, count):
    """the op through the per-call entry points on the first `count` numbers"""
    L = native.lib()
    if op == "mpint_mul":
        from grns_gb300 import mpint_bytes
        nb = count * mpint_bytes(ctx.n)
        return [ctx.mpint_mul(x[:nb], y[:nb])]
    xs = x[:, :count].contiguous()
    ys = y[:, :count].contiguous() if y is not None and y.dim() == 2 else y
    if op == "eval":
        o = torch.empty(count * 32, dtype=torch.uint8, device="cuda")
        native.check(L.grns_eval(ctx.handle, P(xs), count, 0, P(o), None, None))
        return [o]
    if op == "cmp":
        o = torch.empty(count, dtype=torch.int32, device="cuda")
        native.check(L.grns_cmp(ctx.handle, P(xs), P(ys), count, 0, P(o), None, None))
        return [o]
    if op == "div":
        q, r = torch.empty_like(xs), torch.empty_like(xs)
        native.check(L.grns_div(ctx.handle, P(xs), P(ys), count, 0, P(q), P(r), None, None))
        return [q, r]
    if op == "scale2pow":
        o = torch.empty_like(xs)
        D = y[:count].contiguous()
        native.check(L.grns_scale2pow(ctx.handle, P(xs), P(D), 0, count, 0, P(o), None, None))
        return [o]
    if op == "max":
        v = torch.zeros(ctx.n, dtype=torch.int32, device="cuda")
        i = torch.zeros(1, dtype=torch.int64, device="cuda")
        native.check(L.grns_max(ctx.handle, P(xs), count, 0, P(v), P(i), None, 0, None))
        return [v, i]
    raise ValueError(op)


def check_served(A, op, count, got, seed):
    """a served result (the bytes server_bytes returns) against the oracle"""
    n = A["ctx"].n
    raw = np.frombuffer(got, np.uint8)
    code = {"eval": 0, "cmp": 1, "div": 2, "scale2pow": 3, "max": 4, "mpint_mul": 7}[op]
    if op == "max":
        check_job(A["orc"], 4, count, 0, A["x"], None, raw[:4 * n], raw[4 * n:], seed=seed)
    elif op == "div":
        half = len(raw) // 2
        check_job(A["orc"], 2, count, 0, A["x"], A["d"], raw[:half], raw[half:], seed=seed)
    elif op == "mpint_mul":
        check_job(A["orc"], 7, count, 0, A["ma"], A["mc"], raw, None, seed=seed)
    else:
        b = {"cmp": A["y"], "scale2pow": A["D"]}.get(op)
        check_job(A["orc"], code, count, 0, A["x"], b, raw, None, seed=seed)


def as_bytes(ts):
    torch.cuda.synchronize()
    return b"".join(t.cpu().numpy().tobytes() for t in ts)


def server_bytes(srv, rid, op, n):
    st, o0, o1 = srv.wait(rid)
    assert st == 0
    if op == "max":
        raw = srv.get(o0)
        off = ((4 * n + 7) // 8) * 8
        return raw[:4 * n].tobytes() + raw[off:off + 8].tobytes()
    out = srv.get(o0).tobytes()
    if o1:
        out += srv.get(o1).tobytes()
    return out


@pytest.mark.parametrize("direct", [-1, 5000])
def test_results_alone_and_in_the_mix(env, direct):
    """direct = -1: every request inside the packed kernel; 5000: requests of
    5000 numbers or more (whole arrays for div and scale2pow) through the
    per-op kernels in the same launch rounds"""
    G, native, ctxs = env
    from grns_gb300.serve import Server
    srv = Server(slots=4, max_jobs=64, direct_min_count=direct)
    try:
        arrays = {}
        for n, ctx in ctxs.items():
            ci = srv.add_context(ctx)
            cnt = 60000 if n == 32 else 30000
            x = gen(native, ctx, cnt, 1, 100 + n)
            y = gen(native, ctx, cnt, 2, 100 + n)
            d = gen(native, ctx, cnt, 0, 200 + n, divisors=True)
            D = torch.randint(1, 900, (cnt,), dtype=torch.int32, device="cuda")
            mb = G.mpint_bytes(n)
            ma = torch.empty(cnt * mb, dtype=torch.uint8, device="cuda")
            mc = torch.empty_like(ma)
            bits = ctx.log2M // 2 - 10  # products stay below M
            native.check(native.lib().grns_gen_mpint(ctx.handle, 300 + n, cnt, bits, P(ma), None))
            native.check(native.lib().grns_gen_mpint(ctx.handle, 400 + n, cnt, bits, P(mc), None))
            torch.cuda.synchronize()
            arrays[n] = dict(ci=ci, ctx=ctx, x=x, y=y, d=d, D=D, ma=ma, mc=mc, cnt=cnt, orc=Oracle(ctx.moduli),
                             hx=srv.put(ci, x), hy=srv.put(ci, y), hd=srv.put(ci, d),
                             hD=srv.put(ci, D, kind=native.ARRAY_U32),
                             hma=srv.put(ci, ma.view(cnt, mb), kind=native.ARRAY_MPINT),
                             hmc=srv.put(ci, mc.view(cnt, mb), kind=native.ARRAY_MPINT))
        rng = random.Random(3)
        reqs = []
        for t in range(60):
            n = rng.choice([32, 64])
            A = arrays[n]
            op = rng.choice(["eval", "cmp", "div", "scale2pow", "max", "mpint_mul"])
            count = rng.choice([1, 7, 100, 1000, 10000, A["cnt"]]) if op not in ("div",) else \
                rng.choice([1, 50, 2000, A["cnt"]])
            a = A["hma"] if op == "mpint_mul" else A["hx"]
            b = {"cmp": A["hy"], "div": A["hd"], "scale2pow": A["hD"], "mpint_mul": A["hmc"]}.get(op, 0)
            reqs.append((n, op, count, a, b))
        # the mix: everything submitted back to back (they overlap on the device)
        ids = [srv.submit(op, arrays[n]["ci"], a, b, count) for (n, op, count, a, b) in reqs]
        mixed = [server_bytes(srv, rid, op, n) for rid, (n, op, count, a, b) in zip(ids, reqs)]
        st = srv.stats()
        assert st["completed"] == len(reqs) and st["rejected"] == 0
        assert 0 < st["p50_us"] <= st["p99_us"]
        assert st["launches"] < len(reqs)  # requests were packed into shared launches
        # each alone: through the server with nothing else queued, and through the per-call API
        for t, ((n, op, count, a, b), got) in enumerate(zip(reqs, mixed)):
            A = arrays[n]
            alone = server_bytes(srv, srv.submit(op, A["ci"], a, b, count), op, n)
            assert alone == got, (n, op, count)
            y = {"cmp": A["y"], "div": A["d"], "scale2pow": A["D"], "mpint_mul": A["mc"]}.get(op)
            x = A["ma"] if op == "mpint_mul" else A["x"]
            assert as_bytes(per_call(native, A["ctx"], op, x, y, count)) == got, (n, op, count)
            # and the oracle / exact arithmetic on a sample of the mixed result
            check_served(A, op, count, got, seed=t)
    finally:
        srv.close()


def test_gathering_window_packs_a_burst(env):
    """with gather_us set, a burst submitted back to back shares few launches
    (free slots wait while requests keep arriving) and every result is the
    per-call API's"""
    G, native, ctxs = env
    from grns_gb300.serve import Server
    ctx = ctxs[32]
    srv = Server(slots=4, max_jobs=256, gather_us=5000)  # a window well above the gaps between submissions
    try:
        ci = srv.add_context(ctx)
        cnt = 5000
        x = gen(native, ctx, cnt, 1, 501)
        y = gen(native, ctx, cnt, 2, 502)
        torch.cuda.synchronize()
        hx, hy = srv.put(ci, x), srv.put(ci, y)
        counts = [1 + 97 * t for t in range(40)]
        ids = [srv.submit("cmp", ci, hx, hy, c) for c in counts]
        got = [server_bytes(srv, rid, "cmp", 32) for rid in ids]
        st = srv.stats()
        assert st["completed"] == len(ids) and st["mean_jobs_per_launch"] >= 8
        for c, g in zip(counts, got):
            assert as_bytes(per_call(native, ctx, "cmp", x, y, c)) == g, c
    finally:
        srv.close()


def test_cached_evaluations_and_admission(env):
    G, native, ctxs = env
    from grns_gb300.serve import Server
    ctx = ctxs[32]
    cnt = 50000
    x = gen(native, ctx, cnt, 1, 7)
    y = gen(native, ctx, cnt, 2, 7)
    y[:, ::5] = x[:, ::5]
    srv = Server(slots=2)
    try:
        ci = srv.add_context(ctx)
        hx, hy = srv.put(ci, x), srv.put(ci, y)
        plain = server_bytes(srv, srv.submit("cmp", ci, hx, hy), "cmp", 32)
        for h in (hx, hy):
            st, ev, _ = srv.wait(srv.submit("eval", ci, h))
            assert st == 0
        cached = server_bytes(srv, srv.submit("cmp", ci, hx, hy), "cmp", 32)
        assert cached == plain
    finally:
        srv.close()
    # a budget that fits the operands but not a division's outputs next to them: the division
    # is refused after the admission timeout (never hangs), and the queue moves on
    small = Server(budget_bytes=2 * 4 * 32 * cnt + 4 * cnt + (1 << 20), slots=1, admission_timeout_ms=300)
    try:
        ci = small.add_context(ctx)
        hx, hy = small.put(ci, x), small.put(ci, y)
        st, _, _ = small.wait(small.submit("div", ci, hx, hy), timeout_us=30_000_000)
        assert st == 6  # GRNS_ERR_REJECTED
        st, o0, _ = small.wait(small.submit("cmp", ci, hx, hy), timeout_us=30_000_000)
        assert st == 0
    finally:
        small.close()


def test_failures_are_reported_not_fatal(env):
    """host-side fault injection: a request cancelled while it waits for memory,
    allocations beyond a hard cap, a bounded wait that runs out, and a
    corrupted request descriptor -- each reported with its status while the
    server goes on serving"""
    G, native, ctxs = env
    from grns_gb300.serve import Server
    ctx = ctxs[32]
    cnt = 40000
    x = gen(native, ctx, cnt, 1, 11)
    y = gen(native, ctx, cnt, 2, 11)
    operands = 2 * 4 * 32 * cnt
    # budget fits the operands and a comparison's output, not a division's: the division waits
    srv = Server(budget_bytes=operands + 8 * cnt + (1 << 20), slots=1, admission_timeout_ms=20000)
    try:
        ci = srv.add_context(ctx)
        hx, hy = srv.put(ci, x), srv.put(ci, y)
        rid = srv.submit("div", ci, hx, hy)
        srv.cancel(rid)
        st, _, _ = srv.wait(rid, timeout_us=5_000_000)
        assert st == 9  # GRNS_ERR_CANCELLED
        srv.cancel(rid)  # already finished: no-op
        st, o0, _ = srv.wait(srv.submit("cmp", ci, hx, hy), timeout_us=30_000_000)
        assert st == 0
        # a corrupted descriptor (unknown operand handle) is refused at submission
        with pytest.raises(G.GrnsError):
            srv.submit("cmp", ci, hx, 987654321)
    finally:
        srv.close()
    # a hard allocation cap: the operands fit, a division's outputs do not
    capped = Server(alloc_cap_bytes=operands + 8 * cnt + (1 << 20), slots=2)
    try:
        ci = capped.add_context(ctx)
        hx, hy = capped.put(ci, x), capped.put(ci, y)
        st, _, _ = capped.wait(capped.submit("div", ci, hx, hy), timeout_us=30_000_000)
        assert st == 4  # GRNS_ERR_OUT_OF_MEMORY
        with pytest.raises(G.GrnsError) as e:
            capped.put(ci, x)
        assert e.value.status == 4
        st, _, _ = capped.wait(capped.submit("cmp", ci, hx, hy), timeout_us=30_000_000)
        assert st == 0
    finally:
        capped.close()
    # a bounded wait that runs out reports GRNS_ERR_TIMEOUT; the request still completes
    srv = Server(slots=1)
    try:
        ci = srv.add_context(ctx)
        big = gen(native, ctx, 1 << 18, 3, 12)
        d = gen(native, ctx, 1 << 18, 4, 12, divisors=True)
        hb, hd = srv.put(ci, big), srv.put(ci, d)
        rid = srv.submit("div", ci, hb, hd)
        with pytest.raises(G.GrnsError) as e:
            srv.wait(rid, timeout_us=1)
        assert e.value.status == 5
        st, _, _ = srv.wait(rid, timeout_us=60_000_000)
        assert st == 0
    finally:
        srv.close()


def test_served_mpint_division(env):
    """mp_int division requests (GRNS_OP_MPINT_DIV) next to packed requests:
    the same records as grns_mpint_div"""
    G, native, ctxs = env
    from grns_gb300.serve import Server
    ctx = ctxs[32]
    cnt = 20000
    mb = G.mpint_bytes(32)
    ma = torch.empty(cnt * mb, dtype=torch.uint8, device="cuda")
    mc = torch.empty_like(ma)
    native.check(native.lib().grns_gen_mpint(ctx.handle, 5, cnt, 900, P(ma), None))
    native.check(native.lib().grns_gen_mpint(ctx.handle, 6, cnt, 450, P(mc), None))
    torch.cuda.synchronize()
    want = ctx.mpint_div(ma, mc).cpu().numpy().tobytes()
    x = gen(native, ctx, cnt, 1, 9)
    srv = Server(slots=2)
    try:
        ci = srv.add_context(ctx)
        ha = srv.put(ci, ma.view(cnt, mb), kind=native.ARRAY_MPINT)
        hc = srv.put(ci, mc.view(cnt, mb), kind=native.ARRAY_MPINT)
        hx = srv.put(ci, x)
        rids = [srv.submit("eval", ci, hx), srv.submit("mpint_div", ci, ha, hc), srv.submit("mpint_div", ci, ha, hc, 777)]
        outs = [srv.wait(r) for r in rids]
        assert all(st == 0 for st, _, _ in outs)
        assert srv.get(outs[1][1]).tobytes() == want
        assert srv.get(outs[2][1]).tobytes() == want[:777 * mb]
    finally:
        srv.close()


def test_free_waits_for_pending_readers(env):
    """freeing an operand and its cached evaluation right after submitting
    requests that read them: each free returns OK once those requests have
    finished, the results equal the per-call API's, and the freed handles are
    gone (get fails)"""
    G, native, ctxs = env
    from grns_gb300.serve import Server
    ctx = ctxs[32]
    cnt = 1 << 17
    x = gen(native, ctx, cnt, 1, 21)
    y = gen(native, ctx, cnt, 2, 21)
    d = gen(native, ctx, cnt, 0, 22, divisors=True)
    srv = Server(slots=2)
    try:
        ci = srv.add_context(ctx)
        hx, hy, hd = srv.put(ci, x), srv.put(ci, y), srv.put(ci, d)
        evs = []
        for h in (hx, hy):
            st, ev, _ = srv.wait(srv.submit("eval", ci, h))
            assert st == 0
            evs.append(ev)
        # a long division first, so the comparison (reading the cached evaluations) is still pending
        r_div = srv.submit("div", ci, hx, hd)
        r_cmp = srv.submit("cmp", ci, hx, hy)
        for h in (evs[0], hx, evs[1]):  # operand and evaluations freed at once
            srv.free(h)
        for h in (evs[0], hx, evs[1]):
            with pytest.raises(G.GrnsError):
                srv.get(h)
        st, c0, _ = srv.wait(r_cmp)
        assert st == 0
        st, q0, r0 = srv.wait(r_div)
        assert st == 0
        assert srv.get(c0).tobytes() == as_bytes(per_call(native, ctx, "cmp", x, y, cnt))
        assert srv.get(q0).tobytes() + srv.get(r0).tobytes() == as_bytes(per_call(native, ctx, "div", x, d, cnt))
        assert srv.stats()["rejected"] == 0
    finally:
        srv.close()
