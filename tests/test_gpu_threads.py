"""GPU: one context used from several host threads at once, each on its own
stream (the C ABI's calls are stream-ordered and keep no per-call state in the
context): every thread gets the single-threaded results."""
import threading

import numpy as np
import pytest

from grns_gb300 import workload as W
from tests.helpers import moduli_for

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def test_concurrent_calls_on_one_context():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import grns_gb300 as G
    mods = moduli_for("g32")
    ctx = G.RNSContext(mods)
    N = 40000
    x = torch.from_numpy(np.ascontiguousarray(W.uniform_residues(mods, N, 3, W.S_X, layout="aos").T)).cuda()
    y = torch.from_numpy(np.ascontiguousarray(W.uniform_residues(mods, N, 3, W.S_Y, layout="aos").T)).cuda()
    d, _ = W.divisors(mods, ctx.log2M, N, 3, layout="aos")
    d = torch.from_numpy(np.ascontiguousarray(d.T)).cuda()
    D = torch.from_numpy((np.arange(N) % 900 + 1).astype(np.int32)).cuda()
    hx, hd = x.cpu().pin_memory(), d.cpu().pin_memory()

    def run(stream):
        with torch.cuda.stream(stream):
            q, r = ctx.rns_div(x, d, stream=stream)
            s = ctx.rns_scale2pow(x, D, stream=stream)
            c = ctx.rns_cmp(x, y, stream=stream)
            e = ctx.rns_eval_compute(x, stream=stream)
            hq, hr = ctx.rns_div_host(hx, hd, stream=stream)
            stream.synchronize()
            return [t.cpu() for t in (q, r, s, c, e, hq, hr)]

    want = run(torch.cuda.Stream())
    results, errors = {}, []

    def worker(k):
        try:
            for _ in range(3):
                results[k] = run(torch.cuda.Stream())
        except Exception as ex:  # reported below
            errors.append(repr(ex))

    threads = [threading.Thread(target=worker, args=(k,)) for k in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=300)
    assert not errors, errors
    assert len(results) == 4
    for got in results.values():
        for a, b in zip(got, want):
            assert torch.equal(a, b)
