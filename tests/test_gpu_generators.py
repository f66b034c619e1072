"""GPU: the device generators behind the benchmark's synthetic inputs produce
exactly the numbers of grns_gb300/workload.py (the documented host
definitions), so every benchmark input can be rebuilt and checked on the host."""
import ctypes

import numpy as np
import pytest

from grns_gb300 import workload as W
from oracle import oracle as O
from tests.helpers import moduli_for, mpint_dtype

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from grns_gb300 import native
    return native.lib(build_if_missing=True)


def P(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.parametrize("tag", ["ref8", "g32", "g64"])
def test_uniform_divisors_shifts(lib, tag):
    import grns_gb300 as G
    mods = moduli_for(tag)
    ctx = G.RNSContext(mods)
    n, cnt, seed = len(mods), 300, 99
    x = torch.empty((n, cnt), dtype=torch.int32, device="cuda")
    assert lib.grns_gen_uniform(ctx.handle, seed, W.S_X, cnt, 0, P(x), None) == 0
    assert np.array_equal(x.cpu().numpy(), W.uniform_residues(mods, cnt, seed, W.S_X))
    d = torch.empty_like(x)
    assert lib.grns_gen_divisors(ctx.handle, seed, cnt, 0, P(d), None) == 0
    want, _ = W.divisors(mods, ctx.log2M, cnt, seed)
    assert np.array_equal(d.cpu().numpy(), want)
    D = torch.empty(cnt, dtype=torch.int32, device="cuda")
    assert lib.grns_gen_shifts(seed, cnt, 900, P(D), None) == 0
    assert np.array_equal(D.cpu().numpy().astype(np.uint32), W.shifts(cnt, 900, seed))


@pytest.mark.parametrize("tag", ["g8", "g64"])
def test_mpint_records(lib, tag):
    """digits, sign and interval evaluation of the oracle's mp_int construction"""
    import grns_gb300 as G
    mods = moduli_for(tag)
    ctx, orc = G.RNSContext(mods), O.Oracle(mods)
    cnt, seed = 200, 5
    bits = min(950, orc.log2M // 2 - 10)
    out = torch.zeros(cnt * G.mpint_bytes(len(mods)), dtype=torch.uint8, device="cuda")
    assert lib.grns_gen_mpint(ctx.handle, seed, cnt, bits, P(out), None) == 0
    got = out.cpu().numpy().view(mpint_dtype(len(mods)))
    want = orc.mpint_from_ints(W.mpint_values(cnt, bits, seed))
    assert got.tobytes() == want.tobytes()
