"""GPU: division and power-of-two scaling at the benchmark's sizes (2^18
numbers each, n = 32, the benchmark's device generators), checked through
size-independent properties (tests/fullsize_props.py) with the library's own
comparison and evaluation; and the comparison against the evaluation at the
same size.  The reference-faithful kernels are too slow at this size; the
smaller parity tests cover them."""
import ctypes

import numpy as np
import pytest

from oracle.oracle import greedy_moduli
from tests import fullsize_props as F
from tests.helpers import IV_DTYPE

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

COUNT = 1 << 18
SEED = 20240601


@pytest.fixture(scope="module")
def env():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import grns_gb300 as G
    from grns_gb300 import native
    native.lib(build_if_missing=True)
    mods = greedy_moduli(32)
    ctx = G.RNSContext(mods)
    L = native.lib()

    def soa(fill):
        t = torch.empty((ctx.n, COUNT), dtype=torch.int32, device="cuda")
        native.check(fill(t))
        return t

    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    x = soa(lambda t: L.grns_gen_uniform(ctx.handle, SEED, 1, COUNT, 0, P(t), None))
    y = soa(lambda t: L.grns_gen_uniform(ctx.handle, SEED, 2, COUNT, 0, P(t), None))
    d = soa(lambda t: L.grns_gen_divisors(ctx.handle, SEED, COUNT, 0, P(t), None))
    D = torch.empty(COUNT, dtype=torch.int32, device="cuda")
    native.check(L.grns_gen_shifts(SEED, COUNT, 900, P(D), None))
    torch.cuda.synchronize()
    return mods, ctx, x, y, d, D


def aos(t):
    return np.ascontiguousarray(t.cpu().numpy().T)


def device_ops(ctx):
    """cmp and log2 bounds of X/M from the library's comparison and evaluation"""
    def dev(a):
        return torch.from_numpy(np.ascontiguousarray(np.asarray(a).T, dtype=np.int32)).cuda()

    def cmp(a, b):
        return ctx.rns_cmp(dev(a), dev(b)).cpu().numpy()

    def log2_bounds(a):
        iv = ctx.rns_eval_compute(dev(a)).cpu().numpy().view(IV_DTYPE)
        out = []
        for side in ("low", "upp"):
            f, e = iv[side]["frac"], iv[side]["exp"].astype(np.float64)
            with np.errstate(divide="ignore", invalid="ignore"):
                out.append(np.where(f > 0, np.log2(np.where(f > 0, f, 1.0)) + e, -np.inf))
        return out[0], out[1]

    return cmp, log2_bounds


def test_division_full_size(env):
    mods, ctx, x, y, d, D = env
    flags = torch.zeros(COUNT, dtype=torch.uint8, device="cuda")
    q, r = ctx.rns_div(x, d, flags=flags)
    assert int(flags.sum()) == 0
    cmp, lb = device_ops(ctx)
    xa, da = aos(x), aos(d)
    assert F.divisor_bound_ok(lb, da)
    bad = F.division_violations(mods, xa, da, aos(q), aos(r), cmp, lb)
    assert len(bad) == 0, bad[:10]


def test_scale2pow_full_size(env):
    mods, ctx, x, y, d, D = env
    out = ctx.rns_scale2pow(x, D)
    cmp, lb = device_ops(ctx)
    bad = F.scale_violations(mods, aos(x), D.cpu().numpy().astype(np.uint32), aos(out), cmp, lb)
    assert len(bad) == 0, bad[:10]


def test_cmp_agrees_with_evaluation_full_size(env):
    """where the two evaluations are disjoint the sign follows them; equal
    residues compare equal"""
    mods, ctx, x, y, d, D = env
    s = ctx.rns_cmp(x, y).cpu().numpy()
    s_self = ctx.rns_cmp(x, x).cpu().numpy()
    ex = ctx.rns_eval_compute(x).cpu().numpy().view(IV_DTYPE)
    ey = ctx.rns_eval_compute(y).cpu().numpy().view(IV_DTYPE)

    def val(iv, side):
        return np.ldexp(iv[side]["frac"], np.clip(iv[side]["exp"], -2000, 100).astype(np.int32))

    above = val(ex, "low") > val(ey, "upp")
    below = val(ex, "upp") < val(ey, "low")
    assert np.all(s[above] == 1) and np.all(s[below] == -1)
    assert above.sum() + below.sum() > COUNT * 0.99
    assert np.all(s_self == 0)
