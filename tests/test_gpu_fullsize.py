"""GPU: division and power-of-two scaling at the benchmark's sizes (2^18
numbers each, n = 32, the benchmark's device generators), checked through
size-independent properties (tests/fullsize_props.py) with the library's own
comparison and evaluation on every number, and exactly against Python big
integers on a seeded sample of 4096 numbers spread over every 4096-number
segment (each segment's longest divisions and largest shifts included); and
the comparison against the evaluation at the same size.  The
reference-faithful kernels are too slow at this size; the smaller parity
tests cover them."""
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


SEGMENT = 4096  # the division sorts and schedules its numbers in segments of this many


def exact_sample(ctx, d_log2_upper, seed=7):
    """indices of a seeded sample spread over every 4096-number segment: in each
    segment the 16 smallest divisors (the longest quotients, the most digit
    steps) and 48 uniform indices -- 4096 in all at 2^18 numbers"""
    rng = np.random.default_rng(seed)
    idx = []
    for b0 in range(0, COUNT, SEGMENT):
        seg = np.arange(b0, min(COUNT, b0 + SEGMENT))
        longest = seg[np.argsort(d_log2_upper[seg], kind="stable")[:16]]
        idx.append(longest)
        idx.append(rng.choice(np.setdiff1d(seg, longest), 48, replace=False))
    return np.unique(np.concatenate(idx))


def test_division_full_size_exact_sample(env):
    """the benchmark's own 2^18 divisions: q and r equal floor(X/d) and X mod d
    (Python big integers) on a sample that covers every segment"""
    from oracle.oracle import Exact
    mods, ctx, x, y, d, D = env
    q, r = ctx.rns_div(x, d)
    cmp, lb = device_ops(ctx)
    xa, da, qa, ra = aos(x), aos(d), aos(q), aos(r)
    _, du = lb(da)
    idx = exact_sample(ctx, du)
    assert len(idx) >= 4096
    ex = Exact(mods)
    X, Dd = ex.from_rns(xa[idx]), ex.from_rns(da[idx])
    Q, R = ex.from_rns(qa[idx]), ex.from_rns(ra[idx])
    bad = [int(k) for k, a, b, qq, rr in zip(idx, X, Dd, Q, R) if (qq, rr) != divmod(a, b)]
    assert not bad, bad[:10]
    # the sample reaches the longest divisions: quotients of more than 900 bits
    assert max(qq.bit_length() for qq in Q) > 900


def test_scale2pow_full_size_exact_sample(env):
    """the benchmark's own 2^18 scalings: floor(X / 2^D) (Python big integers)
    on 64 numbers of every segment, including each segment's largest shifts"""
    from oracle.oracle import Exact
    mods, ctx, x, y, d, D = env
    out = aos(ctx.rns_scale2pow(x, D))
    xa, Dh = aos(x), D.cpu().numpy().astype(np.int64)
    rng = np.random.default_rng(11)
    idx = []
    for b0 in range(0, COUNT, SEGMENT):
        seg = np.arange(b0, min(COUNT, b0 + SEGMENT))
        top = seg[np.argsort(-Dh[seg], kind="stable")[:8]]
        idx.append(top)
        idx.append(rng.choice(np.setdiff1d(seg, top), 56, replace=False))
    idx = np.unique(np.concatenate(idx))
    assert len(idx) >= 4096
    ex = Exact(mods)
    X, Y = ex.from_rns(xa[idx]), ex.from_rns(out[idx])
    bad = [int(k) for k, a, yy in zip(idx, X, Y) if yy != a >> int(Dh[k])]
    assert not bad, bad[:10]


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
