"""Checks of one job's device outputs against the oracle and exact big-integer
arithmetic, on a seeded sample of its elements -- shared by the batched and
served tests, so that a fused or packed launch is held to the same answers as
the per-call parity tests, not only to the per-call entry points.

Ops (grns_op): 0 eval, 1 cmp, 2 div, 3 scale2pow, 4 max, 5/6/7 mp_int
add/sub/mul, 8 mp_int div.  Residue arrays are SoA (n, count) for layout 0 and
AoS (count, n) for layout 1; mp_int arrays are mp_int_t records.
"""
import numpy as np

from oracle import oracle as O
from tests.helpers import IV_DTYPE, mpint_dtype


def sample(count, k=48, seed=0):
    """sorted distinct indices: the first, the last and k seeded others"""
    if count <= k + 2:
        return np.arange(count)
    rng = np.random.default_rng(seed)
    return np.unique(np.concatenate([[0, count - 1], rng.choice(count, k, replace=False)]))


def _np(t):
    """a numpy view of a device tensor's contents (numpy arrays pass through)"""
    return t if isinstance(t, np.ndarray) else t.cpu().numpy()


def aos(t, layout, count, n):
    """numpy AoS (count, n) residues of a device array"""
    a = _np(t).view(np.int32)
    if layout == 0:
        return np.ascontiguousarray(a.reshape(n, -1)[:, :count].T)
    return np.ascontiguousarray(a.reshape(-1, n)[:count])


def oracle_eval_device(orc, x):
    """the oracle's device-path evaluation with the device's ceil(log2) in the
    refinement loop (the reference GPU code calls CUDA's log2)"""
    from grns_gb300 import RNSContext
    xs = orc.log2_inputs(x)
    cs = RNSContext.device_ceil_log2(xs) if len(xs) else np.zeros(0, np.int32)
    return orc.eval_with_device_log2(x, xs, cs)


def signed(orc, m):
    return [(-v if s else v) for v, s in zip(orc.exact.from_rns(m["digits"]), m["sign"])]


def check_job(orc, op, count, layout, a, b, o0, o1, seed=0, k=48):
    """assert that a sample of the job's outputs equals the oracle's (bit for
    bit: intervals, mp_int records) or exact arithmetic (signs, q and r,
    scaled values, the maximum and its smallest index)"""
    if count == 0:
        return
    n = orc.n
    ex = orc.exact
    idx = sample(count, k, seed)
    if op in (5, 6, 7, 8):
        dt = mpint_dtype(n)
        x = _np(a).view(dt)[:count][idx]
        y = _np(b).view(dt)[:count][idx]
        got = _np(o0).view(dt)[:count][idx]
        if op == 8:
            assert got["digits"].tobytes() == orc.mpint("div", x, y)[0]["digits"].tobytes()
            for xv, yv, qv in zip(signed(orc, x), signed(orc, y), signed(orc, got)):
                assert 0 <= xv - qv * yv < abs(yv), (xv, yv, qv)
            return
        name = {5: "add", 6: "sub", 7: "mul"}[op]
        want, _ = orc.mpint(name, x, y, path=O.PATH_DEVICE)
        # field by field: a fancy-indexed copy of padded records does not keep the padding bytes
        for f in ("digits", "sign", "eval"):
            if got[f].tobytes() != want[f].tobytes():
                k = next(j for j in range(len(idx)) if got[f][j].tobytes() != want[f][j].tobytes())
                raise AssertionError(f"mp_int {name}, element {int(idx[k])} of {count}: {f} differs; "
                                     f"x {x[k]!r} y {y[k]!r} got {got[k]!r} want {want[k]!r}")
        f = {5: lambda p, q: p + q, 6: lambda p, q: p - q, 7: lambda p, q: p * q}[op]
        assert signed(orc, got) == [f(p, q) for p, q in zip(signed(orc, x), signed(orc, y))]
        return
    x = aos(a, layout, count, n)
    if op == 4:
        want = orc.max(x)
        assert int(_np(o1).view(np.int64).reshape(-1)[0]) == want
        assert np.array_equal(_np(o0).view(np.int32).reshape(-1)[:n], x[want])
        return
    xs = x[idx]
    X = ex.from_rns(xs)
    if op == 0:
        got = _np(o0).view(IV_DTYPE)[:count][idx]
        assert got.tobytes() == oracle_eval_device(orc, xs).tobytes()
        assert ex.encloses(got, X).all()
    elif op == 1:
        Y = ex.from_rns(aos(b, layout, count, n)[idx])
        got = _np(o0).view(np.int32).reshape(-1)[:count][idx]
        assert list(got) == [(p > q) - (p < q) for p, q in zip(X, Y)]
    elif op == 2:
        Dv = ex.from_rns(aos(b, layout, count, n)[idx])
        Q = ex.from_rns(aos(o0, layout, count, n)[idx])
        R = ex.from_rns(aos(o1, layout, count, n)[idx])
        assert [(q, r) for q, r in zip(Q, R)] == [divmod(p, d) for p, d in zip(X, Dv)]
    elif op == 3:
        D = _np(b).view(np.int32).reshape(-1)[:count][idx].astype(np.int64)
        Y = ex.from_rns(aos(o0, layout, count, n)[idx])
        assert Y == [p >> int(s) for p, s in zip(X, D)]
    else:
        raise ValueError(f"op {op}")
