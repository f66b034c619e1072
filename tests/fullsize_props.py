"""Size-independent properties of division and power-of-two scaling, for
checking results at sizes where big-integer reconstruction of every number
would take too long.

Arrays are AoS numpy (count, n) residues.  The caller supplies two
comparisons over whole arrays:
  cmp(a, b)        -> signs of X_a - X_b (int array)
  log2_bounds(a)   -> (lower, upper) bounds of log2(X_a / M), -inf for zero
On the GPU they are the library's own comparison and evaluation; on the CPU
(the self-test of this module) exact big-integer arithmetic.

Division (q, r of X by d): accepted iff
  (1) q d + r = x in every residue channel,
  (2) r < d,
  (3) log2(q/M) + log2(d/M) + log2 M <= log2(X/M) + MARGIN  (q d <= X).
(1) and (2) leave only q d + r = X + t M with t >= 1, so q d > X + M - d; when
d <= M (1 - 2^-19) that exceeds X by more than MARGIN in log2 and (3) fails.
Callers assert that bound on d (`divisor_bound_ok`).

Scaling (out = floor(X / 2^D)): with y = out 2^D and z = y + 2^D channel-wise,
accepted iff y <= x < z (two comparisons) and log2(out/M) + D <= log2(X/M) +
MARGIN.  A wrong out that passes the comparisons makes out 2^D wrap mod M,
so out 2^D >= M - 2^D, which (3) rejects unless X >= M - 2^(D+1); uniform X
lands there with probability below 2^(D + 1 - log2 M).
"""
import math

import numpy as np

MARGIN = 1e-6  # log2 units (relative 7e-7)


def channel_pow2(moduli, D):
    """2^D mod m_i for every number (rows) and modulus (columns), D < 2048"""
    D = np.asarray(D, np.uint64)
    assert D.size == 0 or int(D.max()) < 2048
    m = np.asarray(moduli, np.uint64)[None, :]
    out = np.ones((D.shape[0], m.shape[1]), np.uint64)
    base = np.broadcast_to(np.uint64(2) % m, out.shape).copy()
    for bit in range(11):
        sel = ((D >> np.uint64(bit)) & np.uint64(1)).astype(bool)[:, None]
        out = np.where(sel, out * base % m, out)
        base = base * base % m
    return out.astype(np.int64)


def log2_M(moduli):
    return math.fsum(math.log2(m) for m in moduli)


def divisor_bound_ok(log2_bounds, d):
    """every divisor below M (1 - 2^-19), the condition under which the
    division check is complete"""
    _, du = log2_bounds(d)
    return bool(np.all(du <= math.log2(1 - 2.0 ** -19)))


def division_violations(moduli, x, d, q, r, cmp, log2_bounds):
    """indices where (q, r) is not (floor(X / d), X mod d)"""
    m = np.asarray(moduli, np.int64)[None, :]
    x, d, q, r = (np.asarray(a, np.int64) for a in (x, d, q, r))
    bad = ((q * d + r) % m != x).any(axis=1)
    bad |= np.asarray(cmp(r, d)) != -1
    ql, _ = log2_bounds(q)
    dl, _ = log2_bounds(d)
    _, xu = log2_bounds(x)
    nz = np.isfinite(ql) & np.isfinite(dl)
    lhs = np.where(nz, ql + dl, -np.inf) + log2_M(moduli)
    bad |= nz & (lhs > xu + MARGIN)
    return np.flatnonzero(bad)


def scale_violations(moduli, x, D, out, cmp, log2_bounds):
    """indices where out is not floor(X / 2^D)"""
    m = np.asarray(moduli, np.int64)[None, :]
    x, out = np.asarray(x, np.int64), np.asarray(out, np.int64)
    p = channel_pow2(moduli, D)
    y = out * p % m
    z = (y + p) % m
    bad = np.asarray(cmp(y, x)) > 0
    bad |= np.asarray(cmp(x, z)) != -1
    ol, _ = log2_bounds(out)
    _, xu = log2_bounds(x)
    nz = np.isfinite(ol)
    bad |= nz & (np.where(nz, ol, 0.0) + np.asarray(D, np.float64) > xu + MARGIN)
    return np.flatnonzero(bad)


def exact_cmp(moduli):
    """cmp over big integers (CRT)"""
    M = math.prod(moduli)
    basis = [(M // mi) * pow(M // mi, -1, mi) for mi in moduli]

    def value(row):
        return sum(int(v) * b for v, b in zip(row, basis)) % M

    def cmp(a, b):
        return np.array([(value(u) > value(v)) - (value(u) < value(v)) for u, v in zip(a, b)], np.int32)

    def log2_bounds(a):
        vals = [value(row) for row in a]
        lg = np.array([math.log2(v) - log2_M(moduli) if v else -np.inf for v in vals])
        return lg - 1e-12, lg + 1e-12

    return cmp, log2_bounds, value
