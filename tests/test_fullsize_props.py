"""CPU self-test of the full-size property checks (tests/fullsize_props.py):
exact results pass, and each planted mistake is caught."""
import math

import numpy as np

from grns_gb300 import workload as W
from oracle.oracle import greedy_moduli
from tests import fullsize_props as F

MODS = greedy_moduli(32)
M = math.prod(MODS)
LOG2M = M.bit_length() - 1
COUNT = 120


def _rns(values):
    return W.to_residues(values, MODS, layout="aos")


def test_channel_pow2():
    D = np.array([0, 1, 29, 30, 31, 61, 900, 2047], np.uint32)
    p = F.channel_pow2(MODS, D)
    for k, e in enumerate(D):
        assert [int(v) for v in p[k]] == [pow(2, int(e), m) for m in MODS]


def test_division_checks_accept_exact_and_catch_planted():
    cmp, lb, _ = F.exact_cmp(MODS)
    x = W.uniform_residues(MODS, COUNT, seed=5, stream=W.S_X, layout="aos")
    d, dv = W.divisors(MODS, LOG2M, COUNT, seed=5, layout="aos")
    X = W.from_residues(x, MODS, layout="aos")
    q, r = [a // b for a, b in zip(X, dv)], [a % b for a, b in zip(X, dv)]
    assert F.divisor_bound_ok(lb, d)
    assert len(F.division_violations(MODS, x, d, _rns(q), _rns(r), cmp, lb)) == 0
    # planted: remainder off by one (residue channels), quotient one too high
    # with the matching remainder (r >= d), and the wrapped pair
    # q' d + r' = X + M with 0 <= r' < d (only the size check sees it)
    k0, k1, k2 = 3, 7, next(k for k in range(COUNT) if dv[k] > 1 and X[k] > 0)
    q2, r2 = list(q), list(r)
    r2[k0] += 1
    q2[k1] += 1
    r2[k1] = (r2[k1] - dv[k1]) % M
    q2[k2], r2[k2] = divmod(X[k2] + M, dv[k2])
    assert q2[k2] < M and 0 <= r2[k2] < dv[k2]
    bad = F.division_violations(MODS, x, d, _rns(q2), _rns(r2), cmp, lb)
    assert sorted(bad.tolist()) == sorted({k0, k1, k2})


def test_scale_checks_accept_exact_and_catch_planted():
    cmp, lb, _ = F.exact_cmp(MODS)
    x = W.uniform_residues(MODS, COUNT, seed=6, stream=W.S_X, layout="aos")
    D = W.shifts(COUNT, 900, seed=6)
    X = W.from_residues(x, MODS, layout="aos")
    out = [v >> int(e) for v, e in zip(X, D)]
    assert len(F.scale_violations(MODS, x, D, _rns(out), cmp, lb)) == 0
    # planted: one too high, one too low, and out + ceil(M / 2^D), whose
    # product wraps to within 2^D above out 2^D
    k0, k1, k2 = 2, 4, 9
    o2 = list(out)
    o2[k0] += 1
    o2[k1] = (o2[k1] - 1) % M
    o2[k2] += -(-M // (1 << int(D[k2])))
    assert o2[k2] < M
    bad = F.scale_violations(MODS, x, D, _rns(o2), cmp, lb)
    assert sorted(bad.tolist()) == [k0, k1, k2]
