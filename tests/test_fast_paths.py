"""CPU: the integer fast-path algorithms of the product (grns_gb300/csrc/rns_fast.cuh),
compiled for the host, against exact big-integer arithmetic.  Tiny moduli sets are
checked exhaustively (every pair of numbers); the configuration moduli sets on
seeded random and special inputs.  The GPU runs the identical source."""
import ctypes
import os
import random
import subprocess
from fractions import Fraction

import numpy as np
import pytest

from grns_gb300 import workload as W
from tests.helpers import IV_DTYPE as IV, TAGS, moduli_for, sized

HERE = os.path.dirname(os.path.abspath(__file__))
SMALL_SETS = [[3, 5, 7, 11], [3, 5, 7, 11, 13, 17, 19, 23], [3, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43]]


@pytest.fixture(scope="module")
def fc(tmp_path_factory):
    out = tmp_path_factory.mktemp("fast") / "libfast.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-ffp-contract=off",
                    os.path.join(HERE, "native", "fast_check.cpp"), "-o", str(out)], check=True)
    L = ctypes.CDLL(str(out))
    L.fc_create.restype = ctypes.c_void_p
    L.fc_create.argtypes = [ctypes.c_void_p, ctypes.c_int]
    L.fc_destroy.argtypes = [ctypes.c_void_p]
    L.fc_E.restype = ctypes.c_uint64
    L.fc_E.argtypes = [ctypes.c_void_p]
    L.fc_binary_limbs.argtypes = [ctypes.c_void_p]
    L.fc_table.restype = ctypes.c_long
    L.fc_table.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_long]
    for f in ("fc_cmp", "fc_div", "fc_div_rows", "fc_dmuldiv", "fc_scale", "fc_fx", "fc_eval", "fc_eval_tight", "fc_from_binary", "fc_to_binary",
              "fc_eval_fast"):
        getattr(L, f).argtypes = None
    return L


class FC:
    def __init__(self, L, moduli):
        self.L, self.moduli, self.n = L, list(moduli), len(moduli)
        arr = np.array(moduli, np.uint32)
        self.h = ctypes.c_void_p(L.fc_create(ctypes.c_void_p(arr.ctypes.data), self.n))
        self.M = 1
        for m in moduli:
            self.M *= m

    def res(self, vals):
        return W.to_residues(vals, self.moduli, layout="aos").astype(np.uint32)

    def ints(self, arr):
        return W.from_residues(arr, self.moduli, layout="aos")

    @staticmethod
    def P(a):
        return ctypes.c_void_p(a.ctypes.data)

    def cmp(self, X, Y):
        x, y = self.res(X), self.res(Y)
        out = np.zeros(len(X), np.int32)
        self.L.fc_cmp(self.h, self.P(x), self.P(y), ctypes.c_long(len(X)), self.P(out))
        return out

    def div(self, X, D):
        x, d = self.res(X), self.res(D)
        q, r = np.zeros_like(x), np.zeros_like(x)
        fl = np.zeros(len(X), np.uint32)
        self.L.fc_div(self.h, self.P(x), self.P(d), ctypes.c_long(len(X)), self.P(q), self.P(r), self.P(fl))
        # the prepared-row form (pass A row, pass B digit steps, r from the final remainder) agrees
        q2, r2, fl2 = np.zeros_like(x), np.zeros_like(x), np.zeros(len(X), np.uint32)
        self.L.fc_div_rows(self.h, self.P(x), self.P(d), ctypes.c_long(len(X)), self.P(q2), self.P(r2), self.P(fl2))
        assert np.array_equal(q, q2) and np.array_equal(r, r2) and np.array_equal(fl, fl2)
        return self.ints(q), self.ints(r), fl

    def scale(self, X, S):
        x = self.res(X)
        s = np.asarray(S, np.uint32)
        out = np.zeros_like(x)
        self.L.fc_scale(self.h, self.P(x), self.P(s), ctypes.c_long(len(X)), self.P(out))
        # the one-pass form (the low D bits of X from the CRT sum in 26-bit chunks) agrees
        out2 = np.zeros_like(x)
        self.L.fc_scale_bin(self.h, self.P(x), self.P(s), ctypes.c_long(len(X)), self.P(out2))
        assert np.array_equal(out, out2)
        return self.ints(out)

    def from_binary(self, vals, limbs):
        w = np.zeros((len(vals), limbs), np.uint32)
        for k, v in enumerate(vals):
            for j in range(limbs):
                w[k, j] = (v >> (32 * j)) & 0xFFFFFFFF
        out = np.zeros((len(vals), self.n), np.uint32)
        self.L.fc_from_binary(self.h, self.P(w), ctypes.c_int(limbs), ctypes.c_long(len(vals)), self.P(out))
        return out

    def to_binary(self, x):
        x = np.ascontiguousarray(x, np.uint32)
        L = self.L.fc_binary_limbs(self.h)
        out = np.zeros((len(x), L), np.uint32)
        ok = np.zeros(len(x), np.int32)
        self.L.fc_to_binary(self.h, self.P(x), ctypes.c_long(len(x)), self.P(out), self.P(ok))
        return [int.from_bytes(r.astype("<u4").tobytes(), "little") for r in out], ok

    def fx(self, X):
        x = self.res(X)
        a, lo, hi = (np.zeros(len(X), np.uint64) for _ in range(3))
        self.L.fc_fx(self.h, self.P(x), ctypes.c_long(len(X)), self.P(a), self.P(lo), self.P(hi))
        return a, [int(l) + (int(h) << 64) for l, h in zip(lo, hi)]


def sgn(a, b):
    return (a > b) - (a < b)


@pytest.mark.parametrize("moduli", SMALL_SETS[:2])
def test_exhaustive_small_sets(fc, moduli):
    f = FC(fc, moduli)
    M = f.M
    step = max(1, M // 1200)
    vals = list(range(0, M, step)) + [M - 1, M - 2, 1, 2]
    X = [a for a in vals for _ in vals]
    Y = [b for _ in vals for b in vals]
    assert list(f.cmp(X, Y)) == [sgn(a, b) for a, b in zip(X, Y)]
    Dv = [b if b else 1 for b in Y]
    q, r, fl = f.div(X, Dv)
    assert q == [a // b for a, b in zip(X, Dv)] and r == [a % b for a, b in zip(X, Dv)]
    assert not fl.any()
    S = [1 + (k % 40) for k in range(len(X))]
    assert f.scale(X, S) == [a >> s for a, s in zip(X, S)]


def test_fixed_point_enclosure(fc):
    for tag in ("g8", "g32", "g64"):
        f = FC(fc, moduli_for(tag))
        E = int(fc.fc_E(f.h))
        rng = random.Random(3)
        X = [rng.randrange(f.M) for _ in range(300)] + [0, 1, f.M - 1, f.M // 2]
        a64, t96 = f.fx(X)
        for v, a, t in zip(X, a64, t96):
            frac64 = Fraction(v, f.M) * 2 ** 64
            U = t % 2 ** 96
            if int(a) >= E:
                assert int(a) - E <= frac64 <= int(a)
            if U >= E:
                assert U - E <= Fraction(v, f.M) * 2 ** 96 <= U


@pytest.mark.parametrize("tag", TAGS + ["g128", "g256"])
def test_random_and_special(fc, tag):
    f = FC(fc, moduli_for(tag))
    M = f.M
    L = M.bit_length() - 1
    rng = random.Random(17)
    N = sized(f.n, 400, 120)
    X = [rng.randrange(M) for _ in range(N)]
    Y = [rng.randrange(M) for _ in range(N)]
    # ties, neighbours, tiny and near-M values, powers of two
    X += [5, M - 1, M - 1, 0, 1, 1 << (L // 2), M // 2, M // 2 + 1] + [1 << j for j in range(0, L, 37)]
    Y += [5, M - 2, M - 1, 1, 0, (1 << (L // 2)) + 1, M // 2 + 1, M // 2] + [(1 << j) - 1 for j in range(0, L, 37)]
    Y[3] = X[3] + 1 if X[3] + 1 < M else 0
    assert list(f.cmp(X, Y)) == [sgn(a, b) for a, b in zip(X, Y)]
    # division: divisor bit length uniform in [1, L], plus edge cases
    Dv = [rng.randrange(1 << (b - 1), 1 << b) for b in (rng.randrange(1, L + 1) for _ in range(len(X)))]
    Dv[:6] = [1, 2, M - 1, X[3], X[4] + 1 if X[4] + 1 < M else 1, (M - 1) // 2]
    q, r, fl = f.div(X, Dv)
    assert q == [a // b for a, b in zip(X, Dv)]
    assert r == [a % b for a, b in zip(X, Dv)]
    assert not fl.any()
    S = [rng.randrange(1, min(901, L + 40)) for _ in range(len(X))]
    S[:5] = [1, 29, 30, 31, L]
    assert f.scale(X, S) == [a >> s for a, s in zip(X, S)]


@pytest.mark.parametrize("tag", ["ref8", "g12", "g32", "g64", "p16", "p32", "p64", "g256"])
def test_division_quotient_boundaries(fc, tag):
    """dividends just below, at and above multiples of the divisor, divisors
    near M and near powers of two: the certified quotient estimate must never
    overshoot and the final correction must land exactly"""
    f = FC(fc, moduli_for(tag))
    M = f.M
    L = M.bit_length() - 1
    rng = random.Random(99)
    X, Dv = [], []
    for _ in range(sized(f.n, 150, 60)):
        b = rng.randrange(1, L + 1)
        d = rng.randrange(1 << (b - 1), 1 << b)
        qmax = (M - 1) // d
        q = rng.randrange(qmax + 1)
        for x in (q * d, q * d - 1, q * d + d - 1, q * d + 1):
            if 0 <= x < M:
                X.append(x)
                Dv.append(d)
    for d in (M - 1, M - 2, (M + 1) // 2, 1 << L, (1 << L) - 1, 3):
        for x in (M - 1, d, d - 1, d + 1, 2 * d, 2 * d - 1):
            if 0 <= x < M and 0 < d < M:
                X.append(x)
                Dv.append(d)
    q, r, fl = f.div(X, Dv)
    assert q == [a // b for a, b in zip(X, Dv)]
    assert r == [a % b for a, b in zip(X, Dv)]
    assert not fl.any()


@pytest.mark.parametrize("tag", TAGS)
def test_division_remainder_evaluation_wraps(fc, tag):
    """dividends within a hair of M over divisors just below M (above the
    near-M band, within 2^-53 M): the final remainder's fixed-point value
    wraps past 2^96, and the correction must not read it as a small R"""
    from tests.test_gpu_parity import near_m_division_cases
    f = FC(fc, moduli_for(tag))
    X, Dv = near_m_division_cases(f.M)
    q, r, fl = f.div(X, Dv)
    assert q == [a // b for a, b in zip(X, Dv)]
    assert r == [a % b for a, b in zip(X, Dv)]
    assert not fl.any()


@pytest.mark.parametrize("tag", TAGS + ["g256"])
def test_scaling_every_shift(fc, tag):
    """floor(X / 2^D) for every D from 0 to log2M + 2 (the one-pass form's
    last chunk is partial unless 26 divides D) on values at the edges: M - 1,
    powers of two and their neighbours, values with long runs of ones"""
    f = FC(fc, moduli_for(tag))
    M = f.M
    L = M.bit_length() - 1
    rng = random.Random(31)
    base = [M - 1, M - 2, (1 << L) - 1, 1 << L, (M - 1) // 2, 1, 3, rng.randrange(M), rng.randrange(M)]
    base += [(1 << b) - 1 for b in range(26, L, 26)] + [1 << b for b in range(25, L, 26)]
    X, S = [], []
    # 128 and 256 moduli (2048 to 6400 bits): every D near the step and chunk
    # boundaries (multiples of 26 and 52, +-1) and near log2M, every 7th elsewhere
    edge = lambda d: d % 26 in (0, 1, 25) or d % 52 in (0, 1, 51) or d >= L - 3  # noqa: E731
    for d in range(0, L + 3):
        if f.n >= 128 and not (edge(d) or d % 7 == 0):
            continue
        for v in base[:5] + [base[(d * 7) % len(base)]]:
            X.append(v % M)
            S.append(d)
    assert f.scale(X, S) == [a >> s for a, s in zip(X, S)]


@pytest.mark.parametrize("tag", ["ref8", "g8", "g32", "g64", "p16", "p32", "p64"])
def test_division_short_and_extreme_dividends(fc, tag):
    """dividends of every length (the leading zero digits are skipped), and
    dividends within a hair of M or of 0 (where a fixed-point evaluation
    alone cannot tell them apart)"""
    f = FC(fc, moduli_for(tag))
    M = f.M
    L = M.bit_length() - 1
    rng = random.Random(5)
    X, Dv = [], []
    for _ in range(sized(f.n, 200, 80)):
        bx, bd = rng.randrange(1, L + 1), rng.randrange(1, L + 1)
        X.append(rng.randrange(1 << (bx - 1), 1 << bx))
        Dv.append(rng.randrange(1 << (bd - 1), 1 << bd))
    for delta in (1, 2, 3, 1 << 20, 1 << 40, 1 << 70, 1 << 130, 1 << 200):
        for d in (1, 3, 1 << 17, (1 << 61) + 5, 1 << (L // 2), M // 7, M // 3):
            for x in (M - delta, delta):
                if 0 <= x < M and 0 < d < M:
                    X.append(x)
                    Dv.append(d)
    q, r, fl = f.div(X, Dv)
    assert q == [a // b for a, b in zip(X, Dv)]
    assert r == [a % b for a, b in zip(X, Dv)]
    assert not fl.any()


@pytest.mark.parametrize("tag", TAGS)
def test_integer_eval_is_bit_exact(fc, tag):
    """the integer-pipe evaluation returns, on its common path, the same two
    doubles as the reference's FP64 directed-rounding evaluation (device path
    of rns_eval_compute as restated in the oracle), and hands every other
    number (ambiguous integer part, small fraction) to the rare path"""
    from oracle import oracle as O
    mods = moduli_for(tag)
    f, orc = FC(fc, mods), O.Oracle(mods)
    M = f.M
    rng = random.Random(41)
    vals = [rng.randrange(M) for _ in range(3000)]
    vals += [0, 1, 2, M - 1, M - 2, M // 2, M // 3, (M + 1) // 2] + [M >> j for j in range(1, 200, 7)]
    vals += [rng.randrange(max(1, M >> 40)) for _ in range(200)]
    x = f.res(vals)
    st = np.zeros(len(vals), np.int32)
    iv = np.zeros(len(vals), IV)
    fc.fc_eval(f.h, f.P(x), ctypes.c_long(len(vals)), f.P(st), f.P(iv))
    want = orc.eval(x.view(np.int32), path=O.PATH_DEVICE)
    ok = st == 0
    assert ok.sum() > 2500
    assert iv[ok].tobytes() == want[ok].tobytes()
    assert all((s == 2) == (v == 0) for s, v in zip(st, vals))
    assert not (st == 8).any()


@pytest.mark.parametrize("tag", TAGS)
def test_integer_fast_eval_is_bit_exact(fc, tag):
    """the integer-pipe form of rns_eval_compute_fast (no mixed-radix step)
    returns the reference's device doubles on its common path, numbers below M/2"""
    from oracle import oracle as O
    mods = moduli_for(tag)
    f, orc = FC(fc, mods), O.Oracle(mods)
    M = f.M
    rng = random.Random(47)
    vals = [rng.randrange(M // 2) for _ in range(3000)] + [M // 2 - 1, 1, 2] + [M >> j for j in range(2, 200, 7)]
    x = f.res(vals)
    st = np.zeros(len(vals), np.int32)
    iv = np.zeros(len(vals), IV)
    fc.fc_eval_fast(f.h, f.P(x), ctypes.c_long(len(vals)), f.P(st), f.P(iv))
    want = orc.eval(x.view(np.int32), path=O.PATH_DEVICE_FAST)
    ok = st == 0
    assert ok.sum() > 2500
    assert iv[ok].tobytes() == want[ok].tobytes()


def er_fraction(frac, exp):
    return Fraction(float(frac)) * Fraction(2) ** int(exp)


@pytest.mark.parametrize("tag", TAGS)
def test_one_ulp_evaluation(fc, tag):
    """where the 128-bit evaluation certifies it, the interval encloses X/M
    exactly, is at most one ulp wide, and is never wider than the reference's
    interval (rns_eval_compute, device path restated in the oracle)"""
    from oracle import oracle as O
    mods = moduli_for(tag)
    f, orc = FC(fc, mods), O.Oracle(mods)
    M = f.M
    rng = random.Random(43)
    vals = [rng.randrange(M) for _ in range(1500)] + [rng.randrange(max(1, M >> 30)) for _ in range(100)]
    vals += [1, 2, M - 1, M // 2, M // 3, (M + 1) // 2] + [M >> j for j in range(1, 120, 9)]
    x = f.res(vals)
    ok = np.zeros(len(vals), np.int32)
    iv = np.zeros(len(vals), IV)
    fc.fc_eval_tight(f.h, f.P(x), ctypes.c_long(len(vals)), f.P(ok), f.P(iv))
    ref = orc.eval(x.view(np.int32), path=O.PATH_DEVICE)
    assert ok.sum() > 1400
    for k in np.nonzero(ok)[0]:
        v = Fraction(vals[k], M)
        lo = er_fraction(iv[k]["low"]["frac"], iv[k]["low"]["exp"])
        up = er_fraction(iv[k]["upp"]["frac"], iv[k]["upp"]["exp"])
        assert lo < v <= up
        ulp = Fraction(2) ** (int(iv[k]["low"]["exp"]) - 52)
        assert up - lo <= ulp
        rlo = er_fraction(ref[k]["low"]["frac"], ref[k]["low"]["exp"])
        rup = er_fraction(ref[k]["upp"]["frac"], ref[k]["upp"]["exp"])
        assert up - lo <= rup - rlo


@pytest.mark.parametrize("tag", ["ref8", "g12", "g32", "g64", "p16", "p32", "p64", "g256"])
def test_scaling_step_boundaries(fc, tag):
    """exponents at and around multiples of the 52-bit step, the full range,
    and dividends next to 0 and M (the first step's checked rank)"""
    f = FC(fc, moduli_for(tag))
    M = f.M
    L = M.bit_length() - 1
    rng = random.Random(11)
    X, S = [], []
    for D in sorted({1, 2, 51, 52, 53, 103, 104, 105, 156, 157, L - 1, L, L + 1}):
        for x in [M - 1, M - 2, 0, 1, (1 << min(D, L)) - 1, 1 << min(D, L)] + [rng.randrange(M) for _ in range(6)]:
            if 0 <= x < M:
                X.append(x)
                S.append(D)
    assert f.scale(X, S) == [a >> s for a, s in zip(X, S)]


@pytest.mark.parametrize("moduli", SMALL_SETS[:2])
def test_binary_conversion_exhaustive_small(fc, moduli):
    """every X in [0, M) (or a dense sample) through RNS -> binary -> RNS"""
    f = FC(fc, moduli)
    vals = list(range(f.M)) if f.M <= 200000 else sorted(set(random.Random(3).randrange(f.M) for _ in range(200000)))
    x = f.res(vals)
    back, ok = f.to_binary(x)
    assert back == vals and ok.all()
    limbs = max(1, (f.M.bit_length() + 31) // 32)
    assert np.array_equal(f.from_binary(vals, limbs), x)


@pytest.mark.parametrize("tag", TAGS + ["g128", "g256"])
def test_binary_conversion(fc, tag):
    """rns_from_binary / rns_to_binary arithmetic against exact integers: uniform
    values, values of every bit length, near 0 and M (the rank estimate is one
    too high there), inputs of M and more, up to 256 limbs (past 158 chunks the sums fold)"""
    f = FC(fc, moduli_for(tag))
    rng = random.Random(11)
    vals = [rng.randrange(f.M) for _ in range(400)]
    vals += [rng.randrange(1 << b) for b in range(1, f.M.bit_length())]
    vals += list(range(0, 40)) + [f.M - k for k in range(1, 40)] + [f.M // 2 + d for d in (-1, 0, 1)]
    back, ok = f.to_binary(f.res(vals))
    assert back == vals and ok.all()
    for limbs in (1, 3, (f.M.bit_length() + 31) // 32, 128, 256):
        wide = [rng.randrange(1 << (32 * limbs)) for _ in range(60)] + [(1 << (32 * limbs)) - 1]
        assert np.array_equal(f.from_binary(wide, limbs), f.res([v % f.M for v in wide]))
    # a residue >= its modulus is refused
    bad = f.res([5])
    bad[0, 0] = f.moduli[0]
    back, ok = f.to_binary(bad)
    assert ok[0] == 0 and back[0] == 0


TABLE_KEYS = ["w", "recip_rd", "recip_ru", "acc", "ref_factor", "unit", "inv_unit", "mrc_inv", "pow2", "m_pow2_res",
              "mi_pow2_res", "pow2_inv"]


@pytest.mark.parametrize("tag", TAGS)
def test_host_tables_match_oracle(fc, tag):
    """the host-built tables (without GMP) equal the oracle's, which are pinned
    on the reference's rns_const_init, byte for byte, for every set including
    the catalogue's; the same bytes grns_ctx_get_table returns"""
    from oracle import oracle as O
    mods = moduli_for(tag)
    f = FC(fc, mods)
    want = O.Oracle(mods).consts()
    buf = np.zeros(max(1 << 20, max(v.nbytes for v in want.values())), np.uint8)
    for which, key in enumerate(TABLE_KEYS):
        got = fc.fc_table(f.h, which, ctypes.c_void_p(buf.ctypes.data), buf.size)
        assert got == want[key].nbytes, key
        assert buf[:got].tobytes() == want[key].tobytes(), key
    assert fc.fc_table(f.h, len(TABLE_KEYS), ctypes.c_void_p(buf.ctypes.data), buf.size) == -1
    fc.fc_destroy(f.h)


def _fuzz_value(rng, M, L):
    """uniform, of uniform bit length, just below M, near powers of two, near
    M / k, short, or a fixed edge value"""
    k = rng.random()
    if k < 0.3:
        return rng.randrange(M)
    if k < 0.5:
        b = rng.randrange(1, L + 1)
        return rng.randrange(1 << (b - 1), 1 << b)
    if k < 0.6:
        return M - 1 - rng.randrange(1 << rng.randrange(1, 64))
    if k < 0.7:
        return (1 << rng.randrange(L + 1)) + rng.randrange(-3, 4)
    if k < 0.8:
        return M // rng.randrange(1, 1 << 20) + rng.randrange(-3, 4)
    if k < 0.9:
        return rng.randrange(1 << rng.randrange(1, 70))
    return rng.choice([0, 1, 2, M - 1, M - 2, M // 2, (M + 1) // 2])


def test_differential_fuzz(fc):
    """comparison, division (with dividends near multiples of the divisor),
    scaling (with values near multiples of 2^D) and binary <-> RNS against
    exact arithmetic, the integer-pipe evaluation and its fast form against
    the oracle's restatement of the reference's device path, and the one-ulp
    evaluation's enclosure, on mixed value distributions over every set, for
    GRNS_FUZZ_SECONDS (default 5) seconds"""
    import time
    seconds = float(os.environ.get("GRNS_FUZZ_SECONDS", "5"))
    rng = random.Random(int(os.environ.get("GRNS_FUZZ_SEED", "2024")))
    from oracle import oracle as O
    ctxs = {t: FC(fc, moduli_for(t)) for t in TAGS}
    orcs = {t: O.Oracle(moduli_for(t)) for t in TAGS}
    deadline, rounds = time.time() + seconds, 0
    while time.time() < deadline or rounds < len(TAGS):
        tag = TAGS[rounds % len(TAGS)]
        f = ctxs[tag]
        M = f.M
        L = M.bit_length() - 1
        N = 100
        X = [_fuzz_value(rng, M, L) % M for _ in range(N)]
        Y = [_fuzz_value(rng, M, L) % M for _ in range(N)]
        for k in range(0, N, 10):
            Y[k] = X[k]
        assert list(f.cmp(X, Y)) == [sgn(a, b) for a, b in zip(X, Y)], tag
        D = [max(1, y) for y in Y]
        for k in range(1, N, 7):
            q = rng.randrange((M - 1) // D[k] + 1)
            X[k] = min(M - 1, max(0, q * D[k] + rng.randrange(-2, 3)))
        q, r, fl = f.div(X, D)
        assert q == [a // b for a, b in zip(X, D)] and r == [a % b for a, b in zip(X, D)], tag
        assert not fl.any()
        S = [rng.randrange(1, min(L + 40, 2047)) for _ in range(N)]
        for k in range(0, N, 5):
            base = rng.randrange(max(1, M >> S[k])) << S[k]
            X[k] = min(M - 1, max(0, base + rng.randrange(-2, 3)))
        assert f.scale(X, S) == [a >> s for a, s in zip(X, S)], tag
        vals, ok = f.to_binary(f.res(X))
        assert ok.all() and vals == X, tag
        assert np.array_equal(f.from_binary(X, fc.fc_binary_limbs(f.h)), f.res(X)), tag
        # the integer-pipe evaluation: the reference's device doubles on its
        # common path, the rare path exactly for zero
        x = f.res(X)
        st, iv = np.zeros(N, np.int32), np.zeros(N, IV)
        fc.fc_eval(f.h, f.P(x), ctypes.c_long(N), f.P(st), f.P(iv))
        want = orcs[tag].eval(x.view(np.int32), path=O.PATH_DEVICE)
        common = st == 0
        assert iv[common].tobytes() == want[common].tobytes(), tag
        assert all((s == 2) == (v == 0) for s, v in zip(st, X)) and not (st == 8).any(), tag
        # the fast form (no mixed-radix step) on the numbers below M/2
        low = [v for v in X if v < M // 2]
        if low:
            xl = f.res(low)
            st, iv = np.zeros(len(low), np.int32), np.zeros(len(low), IV)
            fc.fc_eval_fast(f.h, f.P(xl), ctypes.c_long(len(low)), f.P(st), f.P(iv))
            want = orcs[tag].eval(xl.view(np.int32), path=O.PATH_DEVICE_FAST)
            assert iv[st == 0].tobytes() == want[st == 0].tobytes(), tag
        # the one-ulp evaluation encloses X/M wherever it certifies
        few = X[:12]
        xf = f.res(few)  # kept alive across the call
        ok, iv = np.zeros(len(few), np.int32), np.zeros(len(few), IV)
        fc.fc_eval_tight(f.h, f.P(xf), ctypes.c_long(len(few)), f.P(ok), f.P(iv))
        for k in np.nonzero(ok)[0]:
            lo = er_fraction(iv[k]["low"]["frac"], iv[k]["low"]["exp"])
            up = er_fraction(iv[k]["upp"]["frac"], iv[k]["upp"]["exp"])
            assert lo < Fraction(few[k], M) <= up and up - lo <= Fraction(2) ** (int(iv[k]["low"]["exp"]) - 52), tag
        rounds += 1
    for f in ctxs.values():
        fc.fc_destroy(f.h)


def test_directed_product_quotient_on_the_integer_pipe(fc):
    """(a b) / c rounded down and up on the integer pipe (the mp_int product's
    interval bound) equals the oracle's IEEE directed-rounding product then
    quotient, wherever it does not defer to the FP64 instructions"""
    from oracle import oracle as O
    L = O.lib()
    rng = np.random.default_rng(8)
    n = 20000
    a = rng.uniform(1.0, 2.0, n) * rng.choice([1.0, -1.0], n)
    b = rng.uniform(1.0, 2.0, n) * rng.choice([1.0, -1.0], n)
    c = rng.uniform(0.5, 1.0, n)
    a[:8] = [0.0, -0.0, 1.0, 1.0, 2 - 2 ** -52, 1.5, 1.0, 1.25]
    b[:8] = [1.5, 1.5, 0.0, 1.0, 2 - 2 ** -52, 1.0 + 2 ** -52, 1.0, 1.75]
    c[:8] = [0.75, 0.75, 0.5, 1.0, 0.5 + 2 ** -53, 1 - 2 ** -53, 0.5, 0.875]
    c[8:40] = 0.5 + np.arange(32) * 2.0 ** -53  # divisors with exact and near-exact quotients
    for up in (0, 1):
        out = np.zeros(n)
        ok = np.zeros(n, np.int32)
        fc.fc_dmuldiv(ctypes.c_void_p(a.ctypes.data), ctypes.c_void_p(b.ctypes.data), ctypes.c_void_p(c.ctypes.data),
                      ctypes.c_long(n), up, ctypes.c_void_p(out.ctypes.data), ctypes.c_void_p(ok.ctypes.data))
        assert not (ok < 0).any()  # the reciprocal form agrees with the division form
        assert ok.mean() > 0.99
        mul, div = (3, 5) if up else (2, 4)
        want = np.array([L.oracle_d_op(div, L.oracle_d_op(mul, x, y), z) for x, y, z in zip(a, b, c)])
        sel = ok.astype(bool)
        assert np.array_equal(out[sel].view(np.uint64), want[sel].view(np.uint64))
