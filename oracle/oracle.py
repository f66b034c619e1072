"""ORACLE -- test infrastructure only.

Python access to the C restatement oracle (oracle/grns_oracle.c) and an
exact big-integer reference (Python ints) for the RNS operations of
kisupov/grns.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline may import this module, and only as the checker.

Arrays of RNS numbers are numpy int32 of shape (N, n) in the reference's
AoS layout ([x1..xn][x1..xn]...).  Interval evaluations are numpy structured
arrays with the interval_t layout (reference src/types.cuh:25).
"""
import ctypes
from fractions import Fraction
from math import gcd

import numpy as np

from . import build_oracle

ER_DTYPE = np.dtype([("frac", "<f8"), ("exp", "<i8")])
IV_DTYPE = np.dtype([("low", ER_DTYPE), ("upp", ER_DTYPE)])

PATH_HOST, PATH_DEVICE, PATH_HOST_FAST, PATH_DEVICE_PARALLEL, PATH_DEVICE_FAST = 0, 1, 2, 3, 4
SUPPORTED_N = (4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 32, 64, 128, 256)

_lib = None


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else ctypes.c_void_p(0)


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = ctypes.CDLL(path)
        L.oracle_ctx_create.restype = ctypes.c_void_p
        L.oracle_ctx_create.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.oracle_ctx_destroy.argtypes = [ctypes.c_void_p]
        L.oracle_n.argtypes = [ctypes.c_void_p]
        L.oracle_log2.argtypes = [ctypes.c_void_p]
        L.oracle_max.restype = ctypes.c_long
        L.oracle_max.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_long]
        L.oracle_d_op.restype = ctypes.c_double
        L.oracle_d_op.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double]
        L.oracle_log2_recorded.restype = ctypes.c_long
        L.oracle_log2_record.argtypes = [ctypes.c_void_p, ctypes.c_long]
        L.oracle_log2_table.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_long]
        for name in ("oracle_eval", "oracle_cmp", "oracle_div", "oracle_scale2pow", "oracle_mrc",
                     "oracle_mpint", "oracle_consts"):
            getattr(L, name).restype = None
        _lib = L
    return _lib


def mpint_dtype(n):
    """numpy dtype with the byte layout of the reference mp_int_t (src/types.cuh:45)."""
    eval_off = ((4 * n + 4 + 7) // 8) * 8
    return np.dtype({"names": ["digits", "sign", "eval"],
                     "formats": [("<i4", (n,)), "<i4", (ER_DTYPE, (2,))],
                     "offsets": [0, 4 * n, eval_off],
                     "itemsize": eval_off + 32})


class Oracle:
    """One moduli set (the reference's params.h convention)."""

    def __init__(self, moduli):
        self.moduli = [int(m) for m in moduli]
        self.n = len(self.moduli)
        arr = np.asarray(self.moduli, dtype=np.int32)
        self._h = lib().oracle_ctx_create(_p(arr), self.n)
        if not self._h:
            raise ValueError("unsupported moduli set for the oracle")
        self.log2M = lib().oracle_log2(self._h)
        self.M = 1
        for m in self.moduli:
            self.M *= m
        self.exact = Exact(self.moduli)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().oracle_ctx_destroy(self._h)
            self._h = None

    # ---- constants (rns_const_init, reference src/rnsbase.cuh:324) ----
    def consts(self):
        n, L = self.n, self.log2M
        c = dict(w=np.zeros(n, np.int32), recip_rd=np.zeros(n), recip_ru=np.zeros(n),
                 acc=np.zeros(1), ref_factor=np.zeros(1, np.int32), unit=np.zeros(1, IV_DTYPE),
                 inv_unit=np.zeros(1, IV_DTYPE), mrc_inv=np.zeros((n, n), np.int32),
                 pow2=np.zeros((L + 1, n), np.int32), m_pow2_res=np.zeros(30, np.int32),
                 mi_pow2_res=np.zeros((30, n), np.int32), pow2_inv=np.zeros((30, n), np.int32))
        lib().oracle_consts(ctypes.c_void_p(self._h), *[_p(c[k]) for k in (
            "w", "recip_rd", "recip_ru", "acc", "ref_factor", "unit", "inv_unit", "mrc_inv", "pow2",
            "m_pow2_res", "mi_pow2_res", "pow2_inv")])
        return c

    # ---- batch operations on AoS arrays ----
    def eval(self, x, path=PATH_DEVICE, threads=1):
        x = np.ascontiguousarray(x, dtype=np.int32)
        out = np.zeros(x.shape[0], IV_DTYPE)
        lib().oracle_eval(ctypes.c_void_p(self._h), _p(x), ctypes.c_long(x.shape[0]), _p(out), path, threads)
        return out

    def log2_inputs(self, x, cap=1 << 20, path=PATH_DEVICE):
        """the distinct values whose ceil(log2) the device-path refinement loop
        evaluates for these numbers (sorted)"""
        buf = np.zeros(cap)
        lib().oracle_log2_record(_p(buf), cap)
        self.eval(x, path=path)
        n = lib().oracle_log2_recorded()
        return np.unique(buf[:n])

    def eval_with_device_log2(self, x, xs, cs, path=PATH_DEVICE):
        """device-path evaluation using the device's ceil(log2 x) values `cs` for inputs `xs`"""
        xs = np.ascontiguousarray(xs, dtype=np.float64)
        cs = np.ascontiguousarray(cs, dtype=np.int32)
        order = np.argsort(xs)
        xs, cs = xs[order], cs[order]
        lib().oracle_log2_table(_p(xs), _p(cs), len(xs))
        try:
            return self.eval(x, path=path)
        finally:
            lib().oracle_log2_table(ctypes.c_void_p(0), ctypes.c_void_p(0), 0)

    def cmp(self, x, y, path=PATH_DEVICE, threads=1):
        x = np.ascontiguousarray(x, dtype=np.int32)
        y = np.ascontiguousarray(y, dtype=np.int32)
        out = np.zeros(x.shape[0], np.int32)
        lib().oracle_cmp(ctypes.c_void_p(self._h), _p(x), _p(y), ctypes.c_long(x.shape[0]), _p(out), path, threads)
        return out

    def div(self, x, d, path=PATH_DEVICE, fast=0, threads=1):
        x = np.ascontiguousarray(x, dtype=np.int32)
        d = np.ascontiguousarray(d, dtype=np.int32)
        q = np.zeros_like(x)
        r = np.zeros_like(x)
        lib().oracle_div(ctypes.c_void_p(self._h), _p(x), _p(d), ctypes.c_long(x.shape[0]), _p(q), _p(r),
                         path, fast, threads)
        return q, r

    def scale2pow(self, x, D, path=PATH_DEVICE, gpu_quirk=0, threads=1):
        x = np.ascontiguousarray(x, dtype=np.int32)
        D = np.ascontiguousarray(D, dtype=np.uint32)
        out = np.zeros_like(x)
        lib().oracle_scale2pow(ctypes.c_void_p(self._h), _p(x), _p(D), ctypes.c_long(x.shape[0]), _p(out),
                               path, gpu_quirk, threads)
        return out

    def mrc(self, x, path=PATH_DEVICE):
        x = np.ascontiguousarray(x, dtype=np.int32)
        out = np.zeros_like(x)
        lib().oracle_mrc(ctypes.c_void_p(self._h), _p(x), ctypes.c_long(x.shape[0]), _p(out), path)
        return out

    def mpint(self, op, x, y, path=PATH_DEVICE, threads=1):
        """op: 'add' | 'sub' | 'mul' | 'div'; x, y arrays of mpint_dtype(n). Returns (out, overflow_flags)."""
        code = {"add": 0, "sub": 1, "mul": 2, "div": 3}[op]
        x = np.ascontiguousarray(x)
        y = np.ascontiguousarray(y)
        out = np.zeros(x.shape[0], mpint_dtype(self.n))
        flags = np.zeros(x.shape[0], np.int32)
        lib().oracle_mpint(ctypes.c_void_p(self._h), code, _p(x), _p(y), ctypes.c_long(x.shape[0]), _p(out),
                           _p(flags), path, threads)
        return out, flags

    def max(self, x):
        x = np.ascontiguousarray(x, dtype=np.int32)
        return int(lib().oracle_max(ctypes.c_void_p(self._h), _p(x), ctypes.c_long(x.shape[0])))

    def mpint_from_ints(self, values, path=PATH_DEVICE):
        """mp_int_t array from Python ints (sign + residues + interval evaluation of |v|)."""
        out = np.zeros(len(values), mpint_dtype(self.n))
        mags = [abs(int(v)) for v in values]
        out["digits"] = self.exact.to_rns(mags)
        out["sign"] = [1 if v < 0 else 0 for v in values]
        ev = self.eval(out["digits"], path=path)
        out["eval"][:, 0] = ev["low"]
        out["eval"][:, 1] = ev["upp"]
        return out


def er_value(frac, exp):
    """Exact rational value of an extended-range float."""
    return Fraction(float(frac)) * (Fraction(2) ** int(exp))


class Exact:
    """Exact reference arithmetic over Python ints (the role GMP/MPFR play in
    the reference's tests: tests/test_perf_rnscmp.cu:132, test_perf_rnsdiv.cu:237,
    test_perf_mpint.cu:86)."""

    def __init__(self, moduli):
        self.moduli = [int(m) for m in moduli]
        self.M = 1
        for m in self.moduli:
            self.M *= m
        self.basis = []
        for m in self.moduli:
            Mi = self.M // m
            self.basis.append(Mi * pow(Mi, -1, m))

    def to_rns(self, values):
        return np.array([[v % m for m in self.moduli] for v in values], dtype=np.int32).reshape(len(values), len(self.moduli))

    def from_rns(self, rows):
        M, B = self.M, self.basis
        return [sum(int(r) * b for r, b in zip(row, B)) % M for row in np.asarray(rows)]

    def encloses(self, iv, values):
        """Bool array: low <= X/M <= upp for each interval and integer X (False
        for exponents no evaluation of X/M can have)."""
        out = []
        lim = 4 * self.M.bit_length() + 64
        for rec, v in zip(iv, values):
            if abs(int(rec["low"]["exp"])) > lim or abs(int(rec["upp"]["exp"])) > lim:
                out.append(False)
                continue
            lo = er_value(rec["low"]["frac"], rec["low"]["exp"])
            up = er_value(rec["upp"]["frac"], rec["upp"]["exp"])
            out.append(lo <= Fraction(v, self.M) <= up)
        return np.array(out)


def greedy_moduli(n, start=2 ** 30 - 1):
    """Pairwise-coprime odd integers taken greedily downward from `start`."""
    out, c = [], start
    while len(out) < n:
        if c % 2 == 1 and all(gcd(c, m) == 1 for m in out):
            out.append(c)
        c -= 1
    return out


# the reference's shipped default moduli set (src/params.h:32)
REFERENCE_DEFAULT_MODULI = [1283742825, 1283742827, 1283742829, 1283742833, 1283742839, 1283742841,
                            1283742847, 1283742851]
