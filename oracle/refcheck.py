"""ORACLE -- test infrastructure only.

ctypes access to the unmodified reference library compiled for the CPU
(oracle/_ref/libgrnsref_<tag>.so, built by oracle/ref/build_ref.py from the
reference checkout).  Used here to pin the C restatement and to generate the
golden vectors under tests/golden/.  Absent on machines without the
reference checkout; callers must skip when `available(tag)` is False.
"""
import ctypes
import os

import numpy as np

from .oracle import IV_DTYPE, ER_DTYPE, mpint_dtype
from .ref import build_ref

REF_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_ref")
SETS = build_ref.SETS
_cache = {}


def available(tag):
    return os.path.exists(os.path.join(REF_DIR, f"libgrnsref_{tag}.so"))


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


class Ref:
    def __init__(self, tag):
        path = os.path.join(REF_DIR, f"libgrnsref_{tag}.so")
        self.L = ctypes.CDLL(path)
        self.L.ref_init()
        self.n = self.L.ref_n()
        self.log2M = self.L.ref_log2()
        self.tag = tag
        self.moduli = SETS[tag]

    def consts(self):
        n, L = self.n, self.log2M
        c = dict(w=np.zeros(n, np.int32), recip_rd=np.zeros(n), recip_ru=np.zeros(n),
                 acc=np.zeros(1), ref_factor=np.zeros(1, np.int32), unit=np.zeros(1, IV_DTYPE),
                 inv_unit=np.zeros(1, IV_DTYPE), mrc_inv=np.zeros((n, n), np.int32),
                 pow2=np.zeros((L + 1, n), np.int32), m_pow2_res=np.zeros(30, np.int32),
                 mi_pow2_res=np.zeros((30, n), np.int32), pow2_inv=np.zeros((30, n), np.int32))
        self.L.ref_consts(*[_p(c[k]) for k in (
            "w", "recip_rd", "recip_ru", "acc", "ref_factor", "unit", "inv_unit", "mrc_inv", "pow2",
            "m_pow2_res", "mi_pow2_res", "pow2_inv")])
        return c

    def eval(self, x, dev=True, fast=False):
        x = np.ascontiguousarray(x, np.int32)
        out = np.zeros(x.shape[0], IV_DTYPE)
        fn = {(False, False): "ref_host_eval", (False, True): "ref_host_eval_fast",
              (True, False): "ref_dev_eval", (True, True): "ref_dev_eval_fast"}[(dev, fast)]
        getattr(self.L, fn)(_p(x), ctypes.c_long(x.shape[0]), _p(out))
        return out

    def cmp(self, x, y, dev=True):
        x = np.ascontiguousarray(x, np.int32)
        y = np.ascontiguousarray(y, np.int32)
        out = np.zeros(x.shape[0], np.int32)
        getattr(self.L, "ref_dev_cmp" if dev else "ref_host_cmp")(_p(x), _p(y), ctypes.c_long(x.shape[0]), _p(out))
        return out

    def div(self, x, d, dev=True, fast=False):
        x = np.ascontiguousarray(x, np.int32)
        d = np.ascontiguousarray(d, np.int32)
        q = np.zeros_like(x)
        r = np.zeros_like(x)
        getattr(self.L, "ref_dev_div" if dev else "ref_host_div")(_p(x), _p(d), ctypes.c_long(x.shape[0]),
                                                                  int(fast), _p(q), _p(r))
        return q, r

    def scale2pow(self, x, D, dev=True):
        x = np.ascontiguousarray(x, np.int32)
        D = np.ascontiguousarray(D, np.uint32)
        out = np.zeros_like(x)
        getattr(self.L, "ref_dev_scale2pow" if dev else "ref_host_scale2pow")(_p(x), _p(D), ctypes.c_long(x.shape[0]), _p(out))
        return out

    def mrc(self, x, dev=True):
        x = np.ascontiguousarray(x, np.int32)
        out = np.zeros_like(x)
        getattr(self.L, "ref_dev_mrc" if dev else "ref_host_mrc")(_p(x), ctypes.c_long(x.shape[0]), _p(out))
        return out

    def mpint(self, op, x, y, dev=True):
        code = {"add": 0, "sub": 1, "mul": 2, "div": 3}[op]
        x = np.ascontiguousarray(x)
        y = np.ascontiguousarray(y)
        out = np.zeros(x.shape[0], mpint_dtype(self.n))
        getattr(self.L, "ref_dev_mpint" if dev else "ref_host_mpint")(code, _p(x), _p(y), ctypes.c_long(x.shape[0]), _p(out))
        return out

    def mpint_set_i(self, v):
        out = np.zeros(1, mpint_dtype(self.n))
        self.L.ref_mpint_set_i(int(v), _p(out))
        return out

    def mpint_from_str(self, s):
        out = np.zeros(1, mpint_dtype(self.n))
        self.L.ref_mpint_from_str(str(s).encode(), _p(out))
        return out

    def from_int(self, values):
        """rns_from_binary of each nonnegative Python int (AoS int32 residues)"""
        out = np.zeros((len(values), self.n), np.int32)
        for k, v in enumerate(values):
            self.L.ref_rns_from_str(str(int(v)).encode(), _p(out[k]))
        return out

    def to_int(self, x):
        """rns_to_binary of each row of AoS residues, as Python ints"""
        x = np.ascontiguousarray(x, np.int32)
        buf = ctypes.create_string_buffer(2048)
        res = []
        for k in range(x.shape[0]):
            self.L.ref_rns_to_str(_p(x[k]), buf)
            res.append(int(buf.value.decode()))
        return res

    def mpint_to_int(self, m):
        """mpint_get_mpz of each mp_int_t record, as Python ints"""
        m = np.ascontiguousarray(m)
        buf = ctypes.create_string_buffer(2048)
        res = []
        for k in range(m.shape[0]):
            self.L.ref_mpint_to_str(_p(m[k:k + 1]), buf)
            res.append(int(buf.value.decode()))
        return res

    def er(self, op, dev, x, y=(0.0, 0), z=(0.0, 0)):
        a = np.array([x], ER_DTYPE)
        b = np.array([y], ER_DTYPE)
        c = np.array([z], ER_DTYPE)
        out = np.zeros(1, ER_DTYPE)
        self.L.ref_er.restype = ctypes.c_int
        r = self.L.ref_er(int(op), int(dev), _p(a), _p(b), _p(c), _p(out))
        return out[0], r


def get(tag):
    if tag not in _cache:
        _cache[tag] = Ref(tag)
    return _cache[tag]


def block_available(tag):
    return os.path.exists(os.path.join(REF_DIR, f"libgrnsref_block_{tag}.so"))


class Block:
    """The reference's n-threaded device functions run as one emulated thread
    block on the CPU (oracle/ref/ref_block.cpp; sets with n a multiple of 32)."""

    def __init__(self, tag):
        self.L = ctypes.CDLL(os.path.join(REF_DIR, f"libgrnsref_block_{tag}.so"))
        self.L.ref_block_init()
        self.n = self.L.ref_block_n()

    def eval(self, x):
        x = np.ascontiguousarray(x, np.int32)
        out = np.zeros(x.shape[0], IV_DTYPE)
        self.L.ref_block_eval(_p(x), ctypes.c_long(x.shape[0]), _p(out))
        return out

    def cmp(self, x, y):
        x, y = np.ascontiguousarray(x, np.int32), np.ascontiguousarray(y, np.int32)
        out = np.zeros(x.shape[0], np.int32)
        self.L.ref_block_cmp(_p(x), _p(y), ctypes.c_long(x.shape[0]), _p(out))
        return out

    def mrc(self, x):
        x = np.ascontiguousarray(x, np.int32)
        out = np.zeros_like(x)
        self.L.ref_block_mrc(_p(x), ctypes.c_long(x.shape[0]), _p(out))
        return out


def block(tag):
    key = ("block", tag)
    if key not in _cache:
        _cache[key] = Block(tag)
    return _cache[key]
