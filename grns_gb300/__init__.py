"""grns_gb300 -- GB300-native RNS interval-evaluation path (host side).

Python mirror of the reference library's interface for this path
(kisupov/grns): the same operation names and argument meanings, applied to
whole device arrays through the C ABI of libgrns_gb300.so.

    ctx = RNSContext(moduli)                  # rns_const_init() + mpint_const_init()
    ctx = RNSContext.from_params("params.h")  # a moduli set in the reference's params.h format
    ev  = ctx.rns_eval_compute(x)             # cuda::rns_eval_compute  (src/rnseval.cuh:182)
    s   = ctx.rns_cmp(x, y)                   # cuda::rns_cmp           (src/rnscmp.cuh:55)
    q,r = ctx.rns_div(x, d)                   # cuda::rns_div           (src/rnsdiv.cuh:128)
    z   = ctx.rns_scale2pow(x, D)             # cuda::rns_scale2pow     (src/rnsscal.cuh:207)
    z   = ctx.mpint_add(a, b) / mpint_sub / mpint_mul / mpint_div
                                              (src/mpint.cuh:336/:407/:478/:511)
    v,i = ctx.rns_max(x)                      # cuda::rns_max           (src/dpp/rnsmax.cuh:129)
    a   = ctx.mrc(x)                          # cuda::mrc               (src/mrc.cuh:101)
    x   = ctx.rns_from_binary(limbs) / w = ctx.rns_to_binary(x)
                                              # rns_from_binary / rns_to_binary (src/rnsbase.cuh:253/:277)
    m   = ctx.mpint_set_binary(limbs, signs) / w,s = ctx.mpint_get_binary(m)
                                              # mpint_set_mpz / mpint_get_mpz (src/mpint.cuh:74/:100)

RNS arrays are int32 CUDA tensors: layout "soa" is shape (n, count) (residue
i of every number contiguous, the native layout), "aos" is shape (count, n)
(the reference layout).  Interval evaluations come back as uint8 tensors of
32 bytes per number (interval_t); `intervals_to_numpy` views them on the
host.  mp_int arrays are uint8 tensors of count * GRNS_MPINT_BYTES(n).
torch is used only as device-memory and stream plumbing.
"""
import ctypes

import numpy as np

from . import native
from .native import GrnsError, check

ER_DTYPE = np.dtype([("frac", "<f8"), ("exp", "<i8")])
IV_DTYPE = np.dtype([("low", ER_DTYPE), ("upp", ER_DTYPE)])
LAYOUTS = {"soa": 0, "aos": 1}
SUPPORTED_N = (4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 32, 64, 128, 256)

FLAG_INVALID_INPUT = 1
FLAG_DIV_BY_ZERO = 2
FLAG_ITER_CAP = 4
FLAG_OVERFLOW = 8
FLAG_MAY_OVERFLOW = 16


def mpint_bytes(n):
    return ((4 * n + 4 + 7) // 8) * 8 + 32


def mpint_dtype(n):
    """numpy dtype with the byte layout of mp_int_t (reference src/types.cuh:45)"""
    off = ((4 * n + 4 + 7) // 8) * 8
    return np.dtype({"names": ["digits", "sign", "eval"], "formats": [("<i4", (n,)), "<i4", (ER_DTYPE, (2,))],
                     "offsets": [0, 4 * n, off], "itemsize": off + 32})


def ints_to_limbs(values, limbs):
    """(count, limbs) int32 array of little-endian 32-bit limbs of nonnegative Python ints"""
    out = np.zeros((len(values), limbs), dtype=np.uint32)
    for k, v in enumerate(values):
        v = int(v)
        if v < 0 or v.bit_length() > 32 * limbs:
            raise ValueError("value out of range for the limb count")
        for j in range(limbs):
            out[k, j] = v & 0xFFFFFFFF
            v >>= 32
    return out.view(np.int32)


def limbs_to_ints(words):
    """Python ints from a (count, limbs) array of little-endian 32-bit limbs"""
    w = np.ascontiguousarray(words).view(np.uint32)
    return [int.from_bytes(row.astype("<u4").tobytes(), "little") for row in w]


def intervals_to_numpy(t):
    """device uint8 tensor of interval_t -> numpy structured array"""
    return t.cpu().numpy().view(IV_DTYPE)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def _stream(stream):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def parse_params(text):
    """(moduli, stated RNS_MODULI_PRODUCT_LOG2 or None) of a moduli set in the
    reference's params.h format (src/params.h); raises GrnsError on bad text"""
    t = text.encode() if isinstance(text, str) else bytes(text)
    n, lg = ctypes.c_int(0), ctypes.c_int(-1)
    check(native.lib().grns_params_parse(t, None, 0, ctypes.byref(n), ctypes.byref(lg)), "grns_params_parse")
    arr = (ctypes.c_int32 * max(1, n.value))()
    check(native.lib().grns_params_parse(t, arr, n.value, ctypes.byref(n), ctypes.byref(lg)), "grns_params_parse")
    return [int(v) for v in arr[:n.value]], (lg.value if lg.value >= 0 else None)


class RNSContext:
    """One moduli set resident on the current CUDA device (replaces the
    reference's process-global tables from rns_const_init)."""

    def __init__(self, moduli):
        import torch
        torch.cuda.init()
        self.moduli = [int(m) for m in moduli]
        self.n = len(self.moduli)
        arr = (ctypes.c_int32 * self.n)(*self.moduli)
        h = ctypes.c_void_p()
        check(native.lib().grns_ctx_create(arr, self.n, ctypes.byref(h)), "grns_ctx_create")
        self._h = h
        self.log2M = native.lib().grns_ctx_log2(h)
        self.M = 1
        for m in self.moduli:
            self.M *= m

    @classmethod
    def from_params(cls, source):
        """context for a params.h file (path) or its text: the reference's way of
        choosing a moduli set (src/params.h, the src/params/ catalogue)"""
        import os
        text = open(source).read() if os.path.exists(str(source)) else source
        moduli, lg = parse_params(text)
        ctx = cls(moduli)
        if lg is not None and lg != ctx.log2M:
            ctx.close()
            raise native.GrnsError(1, "RNS_MODULI_PRODUCT_LOG2 differs from floor(log2 M)")
        return ctx

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            native.lib().grns_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- constants ----
    def table(self, which):
        n, L = self.n, self.log2M
        spec = {0: (np.int32, n), 1: (np.float64, n), 2: (np.float64, n), 3: (np.float64, 1), 4: (np.int32, 1),
                5: (IV_DTYPE, 1), 6: (IV_DTYPE, 1), 7: (np.int32, n * n), 8: (np.int32, (L + 1) * n),
                9: (np.int32, 30), 10: (np.int32, 30 * n), 11: (np.int32, 30 * n)}[which]
        out = np.zeros(spec[1], dtype=spec[0])
        check(native.lib().grns_ctx_get_table(self._h, which, ctypes.c_void_p(out.ctypes.data), out.nbytes),
              "grns_ctx_get_table")
        return out

    def set_path(self, path):
        """"fast" (integer fixed-point enclosures, default) or "reference" (the
        reference's own FP64 algorithms) for cmp / div / scale2pow / max"""
        check(native.lib().grns_ctx_set_path(self._h, {"fast": 0, "reference": 1}[path]), "grns_ctx_set_path")

    @staticmethod
    def device_ceil_log2(xs):
        """ceil(log2 x) as the device evaluates it in the refinement loop (diagnostics)"""
        import torch
        x = torch.as_tensor(np.ascontiguousarray(xs, dtype=np.float64)).cuda()
        out = torch.empty(x.numel(), dtype=torch.int32, device=x.device)
        check(native.lib().grns_device_ceil_log2(_ptr(x), _ptr(out), x.numel(), _stream(None)),
              "grns_device_ceil_log2")
        return out.cpu().numpy()

    # ---- helpers ----
    def _count(self, x, layout):
        if x.dtype.itemsize != 4 or not x.is_cuda or not x.is_contiguous():
            raise ValueError("RNS arrays must be contiguous int32 CUDA tensors")
        if layout == "soa":
            if x.dim() != 2 or x.shape[0] != self.n:
                raise ValueError(f"SoA array must have shape ({self.n}, count)")
            return x.shape[1]
        if x.dim() != 2 or x.shape[1] != self.n:
            raise ValueError(f"AoS array must have shape (count, {self.n})")
        return x.shape[0]

    # ---- operations ----
    def rns_eval_compute(self, x, layout="soa", flags=None, stream=None):
        import torch
        count = self._count(x, layout)
        out = torch.empty(count * 32, dtype=torch.uint8, device=x.device)
        check(native.lib().grns_eval(self._h, _ptr(x), count, LAYOUTS[layout], _ptr(out), _ptr(flags),
                                     _stream(stream)), "grns_eval")
        return out

    def rns_eval_compute_fast(self, x, layout="soa", flags=None, stream=None):
        """cuda::rns_eval_compute_fast (src/rnseval.cuh:266): numbers below about M/2"""
        import torch
        count = self._count(x, layout)
        out = torch.empty(count * 32, dtype=torch.uint8, device=x.device)
        check(native.lib().grns_eval_fast(self._h, _ptr(x), count, LAYOUTS[layout], _ptr(out), _ptr(flags),
                                          _stream(stream)), "grns_eval_fast")
        return out

    def rns_eval_tight(self, x, layout="soa", flags=None, stream=None):
        """one-ulp certified enclosures of X/M, never wider than rns_eval_compute's
        (not bit-identical to them)"""
        import torch
        count = self._count(x, layout)
        out = torch.empty(count * 32, dtype=torch.uint8, device=x.device)
        check(native.lib().grns_eval_tight(self._h, _ptr(x), count, LAYOUTS[layout], _ptr(out), _ptr(flags),
                                           _stream(stream)), "grns_eval_tight")
        return out

    def rns_cmp(self, x, y, layout="soa", flags=None, stream=None):
        import torch
        count = self._count(x, layout)
        if self._count(y, layout) != count:
            raise ValueError("x and y differ in length")
        out = torch.empty(count, dtype=torch.int32, device=x.device)
        check(native.lib().grns_cmp(self._h, _ptr(x), _ptr(y), count, LAYOUTS[layout], _ptr(out), _ptr(flags),
                                    _stream(stream)), "grns_cmp")
        return out

    def rns_div(self, x, d, layout="soa", flags=None, stream=None):
        import torch
        count = self._count(x, layout)
        if self._count(d, layout) != count:
            raise ValueError("x and d differ in length")
        q = torch.empty_like(x)
        r = torch.empty_like(x)
        check(native.lib().grns_div(self._h, _ptr(x), _ptr(d), count, LAYOUTS[layout], _ptr(q), _ptr(r),
                                    _ptr(flags), _stream(stream)), "grns_div")
        return q, r

    # rns_div_fast (reference src/rnsdiv.cuh:67 host, :180 device) returns the
    # same q and r as rns_div; both map to grns_div
    rns_div_fast = rns_div

    def rns_scale2pow(self, x, D, layout="soa", flags=None, stream=None):
        """D: int (same exponent for all) or a uint32/int32 CUDA tensor of per-element exponents"""
        import torch
        count = self._count(x, layout)
        out = torch.empty_like(x)
        if isinstance(D, int):
            dptr, du = ctypes.c_void_p(0), D
        else:
            if D.numel() != count or D.dtype.itemsize != 4 or not D.is_cuda:
                raise ValueError("D must hold one 32-bit exponent per element")
            dptr, du = _ptr(D), 0
        check(native.lib().grns_scale2pow(self._h, _ptr(x), dptr, du, count, LAYOUTS[layout], _ptr(out),
                                          _ptr(flags), _stream(stream)), "grns_scale2pow")
        return out

    # ---- host-buffer forms (copies pipelined with the kernels) ----
    @staticmethod
    def _host(t, name):
        if t.is_cuda or not t.is_contiguous() or t.dtype.itemsize != 4:
            raise ValueError(f"{name} must be a contiguous 32-bit CPU tensor (page-locked for overlap)")

    def _host_count(self, x, layout):
        self._host(x, "x")
        if x.dim() != 2 or x.shape[0 if layout == "soa" else 1] != self.n:
            raise ValueError("RNS host array has the wrong shape for the layout")
        return x.shape[1] if layout == "soa" else x.shape[0]

    def rns_div_host(self, x, d, layout="soa", flags=None, chunks=0, stream=None):
        """rns_div over host arrays: (q, r) host tensors (page-locked like x)"""
        import torch
        count = self._host_count(x, layout)
        self._host(d, "d")
        pin = x.is_pinned()
        q = torch.empty(x.shape, dtype=x.dtype, pin_memory=pin)
        r = torch.empty(x.shape, dtype=x.dtype, pin_memory=pin)
        check(native.lib().grns_div_host(self._h, _ptr(x), _ptr(d), count, LAYOUTS[layout], _ptr(q), _ptr(r),
                                         _ptr(flags), chunks, _stream(stream)), "grns_div_host")
        return q, r

    def rns_scale2pow_host(self, x, D, layout="soa", flags=None, chunks=0, stream=None):
        """rns_scale2pow over host arrays; D an int or a host tensor of per-element exponents"""
        import torch
        count = self._host_count(x, layout)
        out = torch.empty(x.shape, dtype=x.dtype, pin_memory=x.is_pinned())
        if isinstance(D, int):
            dptr, du = ctypes.c_void_p(0), D
        else:
            self._host(D, "D")
            dptr, du = _ptr(D), 0
        check(native.lib().grns_scale2pow_host(self._h, _ptr(x), dptr, du, count, LAYOUTS[layout], _ptr(out),
                                               _ptr(flags), chunks, _stream(stream)), "grns_scale2pow_host")
        return out

    def _mpint(self, fn, x, y, flags, stream):
        import torch
        nb = mpint_bytes(self.n)
        if x.numel() % nb or x.numel() != y.numel():
            raise ValueError("mp_int arrays must be count * mpint_bytes(n) bytes and of equal length")
        count = x.numel() // nb
        out = torch.empty_like(x)
        check(fn(self._h, _ptr(x), _ptr(y), count, _ptr(out), _ptr(flags), _stream(stream)), fn.__name__)
        return out

    def mpint_add(self, x, y, flags=None, stream=None):
        return self._mpint(native.lib().grns_mpint_add, x, y, flags, stream)

    def mpint_sub(self, x, y, flags=None, stream=None):
        return self._mpint(native.lib().grns_mpint_sub, x, y, flags, stream)

    def mpint_mul(self, x, y, flags=None, stream=None):
        return self._mpint(native.lib().grns_mpint_mul, x, y, flags, stream)

    def mpint_div(self, x, y, flags=None, stream=None):
        """Euclidean quotient x / y (cuda::mpint_div, src/mpint.cuh:511)."""
        return self._mpint(native.lib().grns_mpint_div, x, y, flags, stream)

    def mrc(self, x, layout="soa", flags=None, stream=None):
        """mixed-radix digits of each number, in the layout of x (cuda::mrc, src/mrc.cuh:101)"""
        import torch
        count = self._count(x, layout)
        out = torch.empty_like(x)
        check(native.lib().grns_mrc(self._h, _ptr(x), count, LAYOUTS[layout], _ptr(out), _ptr(flags),
                                    _stream(stream)), "grns_mrc")
        return out

    # ---- binary <-> RNS conversion ----
    @property
    def binary_limbs(self):
        """32-bit limbs of an integer below M"""
        return native.lib().grns_ctx_binary_limbs(self._h)

    @staticmethod
    def _words(words):
        if words.dtype.itemsize != 4 or not words.is_cuda or not words.is_contiguous() or words.dim() != 2:
            raise ValueError("binary integers must be a contiguous (count, limbs) 32-bit CUDA tensor")
        return words.shape[0], words.shape[1]

    def rns_from_binary(self, words, layout="soa", stream=None):
        """residues of nonnegative integers given as (count, limbs) little-endian
        32-bit limbs (rns_from_binary, src/rnsbase.cuh:253)"""
        import torch
        count, limbs = self._words(words)
        shape = (self.n, count) if layout == "soa" else (count, self.n)
        out = torch.empty(shape, dtype=torch.int32, device=words.device)
        check(native.lib().grns_from_binary(self._h, _ptr(words), limbs, count, LAYOUTS[layout], _ptr(out),
                                            _stream(stream)), "grns_from_binary")
        return out

    def rns_to_binary(self, x, layout="soa", limbs=None, flags=None, stream=None):
        """X in [0, M) as (count, limbs) little-endian 32-bit limbs (rns_to_binary, src/rnsbase.cuh:277)"""
        import torch
        count = self._count(x, layout)
        limbs = self.binary_limbs if limbs is None else limbs
        out = torch.empty((count, limbs), dtype=torch.int32, device=x.device)
        check(native.lib().grns_to_binary(self._h, _ptr(x), count, LAYOUTS[layout], _ptr(out), limbs, _ptr(flags),
                                          _stream(stream)), "grns_to_binary")
        return out

    def mpint_set_binary(self, words, signs=None, stream=None):
        """mp_int_t records of sign-magnitude integers (mpint_set_mpz, src/mpint.cuh:74):
        magnitudes as (count, limbs) limbs, signs an int32 CUDA tensor (nonzero: negative) or None"""
        import torch
        count, limbs = self._words(words)
        if signs is not None and (signs.numel() != count or signs.dtype.itemsize != 4 or not signs.is_cuda):
            raise ValueError("signs must hold one int32 per integer")
        out = torch.empty(count * mpint_bytes(self.n), dtype=torch.uint8, device=words.device)
        check(native.lib().grns_mpint_from_binary(self._h, _ptr(words), limbs, _ptr(signs), count, _ptr(out),
                                                  _stream(stream)), "grns_mpint_from_binary")
        return out

    def mpint_get_binary(self, x, limbs=None, flags=None, stream=None):
        """(magnitudes as (count, limbs) limbs, signs) of mp_int_t records (mpint_get_mpz, src/mpint.cuh:100)"""
        import torch
        nb = mpint_bytes(self.n)
        if x.numel() % nb:
            raise ValueError("mp_int arrays must be count * mpint_bytes(n) bytes")
        count = x.numel() // nb
        limbs = self.binary_limbs if limbs is None else limbs
        words = torch.empty((count, limbs), dtype=torch.int32, device=x.device)
        signs = torch.empty(count, dtype=torch.int32, device=x.device)
        check(native.lib().grns_mpint_to_binary(self._h, _ptr(x), count, _ptr(words), limbs, _ptr(signs),
                                                _ptr(flags), _stream(stream)), "grns_mpint_to_binary")
        return words, signs

    def rns_max(self, x, layout="soa", scratch=None, stream=None):
        """returns (value residues int32[n], index int64[1]) on the device"""
        import torch
        count = self._count(x, layout)
        val = torch.zeros(self.n, dtype=torch.int32, device=x.device)
        idx = torch.empty(1, dtype=torch.int64, device=x.device)
        nbytes = scratch.numel() if scratch is not None else 0
        check(native.lib().grns_max(self._h, _ptr(x), count, LAYOUTS[layout], _ptr(val), _ptr(idx), _ptr(scratch),
                                    nbytes, _stream(stream)), "grns_max")
        return val, idx

    def max_scratch_size(self, count):
        v = ctypes.c_size_t()
        check(native.lib().grns_max_scratch_size(self._h, count, ctypes.byref(v)), "grns_max_scratch_size")
        return v.value


def rns_const_init(moduli):
    """reference-named constructor: a context for one moduli set"""
    return RNSContext(moduli)
