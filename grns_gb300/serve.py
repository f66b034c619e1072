"""Python access to the serving subsystem (grns_server_* in include/grns/grns.h):
device-resident arrays, request submission, continuous batching, latency stats."""
import ctypes

import numpy as np

from . import native
from .native import check

OPS = {"eval": 0, "cmp": 1, "div": 2, "scale2pow": 3, "max": 4, "mpint_add": 5, "mpint_sub": 6, "mpint_mul": 7,
       "mpint_div": 8}


class Server:
    def __init__(self, budget_bytes=0, slots=4, max_jobs=256, admission_timeout_ms=0, alloc_cap_bytes=0,
                 direct_min_count=0, gather_us=0):
        self.L = native.lib()
        opt = native.ServerOptions(budget_bytes, slots, max_jobs, admission_timeout_ms, direct_min_count,
                                   alloc_cap_bytes, gather_us, 0)
        h = ctypes.c_void_p()
        check(self.L.grns_server_create(ctypes.byref(opt), ctypes.byref(h)), "grns_server_create")
        self.h = h
        self.ctx_n = {}

    def close(self):
        if self.h is not None and self.h.value:
            self.L.grns_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_context(self, ctx):
        idx = ctypes.c_int()
        check(self.L.grns_server_add_context(self.h, ctx.handle, ctypes.byref(idx)), "grns_server_add_context")
        self.ctx_n[idx.value] = ctx.n
        return idx.value

    def put(self, ctx_index, array, kind=native.ARRAY_RNS, layout=0, count=None):
        """array: torch tensor or numpy array, copied into server memory as
        contiguous bytes (int32 for RNS and U32 arrays, uint8 records for
        mp_int arrays).  A CUDA tensor's pending work on the current stream
        finishes first, since the server copies on its own stream; a tensor
        written on another stream must be synchronised by the caller."""
        want = {native.ARRAY_RNS: (4,), native.ARRAY_U32: (4,), native.ARRAY_MPINT: (1,)}.get(kind, (1, 4))
        if array.dtype.itemsize not in want:
            raise ValueError(f"array of kind {kind} must have elements of {want[0]} bytes, not {array.dtype}")
        if hasattr(array, "is_cuda") and array.is_cuda:
            import torch
            array = array.contiguous()
            torch.cuda.current_stream(array.device).synchronize()
            src, on_dev = ctypes.c_void_p(array.data_ptr()), 1
            self._keep = array
        else:
            array = np.ascontiguousarray(array)
            src, on_dev = ctypes.c_void_p(array.ctypes.data), 0
            self._keep = array
        if count is None:
            count = array.shape[1] if (kind == native.ARRAY_RNS and layout == 0) else array.shape[0]
        hd = ctypes.c_uint64()
        check(self.L.grns_server_put(self.h, ctx_index, kind, src, on_dev, count, layout, ctypes.byref(hd)),
              "grns_server_put")
        return hd.value

    def get(self, handle, nbytes=None):
        cnt, nb = ctypes.c_int64(), ctypes.c_size_t()
        check(self.L.grns_server_array_info(self.h, handle, ctypes.byref(cnt), ctypes.byref(nb), None), "info")
        n = nb.value if nbytes is None else nbytes
        out = np.empty(n, np.uint8)
        check(self.L.grns_server_get(self.h, handle, ctypes.c_void_p(out.ctypes.data), n), "grns_server_get")
        return out

    def free(self, handle):
        check(self.L.grns_server_free(self.h, handle), "grns_server_free")

    def submit(self, op, ctx_index, a, b=0, count=0, D_uniform=0):
        r = native.Request(OPS[op] if isinstance(op, str) else op, ctx_index, count, a, b, D_uniform, 0)
        rid = ctypes.c_uint64()
        check(self.L.grns_server_submit(self.h, ctypes.byref(r), ctypes.byref(rid)), "grns_server_submit")
        return rid.value

    def cancel(self, rid):
        """cancel a request still waiting for admission (GrnsError BUSY once launched)"""
        check(self.L.grns_server_cancel(self.h, rid), "grns_server_cancel")

    def wait(self, rid, timeout_us=120_000_000):
        st, o0, o1 = ctypes.c_int32(), ctypes.c_uint64(), ctypes.c_uint64()
        check(self.L.grns_server_wait(self.h, rid, timeout_us, ctypes.byref(st), ctypes.byref(o0), ctypes.byref(o1)),
              "grns_server_wait")
        return st.value, o0.value, o1.value

    def poll(self, rid):
        d, st, o0, o1 = ctypes.c_int(), ctypes.c_int32(), ctypes.c_uint64(), ctypes.c_uint64()
        check(self.L.grns_server_poll(self.h, rid, ctypes.byref(d), ctypes.byref(st), ctypes.byref(o0),
                                      ctypes.byref(o1)), "grns_server_poll")
        return bool(d.value), st.value, o0.value, o1.value

    def stats(self):
        s = native.ServerStats()
        check(self.L.grns_server_stats_get(self.h, ctypes.byref(s)), "grns_server_stats_get")
        return {f: getattr(s, f) for f, _ in native.ServerStats._fields_}

    def reset_stats(self):
        check(self.L.grns_server_reset_stats(self.h), "grns_server_reset_stats")

    def set_gather_us(self, us):
        """the gathering window (grns_server_options.gather_us) on the live server"""
        check(self.L.grns_server_set_gather_us(self.h, int(us)), "grns_server_set_gather_us")
