"""GPU: a user kernel written against the reference's per-number device API
(cuda::rns_eval_compute, rns_cmp, rns_div, rns_scale2pow, mpint_mul, and
rns_const_init), compiled with include/grns/device.cuh in place of the
reference's headers (tests/native/device_drop_in.cu), returns what the C ABI
returns: the same interval bits, signs, quotients, remainders, scaled values
and mp_int results.  The moduli set is the reference's shipped params.h set,
given to the compiler as a params header."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from grns_gb300 import workload as W
from oracle import oracle as O
from tests.helpers import IV_DTYPE, moduli_for, mpint_dtype

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def user_lib(tmp_path_factory):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    mods = moduli_for("ref8")
    d = tmp_path_factory.mktemp("dropin")
    params = d / "params.h"
    params.write_text(f"#define RNS_MODULI_SIZE ({len(mods)})\n"
                      f"#define RNS_MODULI_VALUES {{{','.join(str(m) for m in mods)}}}\n")
    out = d / "libdropin.so"
    from grns_gb300.build import nvcc
    subprocess.run([nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "-shared",
                    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
                    "-include", str(params), os.path.join(ROOT, "tests", "native", "device_drop_in.cu"),
                    "-o", str(out), "-lcudart"], check=True, timeout=900)
    lib = ctypes.CDLL(str(out))
    lib.run_user_kernel.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 12
    return lib, mods


def test_user_kernel_matches_c_abi(user_lib):
    import grns_gb300 as G
    lib, mods = user_lib
    n, cnt, seed = len(mods), 700, 31
    ctx, orc = G.RNSContext(mods), O.Oracle(mods)
    x = W.uniform_residues(mods, cnt, seed, W.S_X, layout="aos")
    y = W.uniform_residues(mods, cnt, seed, W.S_Y, layout="aos")
    y[:50] = x[:50]  # ties
    dv, _ = W.divisors(mods, ctx.log2M, cnt, seed, layout="aos")
    D = W.shifts(cnt, min(900, ctx.log2M), seed)
    ma = orc.mpint_from_ints(W.mpint_values(cnt, ctx.log2M // 2 - 10, seed))
    mb = orc.mpint_from_ints(W.mpint_values(cnt, ctx.log2M // 2 - 10, seed + 1))
    ev = np.zeros(cnt, IV_DTYPE)
    cmp = np.zeros(cnt, np.int32)
    q, r, sc = (np.zeros((cnt, n), np.int32) for _ in range(3))
    mm = np.zeros(cnt, mpint_dtype(n))
    P = lambda a: ctypes.c_void_p(a.ctypes.data)  # noqa: E731
    x, y, dv = (np.ascontiguousarray(a, dtype=np.int32) for a in (x, y, dv))
    D = np.ascontiguousarray(D, dtype=np.uint32)
    assert lib.run_user_kernel(cnt, P(x), P(y), P(dv), P(D), P(ev), P(cmp), P(q), P(r), P(sc), P(ma), P(mb),
                               P(mm)) == 0

    tx, ty, td = (torch.from_numpy(a).cuda() for a in (x, y, dv))
    assert ev.tobytes() == ctx.rns_eval_compute(tx, layout="aos").cpu().numpy().tobytes()
    assert np.array_equal(cmp, ctx.rns_cmp(tx, ty, layout="aos").cpu().numpy())
    gq, gr = ctx.rns_div(tx, td, layout="aos")
    assert np.array_equal(q, gq.cpu().numpy()) and np.array_equal(r, gr.cpu().numpy())
    assert np.array_equal(sc, ctx.rns_scale2pow(tx, torch.from_numpy(D.view(np.int32)).cuda(),
                                                layout="aos").cpu().numpy())
    got = ctx.mpint_mul(torch.from_numpy(ma.view(np.uint8)).cuda(), torch.from_numpy(mb.view(np.uint8)).cuda())
    assert mm.tobytes() == got.cpu().numpy().tobytes()
