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


@pytest.fixture(scope="module", params=["ref8", "g32", "g64", "cat6400_n256"])
def user_lib(request, tmp_path_factory):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    mods = moduli_for(request.param)
    d = tmp_path_factory.mktemp("dropin")
    params = d / "params.h"
    params.write_text(f"#define RNS_MODULI_SIZE ({len(mods)})\n"
                      f"#define RNS_MODULI_VALUES {{{','.join(str(m) for m in mods)}}}\n")
    out = d / "libdropin.so"
    from grns_gb300.build import nvcc
    subprocess.run([nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "-shared",
                    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-fvisibility=hidden",
                    "-I", os.path.join(ROOT, "include"),
                    "-include", str(params), os.path.join(ROOT, "tests", "native", "device_drop_in.cu"),
                    "-o", str(out), "-lcudart"], check=True, timeout=900)
    lib = ctypes.CDLL(str(out))
    lib.run_user_kernel.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 12
    lib.run_user_kernel2.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 17
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
    got = got.cpu().numpy().view(mpint_dtype(n))
    for field in ("digits", "sign", "eval"):
        assert mm[field].tobytes() == got[field].tobytes(), field


def test_user_kernel_more_and_n_threaded_forms(user_lib):
    """cuda::mpint_div, mrc, mrc_compare_rns, rns_div_fast, and the n-threaded
    forms (one block of n threads per number): rns_eval_compute_parallel in the
    reference's n-threaded summation order (oracle), rns_cmp_parallel,
    rns_div_parallel, mrc_pipeline, mrc_pipeline_msd, mrc_pipeline_compare_rns
    equal to the serial results"""
    import grns_gb300 as G
    lib, mods = user_lib
    n, cnt, seed = len(mods), 500, 41
    ctx, orc = G.RNSContext(mods), O.Oracle(mods)
    x = W.uniform_residues(mods, cnt, seed, W.S_X, layout="aos")
    y = W.uniform_residues(mods, cnt, seed, W.S_Y, layout="aos")
    y[:40] = x[:40]
    x[40:60] = orc.exact.to_rns(list(range(1, 21)))  # small values: the refinement loop
    x[60:70] = orc.exact.to_rns([orc.M - k for k in range(1, 11)])  # near M: the mixed-radix branch
    dv, _ = W.divisors(mods, ctx.log2M, cnt, seed, layout="aos")
    vals_a = [(-1) ** k * v for k, v in enumerate(W.mpint_values(cnt, ctx.log2M - 2, seed))]
    vals_b = [v if v else 1 for v in W.mpint_values(cnt, ctx.log2M // 2, seed + 1)]
    ma, mb = orc.mpint_from_ints(vals_a), orc.mpint_from_ints(vals_b)
    dt = mpint_dtype(n)
    md = np.zeros(cnt, dt)
    mr, q, r, pq, pr, pmr = (np.zeros((cnt, n), np.int32) for _ in range(6))
    mcmp, pcmp, pmsd, pmcmp = (np.zeros(cnt, np.int32) for _ in range(4))
    pev = np.zeros(cnt, IV_DTYPE)
    P = lambda a: ctypes.c_void_p(a.ctypes.data)  # noqa: E731
    rc = lib.run_user_kernel2(cnt, P(x), P(y), P(dv), P(ma), P(mb), P(md), P(mr), P(mcmp), P(q), P(r), P(pev),
                              P(pcmp), P(pq), P(pr), P(pmr), P(pmsd), P(pmcmp))
    assert rc == 0
    # serial
    dev = lambda t: torch.from_numpy(np.ascontiguousarray(t)).cuda()  # noqa: E731
    want_md = ctx.mpint_div(dev(ma.view(np.uint8)), dev(mb.view(np.uint8))).cpu().numpy().view(dt)
    for field in ("digits", "sign", "eval"):  # member by member: padding bytes are not written
        assert md[field].tobytes() == want_md[field].tobytes(), field
    want_mr = ctx.mrc(dev(x), layout="aos").cpu().numpy()
    bad = [k for k in range(cnt) if not (np.array_equal(mr[k], want_mr[k]) and np.array_equal(pmr[k], want_mr[k]))]
    assert not bad, [(k, x[k][:3].tolist(), mr[k][:3].tolist(), pmr[k][:3].tolist(), want_mr[k][:3].tolist())
                     for k in bad[:6]] + [len(bad)]
    want_cmp = ctx.rns_cmp(dev(x), dev(y), layout="aos").cpu().numpy()
    assert np.array_equal(mcmp, want_cmp) and np.array_equal(pcmp, want_cmp) and np.array_equal(pmcmp, want_cmp)
    wq, wr = ctx.rns_div(dev(x), dev(dv), layout="aos")
    for got in (q, pq):
        assert np.array_equal(got, wq.cpu().numpy())
    for got in (r, pr):
        assert np.array_equal(got, wr.cpu().numpy())
    assert np.array_equal(pmsd, want_mr[:, -1])
    # the n-threaded evaluation: the oracle's n-threaded order, with the device's ceil(log2)
    xs = orc.log2_inputs(x, path=O.PATH_DEVICE_PARALLEL)
    cs = ctx.device_ceil_log2(xs) if len(xs) else np.zeros(0, np.int32)
    want = orc.eval_with_device_log2(x, xs, cs, path=O.PATH_DEVICE_PARALLEL)
    assert pev.tobytes() == want.tobytes()
    assert orc.exact.encloses(pev, orc.exact.from_rns(x)).all()
