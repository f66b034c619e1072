"""Generate the golden vectors in tests/golden/ from the UNMODIFIED reference
library (kisupov/grns) compiled for the CPU by oracle/ref/build_ref.py.

For each moduli set the fixture holds seeded and special-value inputs and
the reference's outputs from BOTH of its paths: the host functions (global
namespace) and the device functions (namespace cuda, run on the CPU with
exact directed-rounding emulation).  Special values follow the reference's
own verification programs: consecutive numbers from 0 and from M-1
(tests/test_verify_rnseval.cu:87-149, tests/test_verify_mrc.cu:128-152),
powers of two 2^0..2^LOG2 (tests/test_perf_rnseval.cu:679-688), the mp_int
known-answer pair x=-55, y=13 (tests/test_verify_mpint.cu:92-93), signed
mp_int division operands with the Euclidean sign cases, binary <-> RNS
conversions through the reference's GMP routines, and the
extended-range doubles of tests/test_verify_extrange.cu:115-117.

Run from the repository root (all tags, or the tags named):
    GRNS_REFERENCE=<reference checkout> python tests/golden/make_golden.py [tag ...]
(needs the reference checkout and libgmp/libmpfr; the fixtures it writes are
committed, so the tests themselves never need the reference).
"""
import os
import random
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import refcheck  # noqa: E402
from oracle.oracle import REFERENCE_DEFAULT_MODULI  # noqa: E402
from oracle.ref import build_ref  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
TAGS = ["ref8", "g8", "g12", "g32", "g64", "p16", "p32", "p64"] + list(build_ref.CATALOGUE)


def special_values(M, log2M):
    v = [0, 1, 2, 3, M - 1, M - 2, M - 3, M // 2, M // 2 - 1, M // 2 + 1, M // 3, (2 * M) // 3]
    v += list(range(4, 10)) + [M - k for k in range(4, 10)]
    v += [1 << j for j in range(0, log2M + 1, max(1, log2M // 16))] + [1 << log2M, (1 << log2M) - 1]
    return v


def limbs_of(values, limbs):
    """(count, limbs) uint32 little-endian limbs of nonnegative ints"""
    out = np.zeros((len(values), limbs), np.uint32)
    for k, v in enumerate(values):
        for j in range(limbs):
            out[k, j] = (int(v) >> (32 * j)) & 0xFFFFFFFF
    return out


def main(tags):
    built = refcheck.build_ref.build(tags)
    if not built:
        raise SystemExit("reference checker libraries unavailable")
    for tag in tags:
        ref = refcheck.get(tag)
        moduli = build_ref.SETS[tag] or REFERENCE_DEFAULT_MODULI
        if isinstance(moduli, str):  # a params file of the reference's catalogue
            moduli = build_ref.catalogue_moduli(moduli)
        n = len(moduli)
        M = 1
        for m in moduli:
            M *= m
        L = ref.log2M
        rng = random.Random(20241203 + n)
        nrand = 48 if n <= 16 else 24
        X = special_values(M, L) + [rng.randrange(M) for _ in range(nrand)]
        Y = [rng.randrange(M) for _ in range(len(X))]
        # pairs with equal / adjacent values for the comparison tie paths
        Y[0], Y[1], Y[4], Y[7] = 0, 1, M - 1, M // 2 + 1
        Y[-1], Y[-2] = X[-1], X[-2] + 1 if X[-2] + 1 < M else 0
        N = len(X)
        res = lambda vals: np.array([[v % m for m in moduli] for v in vals], dtype=np.int32)  # noqa: E731
        x, y = res(X), res(Y)
        # divisors: random bit lengths plus edge cases
        Dv = []
        for k in range(N):
            b = rng.randrange(1, L + 1)
            Dv.append(rng.randrange(1 << (b - 1), 1 << b))
        Dv[0], Dv[1], Dv[2], Dv[3] = 1, 1, 2, M - 1
        Xd = list(X)
        Xd[5], Dv[5] = 12345, 12345  # x == d
        Xd[6], Dv[6] = 12344, 12345  # x < d
        d = res(Dv)
        xd = res(Xd)
        S = np.array([1 + (k * 37) % 60 for k in range(N)], dtype=np.uint32)
        S[:6] = [29, 30, 31, 60, L, L + 3]
        half = 1 << (L // 2 - 10 if L >= 40 else max(1, L // 2 - 1))  # products stay below M
        A = [rng.randrange(-half, half) for _ in range(N)]
        B = [rng.randrange(-half, half) for _ in range(N)]
        A[0], B[0] = -55, 13
        A[1], B[1] = 0, 7
        A[2], B[2] = 5, -5
        A[3], B[3] = -(half - 1), -(half - 2)
        fx = {"moduli": np.array(moduli, np.int64), "log2M": np.int64(L), "x": x, "y": y, "xd": xd, "d": d,
              "shift": S}
        for path, dev in (("dev", True), ("host", False)):
            fx[f"eval_{path}"] = ref.eval(x, dev=dev).view(np.uint8)
            fx[f"cmp_{path}"] = ref.cmp(x, y, dev=dev)
            q, r = ref.div(xd, d, dev=dev, fast=False)
            fx[f"div_q_{path}"], fx[f"div_r_{path}"] = q, r
            fx[f"scale_{path}"] = ref.scale2pow(x, S, dev=dev)
            fx[f"mrc_{path}"] = ref.mrc(x, dev=dev)
        # rns_eval_compute_fast requires a number "not too large" (src/rnseval.cuh:259;
        # the host form at :112 likewise): near M both forms' refinement index runs
        # past RNS_POW2 (the host form crashed on X = 2^47 of params.12m.47b.h), so
        # only X < M/2 here
        xf = res([v for v in X if v < M // 2])
        fx["xf"] = xf
        fx["eval_fast_host"] = ref.eval(xf, dev=False, fast=True).view(np.uint8)
        fx["eval_fast_dev"] = ref.eval(xf, dev=True, fast=True).view(np.uint8)
        # mp_int inputs through the reference's own constructor (host eval), then both op paths
        ma = np.concatenate([ref.mpint_from_str(v).view(np.uint8) for v in A])
        mb = np.concatenate([ref.mpint_from_str(v).view(np.uint8) for v in B])
        fx["mpint_a"], fx["mpint_b"] = ma, mb
        dt = refcheck.mpint_dtype(n)
        for op in ("add", "sub", "mul"):
            for path, dev in (("dev", True), ("host", False)):
                fx[f"mpint_{op}_{path}"] = ref.mpint(op, ma.view(dt), mb.view(dt), dev=dev).view(np.uint8)
        fx["mpint_kat"] = np.concatenate([ref.mpint_set_i(-55).view(np.uint8), ref.mpint_set_i(13).view(np.uint8)])
        # mpint_div (src/mpint.cuh:286/:511): signed dividends over the whole range,
        # nonzero divisors of random bit lengths, and the Euclidean sign cases
        rd = random.Random(20261203 + n)
        DA, DB = [], []
        for _ in range(nrand + 16):
            DA.append(rd.choice((-1, 1)) * rd.randrange(M))
            b = rd.randrange(1, L + 1)
            DB.append(rd.choice((-1, 1)) * rd.randrange(1 << (b - 1), 1 << b))
        for a, b in ((-55, 13), (55, -13), (-55, -13), (0, 7), (0, -7), (-52, 13), (52, -13), (M - 1, 1),
                     (-(M - 1), 1), (-(M - 2), M - 1), (M - 2, -(M - 1)), (-(M - 2), 2), (12345, 12345),
                     (-12344, 12345), (12344, -12345), (-(M - 1), -(M // 2))):
            DA.append(a)
            DB.append(b)
        da = np.concatenate([ref.mpint_from_str(v).view(np.uint8) for v in DA])
        db = np.concatenate([ref.mpint_from_str(v).view(np.uint8) for v in DB])
        fx["mpdiv_a"], fx["mpdiv_b"] = da, db
        for path, dev in (("dev", True), ("host", False)):
            fx[f"mpint_div_{path}"] = ref.mpint("div", da.view(dt), db.view(dt), dev=dev).view(np.uint8)
        # binary <-> RNS (rns_to_binary / rns_from_binary, src/rnsbase.cuh:277/:253;
        # mpint_get_mpz, src/mpint.cuh:100) as 32-bit little-endian limbs
        LM = (M.bit_length() + 31) // 32
        fx["tobin_words"] = limbs_of(ref.to_int(x), LM)
        rb = random.Random(20261204 + n)
        FB = [rb.randrange(1 << (32 * (LM + 2))) for _ in range(nrand)] + [0, 1, M - 1, M, M + 1, 2 * M + 5]
        FB += [rb.randrange(1 << b) for b in range(1, 32 * (LM + 2), max(1, 32 * (LM + 2) // 24))]
        fx["frombin_words"] = limbs_of(FB, LM + 2)
        fx["frombin_rns"] = ref.from_int(FB)
        mv = ref.mpint_to_int(da.view(dt))
        fx["mpint_tobin_words"] = limbs_of([abs(v) for v in mv], LM)
        fx["mpint_tobin_signs"] = np.array([1 if v < 0 else 0 for v in mv], np.int32)
        # extended-range known answers (tests/test_verify_extrange.cu:115-117)
        if tag == "ref8":
            dvals = [0.00003687544343, 0.41352, 12345.1443575]
            ers = []
            for dv in dvals:
                e, _ = ref.er(16, 0, (dv, 0))
                ers.append(e)
            rows = []
            for op in range(16):
                for dev in (0, 1):
                    out, c = ref.er(op, dev, ers[0], ers[1], ers[2])
                    rows.append((op, dev, out["frac"], out["exp"], c))
            fx["er_inputs"] = np.array([(e["frac"], e["exp"]) for e in ers], dtype=refcheck.ER_DTYPE).view(np.uint8)
            fx["er_results"] = np.array(rows, dtype=[("op", "<i4"), ("dev", "<i4"), ("frac", "<f8"), ("exp", "<i8"),
                                                     ("ret", "<i4")])
        np.savez_compressed(os.path.join(OUT, f"golden_{tag}.npz"), **fx)
        print(tag, "N =", N, "written")


if __name__ == "__main__":
    main(sys.argv[1:] or TAGS)
