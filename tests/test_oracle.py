"""CPU: the C restatement oracle reproduces the reference bit for bit.

Pinned two ways: against the committed golden vectors (generated from the
unmodified reference by tests/golden/make_golden.py) and, where the
reference checkout is present, against the reference compiled for the CPU
on fresh seeded inputs.  Integer results are also checked against exact
big-integer arithmetic, and interval bounds for enclosure of X/M.
"""
import random

import numpy as np
import pytest

from oracle import oracle as O
from oracle import refcheck
from tests.helpers import TAGS, golden, moduli_for, mpint_dtype, thin_golden

PATHS = (("dev", O.PATH_DEVICE), ("host", O.PATH_HOST))


@pytest.fixture(scope="module", params=TAGS)
def case(request):
    tag = request.param
    orc = O.Oracle(moduli_for(tag))
    return tag, orc, thin_golden(golden(tag), orc.n)


def test_constants_match_fixture_moduli(case):
    tag, orc, g = case
    assert list(g["moduli"]) == orc.moduli
    assert int(g["log2M"]) == orc.log2M


@pytest.mark.parametrize("path,code", PATHS)
def test_eval_matches_golden(case, path, code):
    tag, orc, g = case
    got = orc.eval(g["x"], path=code)
    assert got.view(np.uint8).tobytes() == g[f"eval_{path}"].tobytes()


def test_eval_fast_host_matches_golden(case):
    tag, orc, g = case
    assert orc.eval(g["xf"], path=O.PATH_HOST_FAST).view(np.uint8).tobytes() == g["eval_fast_host"].tobytes()


def test_eval_fast_device_matches_golden(case):
    """cuda::rns_eval_compute_fast, src/rnseval.cuh:266"""
    tag, orc, g = case
    assert orc.eval(g["xf"], path=O.PATH_DEVICE_FAST).view(np.uint8).tobytes() == g["eval_fast_dev"].tobytes()


@pytest.mark.parametrize("path,code", PATHS)
def test_cmp_div_scale_mrc_match_golden(case, path, code):
    tag, orc, g = case
    assert np.array_equal(orc.cmp(g["x"], g["y"], path=code), g[f"cmp_{path}"])
    q, r = orc.div(g["xd"], g["d"], path=code)
    assert np.array_equal(q, g[f"div_q_{path}"]) and np.array_equal(r, g[f"div_r_{path}"])
    s = orc.scale2pow(g["x"], g["shift"], path=code, gpu_quirk=int(code == O.PATH_DEVICE))
    assert np.array_equal(s, g[f"scale_{path}"])
    assert np.array_equal(orc.mrc(g["x"], path=code), g[f"mrc_{path}"])


@pytest.mark.parametrize("path,code", PATHS)
@pytest.mark.parametrize("op", ["add", "sub", "mul"])
def test_mpint_matches_golden(case, path, code, op):
    tag, orc, g = case
    dt = mpint_dtype(orc.n)
    out, _ = orc.mpint(op, g["mpint_a"].view(dt), g["mpint_b"].view(dt), path=code)
    assert out.view(np.uint8).tobytes() == g[f"mpint_{op}_{path}"].tobytes()


@pytest.mark.parametrize("path,code", PATHS)
def test_mpint_div_matches_golden(case, path, code):
    """mpint_div, host src/mpint.cuh:286 and device :511"""
    tag, orc, g = case
    dt = mpint_dtype(orc.n)
    out, _ = orc.mpint("div", g["mpdiv_a"].view(dt), g["mpdiv_b"].view(dt), path=code)
    assert out.view(np.uint8).tobytes() == g[f"mpint_div_{path}"].tobytes()


def test_mpint_div_euclidean(case):
    """x = q*y + r with 0 <= r < |y| for every golden pair"""
    tag, orc, g = case
    dt = mpint_dtype(orc.n)
    a, b = g["mpdiv_a"].view(dt), g["mpdiv_b"].view(dt)
    out, _ = orc.mpint("div", a, b, path=O.PATH_DEVICE)
    ex = orc.exact
    signed = lambda m: [(-v if s else v) for v, s in zip(ex.from_rns(m["digits"]), m["sign"])]  # noqa: E731
    X, Y, Q = signed(a), signed(b), signed(out)
    for x, y, q in zip(X, Y, Q):
        r = x - q * y
        assert 0 <= r < abs(y), (x, y, q)
    ivs = [{"low": e[0], "upp": e[1]} for e in out["eval"]]
    assert ex.encloses(ivs, ex.from_rns(out["digits"])).all()


def _ints(words):
    return [int.from_bytes(r.astype("<u4").tobytes(), "little") for r in np.asarray(words)]


def test_binary_conversion_matches_golden(case):
    """rns_to_binary / rns_from_binary (src/rnsbase.cuh:277/:253) and
    mpint_get_mpz (src/mpint.cuh:100) through GMP in the reference"""
    tag, orc, g = case
    ex = orc.exact
    assert ex.from_rns(g["x"]) == _ints(g["tobin_words"])
    vals = _ints(g["frombin_words"])
    assert np.array_equal(ex.to_rns([v % ex.M for v in vals]), g["frombin_rns"])
    dt = mpint_dtype(orc.n)
    m = g["mpdiv_a"].view(dt)
    mags = ex.from_rns(m["digits"])
    assert mags == _ints(g["mpint_tobin_words"])
    assert [int(s == 1 and v != 0) for s, v in zip(m["sign"], mags)] == list(g["mpint_tobin_signs"])


def test_mpint_known_answer(case):
    """x = -55, y = 13 (reference tests/test_verify_mpint.cu:92-93)"""
    tag, orc, g = case
    dt = mpint_dtype(orc.n)
    kat = g["mpint_kat"].view(dt)
    mine = orc.mpint_from_ints([-55, 13], path=O.PATH_HOST)
    assert mine.view(np.uint8).tobytes() == kat.view(np.uint8).tobytes()
    for op, exact in (("add", -42), ("sub", -68), ("mul", -715)):
        out, flags = orc.mpint(op, kat[:1], kat[1:], path=O.PATH_DEVICE)
        v = orc.exact.from_rns(out["digits"])[0]
        assert (-v if out["sign"][0] else v) == exact and flags[0] == 0


def test_results_exact_and_enclosing(case):
    tag, orc, g = case
    ex = orc.exact
    X, Y = ex.from_rns(g["x"]), ex.from_rns(g["y"])
    assert list(orc.cmp(g["x"], g["y"])) == [(a > b) - (a < b) for a, b in zip(X, Y)]
    Xd, D = ex.from_rns(g["xd"]), ex.from_rns(g["d"])
    q, r = orc.div(g["xd"], g["d"])
    assert ex.from_rns(q) == [a // b for a, b in zip(Xd, D)]
    assert ex.from_rns(r) == [a % b for a, b in zip(Xd, D)]
    s = orc.scale2pow(g["x"], g["shift"], path=O.PATH_DEVICE, gpu_quirk=0)
    assert ex.from_rns(s) == [a >> int(k) for a, k in zip(X, g["shift"])]
    for code in (O.PATH_DEVICE, O.PATH_HOST):
        assert ex.encloses(orc.eval(g["x"], path=code), X).all()


def test_max_exact(case):
    tag, orc, g = case
    X = orc.exact.from_rns(g["x"])
    i = orc.max(g["x"])
    assert X[i] == max(X) and i == X.index(max(X))
    assert orc.max(g["x"][:0]) == -1


def test_extrange_known_answers():
    g = golden("ref8")
    ins = g["er_inputs"].view(O.ER_DTYPE)
    # er_set_d of the reference's doubles lands frac in [1, 2)
    assert all(1.0 <= e["frac"] < 2.0 for e in ins)
    rows = g["er_results"]
    # rounding-down results never exceed rounding-up results (add, sub, mul, div, md)
    for lo_op, hi_op in ((1, 2), (4, 5), (7, 8), (10, 11), (12, 13)):
        for dev in (0, 1):
            lo = rows[(rows["op"] == lo_op) & (rows["dev"] == dev)][0]
            hi = rows[(rows["op"] == hi_op) & (rows["dev"] == dev)][0]
            assert O.er_value(lo["frac"], lo["exp"]) <= O.er_value(hi["frac"], hi["exp"])


@pytest.mark.parametrize("op", range(8))
def test_directed_rounding_emulation_brackets(op):
    """device rounding primitives: RD <= exact <= RU and adjacent doubles"""
    from fractions import Fraction
    L = O.lib()
    rng = random.Random(op)
    for _ in range(400):
        a = rng.uniform(-4, 4) * 2.0 ** rng.randint(-40, 40)
        b = rng.uniform(0.5, 4) * 2.0 ** rng.randint(-40, 40)
        base = op // 2 * 2 if op < 6 else 6
        lo, hi = L.oracle_d_op(base, a, b), L.oracle_d_op(base + 1, a, b)
        fa, fb = Fraction(a), Fraction(b)
        exact = {0: fa + fb, 2: fa * fb, 4: fa / fb, 6: fa - fb}[base]
        assert Fraction(lo) <= exact <= Fraction(hi)
        assert lo == hi or np.nextafter(lo, np.inf) == hi


@pytest.mark.parametrize("tag", [t for t in TAGS if not t.endswith("_n256")])
def test_oracle_vs_reference_build(tag):
    """fresh seeded inputs through the reference compiled for the CPU (skipped
    without the checkout).  The 256-moduli sets are pinned by their golden
    vectors only: the reference's constant setup takes ~40 s per set when its
    library loads."""
    if not refcheck.available(tag):
        pytest.skip("reference checker library not built here")
    ref = refcheck.get(tag)
    orc = O.Oracle(moduli_for(tag))
    a, b = ref.consts(), orc.consts()
    for k in a:
        assert a[k].tobytes() == b[k].tobytes(), k
    rng = random.Random(11)
    N = 500 if orc.n <= 16 else 150 if orc.n <= 64 else 40
    X = [rng.randrange(orc.M) for _ in range(N)]
    Y = [rng.randrange(orc.M) for _ in range(N)]
    x, y = orc.exact.to_rns(X), orc.exact.to_rns(Y)
    for dev, code in ((True, O.PATH_DEVICE), (False, O.PATH_HOST)):
        assert ref.eval(x, dev=dev).tobytes() == orc.eval(x, path=code).tobytes()
        assert np.array_equal(ref.cmp(x, y, dev=dev), orc.cmp(x, y, path=code))


@pytest.mark.parametrize("tag", ["g32", "p32", "g64", "p64"])
def test_parallel_order_pinned_on_reference_block_code(tag):
    """rns_eval_compute_parallel (src/rnseval.cuh:332) executed as one thread
    block of the reference's own code on the CPU (one host thread per CUDA
    thread, oracle/ref/ref_block.cpp) gives the oracle's n-threaded order
    (eval_dpar) bit for bit -- the order the device header's
    rns_eval_compute_parallel follows on the GPU; rns_cmp_parallel and
    mrc_pipeline give the serial results"""
    if not refcheck.block_available(tag):
        pytest.skip("reference block checker not built (no reference checkout)")
    orc, g, blk = O.Oracle(moduli_for(tag)), golden(tag), refcheck.block(tag)
    x = g["x"] if orc.n <= 32 else g["x"][:40]  # the special values lead the fixture
    got = blk.eval(x)
    assert got.tobytes() == orc.eval(x, path=O.PATH_DEVICE_PARALLEL).tobytes()
    assert (got != orc.eval(x, path=O.PATH_DEVICE)).any()  # the order differs from the serial tree's
    k = 8
    assert list(blk.cmp(x[:k], g["y"][:k])) == list(orc.cmp(x[:k], g["y"][:k], path=O.PATH_DEVICE))
    assert np.array_equal(blk.mrc(x), orc.mrc(x, path=O.PATH_DEVICE))
