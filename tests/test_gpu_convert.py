"""GPU: binary <-> RNS conversion through the C ABI (rns_from_binary /
rns_to_binary, reference src/rnsbase.cuh:253/:277; mpint_set_mpz /
mpint_get_mpz, src/mpint.cuh:74/:100) against the reference's GMP results
(golden vectors) and exact integer arithmetic."""
import random

import numpy as np
import pytest

import grns_gb300 as G
from oracle import oracle as O
from tests.helpers import TAGS, golden, moduli_for, mpint_dtype, sized

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from grns_gb300 import native
    native.lib(build_if_missing=True)
    return torch.device("cuda:0")


@pytest.fixture(scope="module", params=TAGS)
def case(request, dev):
    tag = request.param
    mods = moduli_for(tag)
    return tag, G.RNSContext(mods), O.Oracle(mods), golden(tag)


def to_dev(a, layout):
    a = np.ascontiguousarray(a if layout == "aos" else a.T, dtype=np.int32)
    return torch.from_numpy(a).cuda()


def from_dev(t, layout):
    a = t.cpu().numpy()
    return a if layout == "aos" else np.ascontiguousarray(a.T)


def limbs_dev(values, limbs):
    return torch.from_numpy(G.ints_to_limbs(values, limbs)).cuda()


def oracle_eval_device(ctx, orc, x):
    """the oracle's reference GPU evaluation with the device's ceil(log2) (CUDA's
    log2 is not exact at every power of two; the reference GPU code calls it)"""
    xs = orc.log2_inputs(x)
    cs = ctx.device_ceil_log2(xs) if len(xs) else np.zeros(0, np.int32)
    return orc.eval_with_device_log2(x, xs, cs)


def edge_values(orc, rng, count):
    M = orc.M
    vals = [rng.randrange(M) for _ in range(count)]
    vals += [rng.randrange(1 << b) for b in range(1, M.bit_length())]
    vals += list(range(0, 33)) + [M - k for k in range(1, 33)] + [M // 2 - 1, M // 2, M // 2 + 1]
    return vals


@pytest.mark.parametrize("layout", ["soa", "aos"])
def test_to_binary(case, layout):
    tag, ctx, orc, g = case
    LM = ctx.binary_limbs
    assert LM == (orc.M.bit_length() + 31) // 32
    got = ctx.rns_to_binary(to_dev(g["x"], layout), layout=layout).cpu().numpy()
    assert got.view(np.uint32).tobytes() == g["tobin_words"].tobytes()
    vals = edge_values(orc, random.Random(5), sized(orc.n, 3000, 1000))
    x = orc.exact.to_rns(vals)
    flags = torch.zeros(len(vals), dtype=torch.uint8, device="cuda")
    wide = ctx.rns_to_binary(to_dev(x, layout), layout=layout, limbs=LM + 3, flags=flags).cpu().numpy()
    assert G.limbs_to_ints(wide) == vals
    assert not wide[:, LM:].any() and int(flags.sum()) == 0


@pytest.mark.parametrize("layout", ["soa", "aos"])
def test_from_binary(case, layout):
    tag, ctx, orc, g = case
    got = from_dev(ctx.rns_from_binary(torch.from_numpy(g["frombin_words"].view(np.int32)).cuda(), layout=layout),
                   layout)
    assert np.array_equal(got, g["frombin_rns"])
    rng = random.Random(6)
    for limbs in (1, 2, ctx.binary_limbs, 128, 256):
        vals = [rng.randrange(1 << (32 * limbs)) for _ in range(700)] + [0, (1 << (32 * limbs)) - 1]
        got = from_dev(ctx.rns_from_binary(limbs_dev(vals, limbs), layout=layout), layout)
        assert np.array_equal(got, orc.exact.to_rns([v % orc.M for v in vals])), limbs


def test_round_trip_and_partial_tiles(case):
    """counts that leave partial 128-number tiles and several tiles per block"""
    tag, ctx, orc, g = case
    rng = random.Random(7)
    for count in (1, 127, 129, 5000):
        vals = [rng.randrange(orc.M) for _ in range(count)]
        x = ctx.rns_from_binary(limbs_dev(vals, ctx.binary_limbs))
        assert G.limbs_to_ints(ctx.rns_to_binary(x).cpu().numpy()) == vals


@pytest.mark.parametrize("n", [128, 256])
def test_round_trip_large_moduli(dev, n):
    """n greedy 30-bit moduli: each CRT chunk sums n products of up to 56.4
    bits, past 2^64 for n = 256 (the 128-bit sums); values of every size up
    to M - 1, and 256-limb inputs reduced mod M"""
    from oracle.oracle import greedy_moduli
    mods = greedy_moduli(n)
    ctx = G.RNSContext(mods)
    M = 1
    for m in mods:
        M *= m
    rng = random.Random(n)
    vals = [rng.randrange(M) for _ in range(300)] + [M - 1, M - 2, 0, 1] + [rng.randrange(1 << b) for b in (1, 64, 3000)]
    x = ctx.rns_from_binary(limbs_dev(vals, ctx.binary_limbs))
    assert G.limbs_to_ints(ctx.rns_to_binary(x).cpu().numpy()) == vals
    wide = [rng.randrange(1 << (32 * 256)) for _ in range(200)] + [(1 << (32 * 256)) - 1]
    y = ctx.rns_from_binary(limbs_dev(wide, 256))
    assert G.limbs_to_ints(ctx.rns_to_binary(y).cpu().numpy()) == [v % M for v in wide]


def test_invalid_residue_flagged(case):
    tag, ctx, orc, g = case
    v = 12345 if orc.M > 12345 else orc.M - 3
    x = orc.exact.to_rns([v, 678 % orc.M])
    x[1, 0] = orc.moduli[0]
    flags = torch.zeros(2, dtype=torch.uint8, device="cuda")
    got = ctx.rns_to_binary(to_dev(x, "aos"), layout="aos", flags=flags).cpu().numpy()
    assert list(flags.cpu().numpy()) == [0, 1]
    assert G.limbs_to_ints(got) == [v, 0]
    with pytest.raises(RuntimeError):
        ctx.rns_to_binary(to_dev(x, "aos"), layout="aos", limbs=ctx.binary_limbs - 1)


def test_mpint_binary(case):
    """mpint_set_mpz / mpint_get_mpz: digits and sign as the reference, the
    evaluation as the device evaluation of the digits"""
    tag, ctx, orc, g = case
    dt = mpint_dtype(orc.n)
    m = torch.from_numpy(g["mpdiv_a"]).cuda()
    words, signs = ctx.mpint_get_binary(m)
    assert words.cpu().numpy().view(np.uint32).tobytes() == g["mpint_tobin_words"].tobytes()
    assert np.array_equal(signs.cpu().numpy(), g["mpint_tobin_signs"])
    rng = random.Random(8)
    vals = [rng.choice((-1, 1)) * v for v in edge_values(orc, rng, sized(orc.n, 800, 300))]
    mags = [abs(v) for v in vals]
    sg = torch.tensor([1 if v < 0 else 0 for v in vals], dtype=torch.int32, device="cuda")
    rec = ctx.mpint_set_binary(limbs_dev(mags, ctx.binary_limbs), sg).cpu().numpy().view(dt)
    want = orc.mpint_from_ints(vals)
    assert rec["digits"].tobytes() == want["digits"].tobytes()
    assert np.array_equal(rec["sign"], want["sign"])
    ev = oracle_eval_device(ctx, orc, rec["digits"])
    assert rec["eval"].tobytes() == np.stack([ev["low"], ev["upp"]], axis=1).tobytes()
    w2, s2 = ctx.mpint_get_binary(torch.from_numpy(rec.view(np.uint8)).cuda())
    back = [(-v if s else v) for v, s in zip(G.limbs_to_ints(w2.cpu().numpy()), s2.cpu().numpy())]
    assert back == vals
    # no signs: all nonnegative
    rec0 = ctx.mpint_set_binary(limbs_dev(mags[:50], ctx.binary_limbs)).cpu().numpy().view(dt)
    assert not rec0["sign"].any()
