"""Shared test helpers: golden fixtures and moduli sets."""
import os

import numpy as np

from oracle.oracle import REFERENCE_DEFAULT_MODULI, greedy_moduli

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
# moduli sets: the reference's shipped default (ref8), greedy 30-bit sets (gN),
# three sets of the reference's params catalogue (pN: moduli 3..59, 17-bit,
# 26-bit) and the catalogue's other files (catFAMILY_nK =
# src/params/moduli-*-FAMILY-bit/params.Km.*.h; BIG_TAGS: 128 and 256 moduli)
BASE_TAGS = ["ref8", "g8", "g12", "g32", "g64", "p16", "p32", "p64"]
CATALOGUE_TAGS = ["cat69_n%d" % n for n in range(4, 16)] + ["cat4096_n%d" % n for n in (4, 8, 16, 64)] + \
    ["cat6400_n%d" % n for n in (4, 8, 16, 32)]
BIG_TAGS = ["cat4096_n128", "cat6400_n128", "cat4096_n256", "cat6400_n256"]
CATALOGUE_TAGS += BIG_TAGS
TAGS = BASE_TAGS + CATALOGUE_TAGS

ER_DTYPE = np.dtype([("frac", "<f8"), ("exp", "<i8")])
IV_DTYPE = np.dtype([("low", ER_DTYPE), ("upp", ER_DTYPE)])


def moduli_for(tag):
    if tag == "ref8":
        return list(REFERENCE_DEFAULT_MODULI)
    if tag.startswith(("p", "cat")):  # recorded in the fixture by tests/golden/make_golden.py
        return [int(m) for m in np.load(os.path.join(GOLDEN, f"golden_{tag}.npz"))["moduli"]]
    return greedy_moduli(int(tag[1:]))


def golden(tag):
    return dict(np.load(os.path.join(GOLDEN, f"golden_{tag}.npz")))


def thin_golden(g, n, keep=12):
    """For 128 and 256 moduli, every k-th entry of each per-number array (the
    rows stay aligned: arrays of one length are thinned alike; byte arrays of
    intervals and mp_int records by record), so that the CPU suite stays
    short: the reference's one-bit division runs ~log2 M steps per pair.
    Smaller sets are returned whole."""
    if n < 128:
        return g
    out = {}
    for k, v in g.items():
        rec = None
        if v.dtype == np.uint8 and v.ndim == 1:
            rec = 32 if k.startswith("eval") else mpint_dtype(n).itemsize
            v = v.reshape(-1, rec)
        if k not in ("moduli", "mpint_kat") and v.ndim and len(v) > keep:
            v = v[::-(-len(v) // keep)]
        out[k] = v.reshape(-1) if rec else v
    return out


def sized(n, small, large):
    """random-input counts of a test: `small` up to 16 moduli, `large` up to
    64, a quarter of `large` (at least 8) for 128 and 256 moduli, whose
    oracle checks on the CPU cost ~log2 M steps per number"""
    return small if n <= 16 else large if n <= 64 else max(8, large // 4)


def mpint_dtype(n):
    off = ((4 * n + 4 + 7) // 8) * 8
    return np.dtype({"names": ["digits", "sign", "eval"], "formats": [("<i4", (n,)), "<i4", (ER_DTYPE, (2,))],
                     "offsets": [0, 4 * n, off], "itemsize": off + 32})


def product_safe_bits(log2M):
    """bit length of mp_int operands whose products stay below M (the
    catalogue's smallest sets have M of 10 to 36 bits)"""
    return log2M // 2 - 10 if log2M >= 40 else max(1, log2M // 2 - 1)
