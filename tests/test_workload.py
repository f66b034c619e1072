"""CPU: the seeded input generator shared by the benchmark, the tests and
the device generators (grns_gb300/workload.py, csrc/gen.cu)."""
import math

import numpy as np

from grns_gb300 import workload as W
from oracle.oracle import greedy_moduli


def test_generator_is_splitmix64():
    """the mixing step is splitmix64: from state 0 it gives the published
    first outputs e220a8397b1dcdaf, 6e789e6aa1b965f4, 06c45d188009454f"""
    z = np.array([0, W.GOLDEN, (2 * W.GOLDEN) % (1 << 64)], dtype=np.uint64)
    assert [int(v) for v in W._splitmix(z)] == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]


def test_residues_in_range_and_layouts_agree():
    mods = greedy_moduli(12)
    soa = W.uniform_residues(mods, 5000, seed=3, stream=W.S_X)
    aos = W.uniform_residues(mods, 5000, seed=3, stream=W.S_X, layout="aos")
    assert np.array_equal(soa.T, aos)
    assert all((soa[i] >= 0).all() and (soa[i] < m).all() for i, m in enumerate(mods))
    other = W.uniform_residues(mods, 5000, seed=3, stream=W.S_Y)
    assert not np.array_equal(soa, other)  # streams are independent


def test_divisors_shifts_and_bit_lengths():
    mods = greedy_moduli(8)
    log2M = math.prod(mods).bit_length() - 1
    res, vals = W.divisors(mods, log2M, 400, seed=9, layout="aos")
    L = W.bit_lengths(log2M, 400, seed=9)
    assert [v.bit_length() for v in vals] == [int(b) for b in L]
    assert L.min() >= 1 and L.max() <= log2M
    assert np.array_equal(res, W.to_residues(vals, mods, layout="aos"))
    D = W.shifts(1000, 900, seed=9)
    assert D.min() >= 1 and D.max() <= 900 and D.dtype == np.uint32
