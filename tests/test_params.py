"""CPU: moduli sets in the reference's params.h format (src/params.h:11-39 and
the src/params/ catalogue) through grns_params_parse."""
import pytest

import grns_gb300 as G
from grns_gb300 import build
from tests.helpers import TAGS, moduli_for


@pytest.fixture(scope="module", autouse=True)
def lib():
    build.build()


def params_text(moduli, log2=None, threshold=30, error="0.0000001", per_line=8):
    """a params file in the reference's layout: guard, defines, continuation lines"""
    M = 1
    for m in moduli:
        M *= m
    rows = [",".join(str(m) for m in moduli[k:k + per_line]) for k in range(0, len(moduli), per_line)]
    vals = ", \\\n                          ".join(rows)
    return f"""/*
 *  The set of RNS moduli and other parameters
 */
#ifndef GRNS_PARAMS_H
#define GRNS_PARAMS_H

#define RNS_MODULI_SIZE ({len(moduli)})

#define RNS_MODULI_PRODUCT_LOG2 ({M.bit_length() - 1 if log2 is None else log2})  // floor(log2 M)

#define RNS_P2_SCALING_THRESHOLD ({threshold})

#define RNS_EVAL_RELATIVE_ERROR ({error})

#define RNS_MODULI_VALUES {{{vals}}}

constexpr int RNS_MODULI[RNS_MODULI_SIZE] = RNS_MODULI_VALUES;

#define EMPLOY_STD_FMA false

#endif  //GRNS_PARAMS_H
"""


@pytest.mark.parametrize("tag", TAGS)
def test_parse_round_trip(tag):
    mods = moduli_for(tag)
    M = 1
    for m in mods:
        M *= m
    got, lg = G.parse_params(params_text(mods))
    assert got == mods and lg == M.bit_length() - 1


def test_parse_without_optional_defines():
    text = "#define RNS_MODULI_SIZE 4\n#define RNS_MODULI_VALUES { 3, 5, 7, 11 }\n"
    assert G.parse_params(text) == ([3, 5, 7, 11], None)


@pytest.mark.parametrize("bad,status", [
    ("#define RNS_MODULI_SIZE (4)\n#define RNS_MODULI_VALUES {3,5,7}\n", 1),        # count differs
    ("#define RNS_MODULI_VALUES {3,5,7,11}\n", 1),                                     # no size
    ("#define RNS_MODULI_SIZE (4)\n#define RNS_MODULI_VALUES {3,5,x,11}\n", 1),        # not a number
    (params_text([3, 5, 7, 11], threshold=31), 2),                                     # other scaling step
    (params_text([3, 5, 7, 11], error="0.000001"), 2),                                 # other error bound
    (params_text([3, 5, 7, 11], error=" "), 2),                                        # empty error bound
    ("#define RNS_MODULI_SIZE 2\n#define RNS_MODULI_VALUES {3,5}\n#define RNS_EVAL_RELATIVE_ERROR  (\n", 2),
    ("#define RNS_MODULI_SIZE (4)\n#define RNS_MODULI_VALUES {3,5,7," + "9" * 40 + "}\n", 1),  # overlong
    ("#define RNS_MODULI_SIZE (" + "9" * 25 + ")\n#define RNS_MODULI_VALUES {3}\n", 1),  # overlong size
    (params_text([3, 5, 7, 11], log2=1 << 30), 1),                                     # absurd log2
])
def test_parse_rejects(bad, status):
    with pytest.raises(G.GrnsError) as e:
        G.parse_params(bad)
    assert e.value.status == status


def test_commented_out_definitions_are_ignored():
    text = params_text([3, 5, 7, 11]) + "/* #define RNS_MODULI_SIZE (8) */\n// #define RNS_MODULI_VALUES {1}\n"
    assert G.parse_params(text)[0] == [3, 5, 7, 11]


def test_mutated_files_parse_or_fail_cleanly():
    """byte mutations and truncations of a valid file: the parser returns the
    original set or an error status, never anything else"""
    import random
    mods = moduli_for("g12")
    text = params_text(mods)
    rng = random.Random(11)
    alphabet = "0123456789(){},;/*\\\n #defineRNS_MODULI_SIZEVALUES.-x\t"
    outcomes = set()
    for trial in range(3000):
        t = list(text)
        for _ in range(rng.randint(1, 6)):
            k = rng.randrange(len(t))
            op = rng.random()
            if op < 0.4:
                t[k] = rng.choice(alphabet)
            elif op < 0.7:
                del t[k]
            else:
                t.insert(k, rng.choice(alphabet))
        if trial % 7 == 0:
            t = t[:rng.randrange(len(t))]
        try:
            got, lg = G.parse_params("".join(t))
        except G.GrnsError as e:
            assert e.status in (1, 2)
            outcomes.add(e.status)
            continue
        assert len(got) >= 0 and all(1 <= v <= 0x7FFFFFFF for v in got)
        outcomes.add(0)
    assert outcomes >= {0, 1}
