"""CPU: the product's modular arithmetic (Shoup / Barrett / add / sub),
compiled for the host from the same header the kernels use, against exact
arithmetic for every supported modulus size."""
import ctypes
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def arith(tmp_path_factory):
    out = tmp_path_factory.mktemp("arith") / "libarith.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", os.path.join(HERE, "native", "arith_check.cpp"),
                    "-o", str(out)], check=True)
    L = ctypes.CDLL(str(out))
    L.check_modular.restype = ctypes.c_long
    L.check_modular.argtypes = [ctypes.c_uint32, ctypes.c_long, ctypes.c_uint64]
    return L


@pytest.mark.parametrize("m", [3, 5, 7, 255, 257, 65537, 1 << 20 | 1, 1073741823, 1073741419, 1283742851,
                               1431655765, 1431655761, 536870913, 536870911])
def test_modular_primitives(arith, m):
    assert arith.check_modular(m, 200000, m * 7919) == 0
