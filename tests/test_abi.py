"""CPU: the C-ABI library builds for sm_103a, loads, and exports every
entry point declared in include/grns/*.h; the product never reaches into the
oracle."""
import ctypes
import os
import re

import pytest

from grns_gb300 import build, native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include", "grns")
    for f in os.listdir(inc):
        if not f.endswith(".h"):  # device.cuh is the header-only namespace-cuda drop-in, not C ABI
            continue
        src = open(os.path.join(inc, f)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        names.update(re.findall(r"\b(grns_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    build.build()
    return native.lib()


def test_every_declared_symbol_is_exported(lib):
    syms = declared_symbols()
    assert len(syms) >= 15
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_bindings_cover_declarations():
    assert set(declared_symbols()) <= set(native.SIGNATURES), set(declared_symbols()) - set(native.SIGNATURES)


def test_status_strings(lib):
    assert lib.grns_status_string(0) == b"ok"
    assert b"sm_103a" in lib.grns_version()


def test_invalid_arguments_rejected_without_gpu(lib):
    out = ctypes.c_void_p()
    assert lib.grns_ctx_create(None, 8, ctypes.byref(out)) == 1
    mods = (ctypes.c_int32 * 17)(*([3] * 17))
    assert lib.grns_ctx_create(mods, 17, ctypes.byref(out)) == 2  # unsupported n
    assert lib.grns_eval(None, None, 1, 0, None, None, None) == 1


def test_product_does_not_use_oracle():
    for d, _, files in os.walk(os.path.join(ROOT, "grns_gb300")):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".cpp")):
                src = open(os.path.join(d, f)).read()
                assert "oracle" not in src.replace("oracle is", ""), os.path.join(d, f)


def test_header_is_plain_c(tmp_path, lib):
    """include/grns/grns.h compiles as C99 and a C program links against the
    library and calls it (no GPU needed for these entry points)"""
    import subprocess
    src = tmp_path / "user.c"
    src.write_text('#include <stdio.h>\n#include <string.h>\n#include "grns/grns.h"\n'
                   'int main(void) {\n'
                   '  grns_ctx *c = 0; int n = 0, lg = 0; int32_t m[8];\n'
                   '  const char *t = "#define RNS_MODULI_SIZE (4)\\n#define RNS_MODULI_VALUES {3,5,7,11}\\n";\n'
                   '  if (strcmp(grns_status_string(GRNS_OK), "ok")) return 1;\n'
                   '  if (grns_params_parse(t, m, 8, &n, &lg) != GRNS_OK || n != 4 || m[3] != 11) return 2;\n'
                   '  if (grns_ctx_create(0, 8, &c) != GRNS_ERR_INVALID_ARGUMENT) return 3;\n'
                   '  printf("%s\\n", grns_version());\n  return 0;\n}\n')
    exe = tmp_path / "user"
    cuda_inc = "/usr/local/cuda/include"
    libdir = os.path.dirname(native.lib_path())
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), "-I", cuda_inc,
                    str(src), "-o", str(exe), "-L", libdir, "-lgrns_gb300", f"-Wl,-rpath,{libdir}"], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, (out.returncode, out.stderr)
    assert "sm_103a" in out.stdout


# entry points whose first argument is a handle (context, batch, server)
_NOT_HANDLE_FIRST = {"grns_status_string", "grns_version", "grns_ctx_create", "grns_params_parse",
                     "grns_ctx_create_from_params", "grns_server_create", "grns_device_ceil_log2", "grns_gen_shifts"}
# queries that answer with a value rather than a status
_QUERIES = {"grns_ctx_n": 0, "grns_ctx_log2": 0, "grns_ctx_binary_limbs": 0, "grns_batch_chunks": -1,
            "grns_batch_grid": -1, "grns_ctx_get_eval_split": -1}


def test_null_handle_rejected_by_every_entry(lib):
    """Each entry point checks its handle before touching anything else: a
    NULL context, batch or server gives GRNS_ERR_INVALID_ARGUMENT (the
    context queries answer 0, the batch queries -1), whatever the other
    arguments."""
    from grns_gb300.native import SIGNATURES
    checked = 0
    for name, (_, args) in SIGNATURES.items():
        if name in _NOT_HANDLE_FIRST:
            continue
        vals = []
        for a in args:
            if a in (ctypes.c_int64, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_size_t):
                vals.append(1)
            elif a is ctypes.c_double:
                vals.append(0.0)
            else:
                vals.append(None)
        got = getattr(lib, name)(*vals)
        want = _QUERIES.get(name, 1)
        assert got == want, (name, got)
        checked += 1
    assert checked >= 45
    # the two entries without a handle check their pointers first
    assert lib.grns_device_ceil_log2(None, None, 1, None) == 1
    assert lib.grns_gen_shifts(1, 1, 1, None, None) == 1


def test_mirror_keeps_reference_operation_names():
    import grns_gb300 as G
    for name in ("rns_eval_compute", "rns_eval_compute_fast", "rns_cmp", "rns_div", "rns_div_fast", "rns_scale2pow",
                 "mpint_add", "mpint_sub", "mpint_mul", "mpint_div", "mrc", "rns_max", "rns_from_binary",
                 "rns_to_binary"):
        assert callable(getattr(G.RNSContext, name)), name
    assert G.RNSContext.rns_div_fast is G.RNSContext.rns_div
