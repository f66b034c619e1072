"""CPU: the source-level drop-in header (include/grns/device.cuh) compiles for
sm_103a inside a user translation unit that calls every per-number function
and n-threaded form (tests/native/device_drop_in.cu), for moduli sets given
the reference's params.h way.  No GPU: compile only; the GPU tests run it."""
import os
import shutil
import subprocess

import pytest

from tests.helpers import moduli_for

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("tag", ["ref8", "g32", "cat6400_n256"])
def test_drop_in_compiles(tmp_path, tag):
    from grns_gb300.build import nvcc
    exe = nvcc()
    if not exe or not (os.path.exists(exe) or shutil.which(exe)):
        pytest.skip("nvcc not found")
    mods = moduli_for(tag)
    params = tmp_path / "params.h"
    params.write_text(f"#define RNS_MODULI_SIZE ({len(mods)})\n"
                      f"#define RNS_MODULI_VALUES {{{','.join(str(m) for m in mods)}}}\n")
    out = tmp_path / "drop_in.o"
    r = subprocess.run([exe, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17",
                        "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
                        "-include", str(params), "-c", os.path.join(ROOT, "tests", "native", "device_drop_in.cu"),
                        "-o", str(out)], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    assert out.stat().st_size > 0
