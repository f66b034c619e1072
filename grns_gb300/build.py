"""Build libgrns_gb300.so in-tree with nvcc for sm_103a.

Each translation unit compiles in parallel to an object file under
grns_gb300/_build/, then nvcc links the shared library.  A source that names
GRNS_SPLIT_BY_N in its header comment compiles as GRNS_N_PARTS units, one per
group of moduli counts (-DGRNS_PART=k; the groups are in csrc/internal.h).  Nothing is
installed; the library is loaded from grns_gb300/_build/ by grns_gb300.native.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libgrns_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include")]


def nvcc():
    for p in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if p and (os.path.sep not in p or os.path.exists(p)):
            return p
    return "nvcc"


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    inc = os.path.join(ROOT, "include", "grns")
    hs += [os.path.join(inc, f) for f in os.listdir(inc)]
    return hs


N_PARTS = 4  # GRNS_N_PARTS in csrc/internal.h


def units():
    """(source, part) for every translation unit; part None = the whole file"""
    out = []
    for src in sources():
        with open(src) as f:
            head = f.read(2048)
        if "GRNS_SPLIT_BY_N" in head:
            out += [(src, k) for k in range(N_PARTS)]
        else:
            out.append((src, None))
    # the longest units first, so that they do not start last
    return sorted(out, key=lambda u: -os.path.getsize(u[0]))


def _compile(unit, extra):
    src, part = unit
    tag = "" if part is None else f".p{part}"
    obj = os.path.join(OUT, os.path.basename(src) + tag + ".o")
    extra = list(extra) + ([] if part is None else [f"-DGRNS_PART={part}"])
    newest = max([os.path.getmtime(src)] + [os.path.getmtime(h) for h in headers()])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest:
        return obj
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + extra + ["-c", src, "-o", obj + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stderr[-6000:]}")
    os.replace(obj + ".tmp", obj)
    return obj


def build(verbose=False, extra=()):
    os.makedirs(OUT, exist_ok=True)
    us = units()
    with ThreadPoolExecutor(max(1, min(len(us), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(lambda u: _compile(u, list(extra)), us))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr[-4000:])
        os.replace(LIB + ".tmp", LIB)
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
