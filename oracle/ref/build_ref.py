"""Build recipe for oracle/_ref: the UNMODIFIED reference library
(kisupov/grns, src/*.cuh) compiled for the CPU as a checker.

The reference is header-only CUDA C++.  Its host path compiles with g++ as
is; its device path (`namespace cuda`) compiles with g++ through the host
emulation in oracle/ref/shim/cuda_host_shim.h.  GMP/MPFR come from the
system's libgmp.so.10 / libmpfr.so.6 through the prototype shims in
oracle/ref/shim/ (the system has no GMP/MPFR headers).

One shared library per moduli set.  A params header generated into
oracle/_ref/ is pre-included ahead of the reference's src/params.h, whose
include guard (GRNS_PARAMS_H) then skips the shipped default set; the tag
"ref8" keeps the shipped default set instead.

Reads the reference sources where they lie -- the checkout named by the
`ref` argument of build() or by $GRNS_REFERENCE (no default) -- and writes
only into oracle/_ref/.  When no checkout is named, or its sources or the
GMP/MPFR runtime libraries are absent, it builds nothing and says so.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from math import gcd

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
REF = os.environ.get("GRNS_REFERENCE")  # the reference checkout (build(ref=...) overrides)


def greedy_moduli(n, start=2 ** 30 - 1):
    """Pairwise-coprime odd integers taken greedily downward from `start`."""
    out, c = [], start
    while len(out) < n:
        if c % 2 == 1 and all(gcd(c, m) == 1 for m in out):
            out.append(c)
        c -= 1
    return out


def floor_log2_product(moduli):
    M = 1
    for m in moduli:
        M *= m
    return M.bit_length() - 1


# tag -> moduli (None = the reference's shipped src/params.h; a string = a
# params file of the reference's catalogue, pre-included as it is).  BASE is
# what build() compiles by default; make_golden.py also builds CATALOGUE.
BASE = {
    "ref8": None,
    "g8": greedy_moduli(8),
    "g12": greedy_moduli(12),
    "g32": greedy_moduli(32),
    "g64": greedy_moduli(64),
    "p16": "src/params/moduli-10-69-bit/params.16m.69b.h",    # moduli 3..59
    "p32": "src/params/moduli-64-4096-bit/params.32m.512b.h",  # 17-bit moduli
    "p64": "src/params/moduli-100-6400-bit/params.64m.1600b.h",  # 26-bit moduli
}

# the rest of the catalogue: catNN_nK = params.Km.*.h of the
# family moduli-*-NN-bit (p16 / p32 / p64 above are cat69_n16 / cat4096_n32 /
# cat6400_n64)
_FAMILIES = {
    "69": ("moduli-10-69-bit", {4: 10, 5: 13, 6: 17, 7: 22, 8: 26, 9: 31, 10: 36, 11: 41, 12: 47, 13: 52, 14: 58,
                                15: 63}),
    "4096": ("moduli-64-4096-bit", {4: 64, 8: 128, 16: 256, 64: 1024, 128: 2048, 256: 4096}),
    "6400": ("moduli-100-6400-bit", {4: 100, 8: 200, 16: 400, 32: 800, 128: 3200, 256: 6400}),
}
CATALOGUE = {f"cat{fam}_n{n}": f"src/params/{d}/params.{n}m.{b}b.h"
             for fam, (d, sizes) in _FAMILIES.items() for n, b in sizes.items()}
SETS = {**BASE, **CATALOGUE}


def catalogue_moduli(relpath):
    """RNS_MODULI_VALUES of a params file of the reference's catalogue"""
    import re
    text = open(os.path.join(REF, relpath)).read().replace("\\\n", " ")
    vals = re.search(r"#define\s+RNS_MODULI_VALUES\s*\{([^}]*)\}", text).group(1)
    return [int(v) for v in vals.split(",")]


def params_header(moduli):
    n = len(moduli)
    vals = ",".join(str(m) for m in moduli)
    return f"""/* generated by oracle/ref/build_ref.py */
#ifndef GRNS_PARAMS_H
#define GRNS_PARAMS_H
#define RNS_MODULI_SIZE ({n})
#define RNS_MODULI_PRODUCT_LOG2 ({floor_log2_product(moduli)})
#define RNS_P2_SCALING_THRESHOLD (30)
#define RNS_EVAL_RELATIVE_ERROR (0.0000001)
#define RNS_MODULI_VALUES {{{vals}}}
constexpr int RNS_MODULI[RNS_MODULI_SIZE] = RNS_MODULI_VALUES;
#define EMPLOY_STD_FMA false
#endif
"""


def find_lib(name):
    for d in ("/usr/lib/x86_64-linux-gnu", "/usr/lib/aarch64-linux-gnu", "/usr/lib64", "/usr/lib"):
        p = os.path.join(d, name)
        if os.path.exists(p):
            return p
    return None


# the sets whose n-threaded device functions run as one emulated block
# (oracle/ref/ref_block.cpp: n a multiple of 32, whole warps)
BLOCK_TAGS = ["g32", "g64", "p32", "p64"]


def build_one(tag, gmp, mpfr, block=False):
    src = os.path.join(REF, "src")
    out = os.path.join(OUT, f"libgrnsref_block_{tag}.so" if block else f"libgrnsref_{tag}.so")
    drv = os.path.join(HERE, "ref_block.cpp" if block else "ref_driver.cpp")
    cmd = ["g++", "-std=c++14", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-frounding-math",
           "-w", "-include", os.path.join(HERE, "shim", "cuda_host_shim.h")]
    if block:
        # -fno-gnu-unique: the block-wide statics of inline functions stay
        # private to each set's library (as GNU-unique symbols the loader
        # would merge the n = 32 and n = 64 sets' arrays across libraries)
        cmd += ["-DORACLE_BLOCK_EMULATION", "-pthread", "-fno-gnu-unique"]
        # the translation unit comes on standard input: pairwise.cuh with its
        # `static __shared__` written `__shared__` (the driver makes __shared__
        # a static; a doubled `static` does not compile), then the driver,
        # whose includes of the other headers read them from the checkout
        with open(os.path.join(src, "pairwise.cuh")) as f:
            pairwise = f.read().replace("static __shared__", "__shared__")
        stdin_unit = ("#undef __shared__\n#define __shared__ static\n" + pairwise +
                      "\n#undef __shared__\n#define __shared__\n#include \"" + drv + "\"\n")
    if isinstance(SETS[tag], str):
        cmd += ["-include", os.path.join(REF, SETS[tag])]
    elif SETS[tag] is not None:
        hdr = os.path.join(OUT, f"params_{tag}.h")
        with open(hdr, "w") as f:
            f.write(params_header(SETS[tag]))
        cmd += ["-include", hdr]
    cmd += ["-I", os.path.join(HERE, "shim"), "-I", src]
    cmd += (["-x", "c++", "-", "-x", "none"] if block else [drv]) + ["-o", out, mpfr, gmp]
    newest_input = max(os.path.getmtime(p) for p in [drv, os.path.abspath(__file__)] +
                       [os.path.join(HERE, "shim", f) for f in os.listdir(os.path.join(HERE, "shim"))])
    if os.path.exists(out) and os.path.getmtime(out) >= newest_input:
        return out
    subprocess.run(cmd, check=True, input=stdin_unit if block else None, text=True)
    return out


def build(tags=None, quiet=False, ref=None):
    """Compile the checker libraries from the checkout `ref` (else
    $GRNS_REFERENCE); returns {tag: path} (empty if unavailable)."""
    global REF
    if ref:
        REF = ref
    if not REF or not os.path.isdir(os.path.join(REF, "src")):
        if not quiet:
            print(f"oracle/_ref: reference sources not found at {REF}; nothing built")
        return {}
    gmp, mpfr = find_lib("libgmp.so.10"), find_lib("libmpfr.so.6")
    if not gmp or not mpfr:
        if not quiet:
            print("oracle/_ref: libgmp.so.10 / libmpfr.so.6 not found; nothing built")
        return {}
    os.makedirs(OUT, exist_ok=True)
    tags = list(tags or BASE)
    blocks = [t for t in BLOCK_TAGS if t in tags]
    with ThreadPoolExecutor(min(len(tags) + len(blocks), os.cpu_count() or 4)) as ex:
        paths = list(ex.map(lambda t: build_one(t, gmp, mpfr), tags))
        list(ex.map(lambda t: build_one(t, gmp, mpfr, block=True), blocks))
    return dict(zip(tags, paths))


if __name__ == "__main__":
    # python oracle/ref/build_ref.py [--ref CHECKOUT] [tag ...]
    argv = sys.argv[1:]
    where = None
    if argv[:1] == ["--ref"]:
        where, argv = argv[1], argv[2:]
    res = build(argv or None, ref=where)
    for k, v in res.items():
        print(k, v)
