"""Build recipe for the C restatement oracle (test infrastructure only).

Compiles oracle/grns_oracle.c into oracle/_build/libgrns_oracle.so with the
host compiler.  -ffp-contract=off is required: the reference host arithmetic
(Rump-style rounding in round-to-nearest) is defined without fused
multiply-add, and aarch64 gcc would otherwise contract x*y+z.
OpenMP is used when the compiler supports it (threads for the CPU baseline).
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libgrns_oracle.so")
SRCS = [os.path.join(HERE, f) for f in ("grns_oracle.c", "grns_oracle_common.h", "grns_oracle_n.h")]


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(s) for s in SRCS):
        return LIB
    base = ["gcc", "-std=gnu11", "-O3", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
            os.path.join(HERE, "grns_oracle.c"), "-o", LIB + ".tmp", "-lm"]
    try:
        subprocess.run(base[:1] + ["-fopenmp"] + base[1:], check=True, capture_output=True)
    except subprocess.CalledProcessError:
        subprocess.run(base, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
