"""Build recipe for the oracle (test infrastructure only).

Compiles oracle/drot_oracle.c into oracle/liboracle_drot.so with gcc.  FP
contraction is off so that the host parameter arithmetic rounds the same on
x86-64 and aarch64; the element operations that the reference kernels fuse
are written as explicit fmaf()/fma() calls instead.

Usage: python oracle/build_oracle.py
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "drot_oracle.c")
IMPL = os.path.join(HERE, "drot_oracle_impl.h")
OUT = os.path.join(HERE, "liboracle_drot.so")


def build(force=False, verbose=False):
    """Compile the oracle shared library if it is missing or stale; return its path."""
    newest = max(os.path.getmtime(SRC), os.path.getmtime(IMPL))
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= newest:
        return OUT
    cmd = ["gcc", "-O2", "-std=c99", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", "-o", OUT + ".tmp", SRC, "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
