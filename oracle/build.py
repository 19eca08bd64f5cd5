"""Build recipe for the oracle shared library (test infrastructure only).

Compiles ``aenet_oracle.c`` with gcc into ``oracle/_build/liboracle.so``.
``-ffp-contract=off`` keeps every multiply and add separately rounded, which
is the arithmetic the neighbour predicate is defined on; ``-fopenmp`` lets
the CPU baseline split the atom loop over host threads.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "aenet_oracle.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")


def build(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", "-fvisibility=hidden", "-Wall",
           "-Wno-unused-function", SRC, "-o", tmp, "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
