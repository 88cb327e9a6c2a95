"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``oracle/mgmc_oracle.cc`` into ``oracle/_build/libmgmc_oracle.so``
with plain g++ (no Eigen, no reference build system) at -O3.
``-ffp-contract=off`` keeps the floating-point operation order of the
restatement free of FMA contraction on both x86_64 and aarch64 hosts; no
-march=native, so the library gives the same results on both.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "mgmc_oracle.cc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libmgmc_oracle.so")


def build(force=False, verbose=False):
    """Compile the oracle shared library if it is missing or stale."""
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC), os.path.getmtime(__file__))):
        return LIB
    cmd = ["g++", "-O3", "-std=c++17", "-ffp-contract=off", "-fopenmp",
           "-shared", "-fPIC", "-o", LIB + ".tmp", SRC]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
