"""Build oracle/_ref/libref_random.so from the reference's own sources.

Test infrastructure only.  The reference's random number generator
(src/auxilliary/parallel_random.cc) is the one piece of its sampling path
that compiles without Eigen, libconfig or LAPACK; this recipe compiles it
where it lies, together with oracle/ref_random_shim.cc (a C ABI of this
repository), so that tests can compare the oracle's restatement with the
reference's draws.  Outputs go to oracle/_ref/ only.  Without the reference
sources (e.g. on a machine that only has this repository) nothing is built
and the comparison tests skip.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference checkout's src/ directory: MGMC_REFERENCE_SRC, else the
# directory `reference` next to this repository
REF_SRC = os.environ.get("MGMC_REFERENCE_SRC",
                         os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference", "src"))
OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT, "libref_random.so")


def build(verbose=False):
    """Compile the reference RNG shim if the reference sources exist; return
    the library path or None."""
    aux = os.path.join(REF_SRC, "auxilliary")
    src = os.path.join(aux, "parallel_random.cc")
    if not os.path.exists(src):
        return None
    os.makedirs(OUT, exist_ok=True)
    shim = os.path.join(HERE, "ref_random_shim.cc")
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(src), os.path.getmtime(shim)):
        return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-I" + aux, shim, src, "-o", LIB + ".tmp"]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True) or "reference sources not found: nothing built", file=sys.stdout)
