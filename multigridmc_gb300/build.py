"""In-tree build of libmgmc_gb300.so (CUDA for sm_103a + host C++).

Two translation units compiled in parallel -- ``csrc/api.cu`` with nvcc
(``-gencode arch=compute_103a,code=sm_103a``) and ``csrc/setup.cc`` with g++
-- then linked with nvcc into ``multigridmc_gb300/_build/libmgmc_gb300.so``.
No CMake, no torch extension machinery.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libmgmc_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

SOURCES = {
    "api.o": ("api.cu", ["kernels.cuh", "setup.h"]),
    "noalloc.o": ("noalloc.cu", []),
    "peaks.o": ("peaks.cu", []),
    "setup.o": ("setup.cc", ["setup.h"]),
}


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(obj, src, deps, verbose, extra_nvcc):
    out = os.path.join(OUT, obj)
    srcp = os.path.join(CSRC, src)
    depp = [srcp] + [os.path.join(CSRC, d) for d in deps] + [os.path.join(INCLUDE, "mgmc_gb300.h")]
    if not _stale(out, depp):
        return
    if src.endswith(".cu"):
        cmd = [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
               "-I" + INCLUDE, *extra_nvcc, "-c", srcp, "-o", out + ".tmp.o"]
    else:
        cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-fopenmp", "-I" + INCLUDE, "-c", srcp, "-o", out + ".tmp.o"]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.check_call(cmd)
    os.replace(out + ".tmp.o", out)


def build(verbose=False, extra_nvcc=()):
    """Compile (if stale) and return the path of libmgmc_gb300.so."""
    os.makedirs(OUT, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        futs = [ex.submit(_compile, obj, src, deps, verbose, list(extra_nvcc))
                for obj, (src, deps) in SOURCES.items()]
        for f in futs:
            f.result()
    objs = [os.path.join(OUT, o) for o in SOURCES]
    if _stale(LIB, objs):
        cmd = [_nvcc(), *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-Xcompiler", "-fopenmp", "-lgomp"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.check_call(cmd)
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    extra = [a for a in sys.argv[1:] if a.startswith("-X") or a.startswith("--")]
    print(build(verbose=True, extra_nvcc=[a for a in extra if a != "--verbose"]))
