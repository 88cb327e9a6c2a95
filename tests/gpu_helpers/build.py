"""Builds the GPU test helpers (test infrastructure, not part of the library)."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")


def build(name="philox_check"):
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(HERE, name + ".cu")
    lib = os.path.join(OUT, "lib" + name + ".so")
    deps = [src, os.path.join(HERE, "..", "..", "multigridmc_gb300", "csrc", "kernels.cuh")]
    if os.path.exists(lib) and all(os.path.getmtime(lib) >= os.path.getmtime(d) for d in deps):
        return lib
    nvcc = "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc"
    subprocess.check_call([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-shared",
                           "-Xcompiler", "-fPIC", "-o", lib + ".tmp", src])
    os.replace(lib + ".tmp", lib)
    return lib


if __name__ == "__main__":
    print(build())
