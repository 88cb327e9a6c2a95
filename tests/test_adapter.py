"""The reference-side C++ adapter (include/mgmc_gb300_sampler.hh).

It is compiled against stand-ins of the reference's interfaces
(tests/adapter_stub/: Sampler, LinearOperator, RandomGenerator,
MultigridParameters and the Eigen types they use) and linked with
libmgmc_gb300.so.  On the GPU the program drives it the way
measure_sampling_time does (fix_rhs, then apply(f, x) per step; see
src/measurements/sampling_time.cc:28-41) and the chain must equal, bit for
bit, the same calls made through the Python binding.
"""
import os
import subprocess

import numpy as np
import pytest

import multigridmc_gb300 as M

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STUB = os.path.join(ROOT, "tests", "adapter_stub")


def _build(tmp_path):
    from multigridmc_gb300 import build as B
    lib = B.build()
    exe = str(tmp_path / "adapter_main")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"), "-I" + STUB,
           os.path.join(STUB, "adapter_main.cc"), "-L" + os.path.dirname(lib), "-lmgmc_gb300",
           "-Wl,-rpath," + os.path.dirname(lib), "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_adapter_compiles_and_links(tmp_path):
    """The adapter header compiles with -Wall -Werror against the reference's
    interfaces and links with the library (no GPU needed)."""
    assert os.path.exists(_build(tmp_path))


@pytest.mark.gpu
def test_adapter_chain_equals_binding(tmp_path):
    exe = _build(tmp_path)
    out = str(tmp_path / "adapter.bin")
    r = subprocess.run([exe, out], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    raw = np.fromfile(out, dtype=np.float64)
    shape = (16, 16, 16)
    n = 15 ** 3
    centres = [[0.3, 0.3, 0.3], [0.6, 0.4, 0.5], [0.4, 0.7, 0.6], [0.7, 0.6, 0.3]]
    cols = [M.measurement_vector(shape, c, 0.1) for c in centres]
    op = M.LinearOperator.shifted_laplace_fd(shape, 10.0).with_lowrank(cols, np.full(4, 1e-4))
    y = np.array([1.0, -0.5, 0.25, 2.0])
    f = op.B_dense() @ (y / op.Sigma)
    prm = M.MultigridParameters(nlevel=3)

    def sampler(u):
        return M.MultigridMCSampler(op, prm, ordering=M.MULTICOLOUR, precision=M.FP64, noise=M.PHILOX,
                                    seed=int(u * 9007199254740992.0))

    s = sampler(0.25)
    x = np.zeros(n)
    s.fix_rhs(f)
    for _ in range(5):
        s.apply(None, x)
    assert np.array_equal(raw[:n], x), "fix_rhs + apply"
    s.apply(f, x)
    assert np.array_equal(raw[n:2 * n], x), "apply after unfix_rhs"
    s.fix_rhs(f)
    s.set_observable(cols[0][0], cols[0][1], 8)
    s.step(3)
    z = s.read_observations(8)
    k = int(raw[2 * n])
    assert k == 3 and np.array_equal(raw[2 * n + 1:2 * n + 1 + k], z), "device-resident observable loop"
    c = sampler(0.5)
    x2 = np.zeros(n)
    c.fix_rhs(f)
    c.apply(None, x2)
    assert np.array_equal(raw[2 * n + 1 + k:], x2), "deep_copy"
    s.close()
    c.close()
