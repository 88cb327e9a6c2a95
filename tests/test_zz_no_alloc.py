"""The no-allocation entry point mgmc_measured_apply_noalloc.

Callers that cannot allocate device memory (work captured into a CUDA graph,
applications that lend the library buffers from their own memory pool) get
y = A x for the measured operator with every buffer passed in and the B^T x
scratch in the library's static device array.  Its output must match the
allocating path (mgmc_level_apply on level 0 of a sampler) on two calls in a
row -- the second call reuses the scratch the first one left behind.

This file is collected last so that a stop-at-first-failure run has already
run every other test; it also passes alone in a fresh process (the first
call on the device does the one-time set-up).
"""
import numpy as np
import pytest

import multigridmc_gb300 as M
from problems import posterior

pytestmark = pytest.mark.gpu


def test_noalloc_apply_matches_level_apply():
    import torch
    _, op = posterior((32, 32, 32), m=12, radius=0.1)
    ref = M.MultigridMCSampler(op, M.MultigridParameters(nlevel=2), precision=M.FP64)
    dev = torch.device("cuda", 0)
    ptr = torch.tensor(op.B_ptr, dtype=torch.int64, device=dev)
    idx = torch.tensor(op.B_idx, dtype=torch.int64, device=dev)
    val = torch.tensor(op.B_val, dtype=torch.float64, device=dev)
    sig = torch.tensor(op.Sigma, dtype=torch.float64, device=dev)
    y = torch.empty(op.n, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    rng = np.random.default_rng(17)
    for call in range(2):
        x_host = rng.standard_normal(op.n) * (1.0 + call)
        x = torch.tensor(x_host, dtype=torch.float64, device=dev)
        M.measured_apply_noalloc(op, ptr.data_ptr(), idx.data_ptr(), val.data_ptr(), sig.data_ptr(), x.data_ptr(),
                                 y.data_ptr(), stream.cuda_stream)
        stream.synchronize()
        want = ref.level_apply(0, x_host)
        got = y.cpu().numpy()
        assert np.linalg.norm(got - want) <= 1e-12 * np.linalg.norm(want), f"call {call}"


def test_noalloc_rejects_too_many_columns():
    import torch
    _, op = posterior((8, 8, 8))
    dev = torch.device("cuda", 0)
    x = torch.zeros(op.n, dtype=torch.float64, device=dev)
    big = M.LinearOperator(op.shape, op.stencil, np.zeros(4098, np.int64), np.zeros(0, np.int64), np.zeros(0),
                           np.ones(4097))
    with pytest.raises(M.MGMCError) as e:
        M.measured_apply_noalloc(big, x.data_ptr(), x.data_ptr(), x.data_ptr(), x.data_ptr(), x.data_ptr(),
                                 x.data_ptr(), 0)
    assert e.value.status == 1 and "4096" in str(e.value)
