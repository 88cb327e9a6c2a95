"""The no-allocation entry point mgmc_measured_apply_noalloc.

Callers that cannot allocate device memory (work captured into a CUDA graph,
applications that lend the library buffers from their own memory pool) get
y = A x for the measured operator with every buffer passed in and the B^T x
scratch in the library's static device array.  Its output must match the
oracle's LinearOperator::apply and the allocating path (mgmc_level_apply on
level 0 of a sampler) on two calls in a row -- the second call reuses the
scratch the first one left behind -- and a call captured into a CUDA graph
in global capture mode, where allocation is not allowed, must give the same
result when the graph is replayed.

This file is collected last so that a stop-at-first-failure run has already
run every other test; it also passes alone in a fresh process (the first
call on the device does the one-time set-up).
"""
import numpy as np
import pytest

import multigridmc_gb300 as M
from problems import operator_1d, posterior

pytestmark = pytest.mark.gpu

TOL = 1e-12

CASES = [
    ("3d-m12", lambda: posterior((32, 32, 32), m=12, radius=0.1)),
    ("3d-m0", lambda: posterior((16, 16, 16))),
    ("2d-m4", lambda: posterior((32, 32), m=4, radius=0.1)),
    ("1d-lowrank", lambda: operator_1d(True)),
]


def _device_operator(op):
    import torch
    dev = torch.device("cuda", 0)
    return dict(ptr=torch.tensor(op.B_ptr, dtype=torch.int64, device=dev),
                idx=torch.tensor(op.B_idx, dtype=torch.int64, device=dev),
                val=torch.tensor(op.B_val, dtype=torch.float64, device=dev),
                sig=torch.tensor(op.Sigma, dtype=torch.float64, device=dev))


def _call(op, d, x, y, stream):
    M.measured_apply_noalloc(op, d["ptr"].data_ptr(), d["idx"].data_ptr(), d["val"].data_ptr(),
                             d["sig"].data_ptr(), x.data_ptr(), y.data_ptr(), stream)


@pytest.mark.parametrize("name,mk", CASES, ids=[c[0] for c in CASES])
def test_noalloc_apply_matches_oracle_and_level_apply(name, mk):
    import torch
    op_o, op = mk()
    ref = M.MultigridMCSampler(op, M.MultigridParameters(nlevel=2), precision=M.FP64)
    d = _device_operator(op)
    y = torch.empty(op.n, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    rng = np.random.default_rng(17)
    for call in range(2):
        x_host = rng.standard_normal(op.n) * (1.0 + call)
        x = torch.tensor(x_host, dtype=torch.float64, device="cuda")
        _call(op, d, x, y, stream.cuda_stream)
        stream.synchronize()
        got = y.cpu().numpy()
        want_o = op_o.apply(x_host)
        want_l = ref.level_apply(0, x_host)
        assert np.linalg.norm(got - want_o) <= TOL * np.linalg.norm(want_o), f"{name} call {call}: vs oracle"
        assert np.linalg.norm(got - want_l) <= TOL * np.linalg.norm(want_l), f"{name} call {call}: vs level_apply"
    ref.close()


def test_noalloc_apply_inside_graph_capture():
    """One ordinary call, then a call captured into a CUDA graph on a side
    stream (torch.cuda.graph, global capture mode: any cudaMalloc inside
    would end the capture with an error); replaying the graph on two
    different inputs gives the oracle's A x both times."""
    import torch
    op_o, op = posterior((16, 16, 16), m=6, radius=0.1)
    d = _device_operator(op)
    x = torch.zeros(op.n, dtype=torch.float64, device="cuda")
    y = torch.zeros_like(x)
    _call(op, d, x, y, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    with torch.cuda.graph(g, stream=side, capture_error_mode="global"):
        _call(op, d, x, y, torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(23)
    for rep in range(2):
        x_host = rng.standard_normal(op.n)
        x.copy_(torch.from_numpy(x_host))
        y.zero_()
        g.replay()
        torch.cuda.synchronize()
        want = op_o.apply(x_host)
        assert np.linalg.norm(y.cpu().numpy() - want) <= TOL * np.linalg.norm(want), f"replay {rep}"


def test_noalloc_rejects_too_many_columns():
    import torch
    _, op = posterior((8, 8, 8))
    x = torch.zeros(op.n, dtype=torch.float64, device="cuda")
    big = M.LinearOperator(op.shape, op.stencil, np.zeros(4098, np.int64), np.zeros(0, np.int64), np.zeros(0),
                           np.ones(4097))
    with pytest.raises(M.MGMCError) as e:
        M.measured_apply_noalloc(big, x.data_ptr(), x.data_ptr(), x.data_ptr(), x.data_ptr(), x.data_ptr(),
                                 x.data_ptr(), 0)
    assert e.value.status == 1 and "4096" in str(e.value)
