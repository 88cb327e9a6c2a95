"""The GPU LowRankCholeskySampler (cholesky_sampler.cc:41-129) against the
oracle's restatement (dense natural-order factor of A_0, Householder QR of
L^{-1} B): with the same injected normals the samples agree to 1e-12 (the
Cholesky factor and the sign-normalised thin QR are unique, so the two
differ by rounding only), and Philox samples have the exact mean and
covariance within Monte Carlo error."""
import numpy as np
import pytest

import multigridmc_gb300 as M
import oracle as O
from problems import operator_1d, posterior

pytestmark = pytest.mark.gpu

CASES = [
    ("1d", lambda: operator_1d(False)),
    ("1d-lowrank", lambda: operator_1d(True)),
    ("2d-prior-16", lambda: posterior((16, 16))),
    ("2d-post-16", lambda: posterior((16, 16), m=3, radius=0.1)),
    ("3d-post-8", lambda: posterior((8, 8, 8), m=4, radius=0.15)),
    ("3d-post-16", lambda: posterior((16, 16, 16), m=8, radius=0.1)),
]


@pytest.mark.parametrize("name,mk", CASES, ids=[c[0] for c in CASES])
def test_lowrank_cholesky_equals_oracle(name, mk):
    op_o, op = mk()
    nsamples = 20
    noise = O.CLCG().draw_normal(op.n * nsamples)
    orc = O.lowrank_cholesky_sampler(op_o, O.Source(noise))
    gpu = M.LowRankCholeskySampler(op, noise=M.INJECTED)
    gpu.inject_noise(noise)
    f = np.random.default_rng(3).standard_normal(op.n)
    if op.m:
        f += op.B_dense() @ (np.linspace(-1.0, 1.0, op.m) / op.Sigma)
    worst = 0.0
    xo, xg = np.zeros(op.n), np.zeros(op.n)
    for k in range(nsamples):
        orc.apply(f, xo)
        gpu.apply(f, xg)
        worst = max(worst, np.linalg.norm(xg - xo) / np.linalg.norm(xo))
    assert worst < 1e-12, f"{name}: {worst:.3e}"
    gpu.close()


def test_lowrank_cholesky_fixed_rhs():
    """fix_rhs(f) then apply(None, x) draws what apply(f, x) draws."""
    _, op = posterior((16, 16), m=3, radius=0.1)
    f = np.random.default_rng(5).standard_normal(op.n)
    a = M.LowRankCholeskySampler(op, seed=9)
    b = M.LowRankCholeskySampler(op, seed=9)
    a.fix_rhs(f)
    xa, xb = np.zeros(op.n), np.zeros(op.n)
    for _ in range(3):
        a.apply(None, xa)
        b.apply(f, xb)
    assert np.array_equal(xa, xb)


@pytest.mark.parametrize("shape,m", [((16, 16), 3), ((8, 8, 8), 4)])
def test_lowrank_cholesky_moments(shape, m):
    """Philox samples: mean and covariance against Q^{-1} f and Q^{-1}
    (4e4 independent samples; z-scores of the mean and of the variances)."""
    op_o, op = posterior(shape, m=m, radius=0.15, variance=1e-2)
    Q = op_o.precision()
    C = np.linalg.inv(Q)
    mu = np.random.default_rng(1342517).uniform(0.0, 1.0, op.n)
    s = M.LowRankCholeskySampler(op, seed=21)
    s.fix_rhs(Q @ mu)
    N = 40000
    X = np.zeros((N, op.n))
    x = np.zeros(op.n)
    for k in range(N):
        s.apply(None, x)
        X[k] = x
    d = np.diag(C)
    zm = (X.mean(0) - mu) / np.sqrt(d / N)
    zv = (X.var(0) - d) / (d * np.sqrt(2.0 / N))
    assert np.abs(zm).max() < 5.0 and np.sqrt(np.mean(zm ** 2)) < 1.3, zm
    assert np.abs(zv).max() < 5.0 and np.sqrt(np.mean(zv ** 2)) < 1.3, zv
    Ch = np.cov(X.T, bias=True)
    expected = np.sqrt(np.sum(C ** 2 + np.outer(d, d)) / N) / np.linalg.norm(C)
    assert np.linalg.norm(Ch - C) / np.linalg.norm(C) < 1.3 * expected
    s.close()


def test_lowrank_cholesky_refuses_variable_stencil():
    op = M.LinearOperator.shifted_laplace_fd_periodic((8, 8), 0.12, 0.23)
    with pytest.raises(M.MGMCError) as e:
        M.LowRankCholeskySampler(op)
    assert e.value.status == 8
