"""Exact sampler x = Q^{-1}(f + eta), eta ~ N(0, Q): the comparator role of
the reference's SparseCholeskySampler (src/sampler/cholesky_sampler.cc:9-23)
at sizes a factorisation does not reach.  Mean and covariance against the
exact ones (the reference's Cholesky sampler tests, test_sampler.hh:165-209,
restated with Monte Carlo tolerances), reproducibility, and the stencil
condition of the perturbation."""
import numpy as np
import pytest

import multigridmc_gb300 as M
from problems import operator_1d, posterior

pytestmark = pytest.mark.gpu


def _moments(op, f, nlevel, nsamples, precision, seed=3):
    s = M.MultigridMCSampler(op, M.MultigridParameters(nlevel=nlevel), precision=precision, seed=seed)
    X = np.empty((nsamples, op.n))
    for i in range(nsamples):
        X[i], _ = s.exact_sample(f, rtol=1e-11)
    s.close()
    return X


@pytest.mark.parametrize("name,mk,nlevel", [
    ("1d-testop-lowrank", lambda: operator_1d(True)[1], 2),
    ("2d-post-8", lambda: posterior((8, 8), m=2, radius=0.2, variance=1e-2)[1], 2),
    ("3d-post-4", lambda: posterior((4, 4, 4), m=1, radius=0.3, variance=1e-2)[1], 1),
])
@pytest.mark.parametrize("precision", [M.FP64, M.FP32_MIXED], ids=["fp64", "fp32-mixed"])
def test_exact_sampler_moments(name, mk, nlevel, precision):
    """Sample mean and covariance of 4000 draws against Q^{-1} f and Q^{-1}
    within 4.5 Monte Carlo standard errors (Frobenius norms; draws are
    independent)."""
    op = mk()
    Q = op.to_scipy().toarray()
    C = np.linalg.inv(Q)
    f = np.random.default_rng(1).standard_normal(op.n)
    mu = C @ f
    N = 4000
    X = _moments(op, f, nlevel, N, precision)
    se_mean = np.sqrt(np.trace(C) / N)
    assert np.linalg.norm(X.mean(0) - mu) <= 4.5 * se_mean
    Cs = np.cov(X.T)
    se_cov = np.sqrt(np.sum(C ** 2 + np.outer(np.diag(C), np.diag(C))) / N)
    assert np.linalg.norm(Cs - C) <= 4.5 * se_cov


def test_exact_sampler_reproducible_and_independent():
    """The same seed reproduces the draws; consecutive draws differ; the
    chain's state is untouched."""
    _, op = posterior((16, 16, 16), m=4)
    f = np.zeros(op.n)
    a = M.MultigridMCSampler(op, M.MultigridParameters(nlevel=3), seed=9)
    b = M.MultigridMCSampler(op, M.MultigridParameters(nlevel=3), seed=9)
    x0 = np.random.default_rng(2).standard_normal(op.n)
    a.set_state(x0)
    xa1, _ = a.exact_sample(f)
    xa2, _ = a.exact_sample(f)
    xb1, _ = b.exact_sample(f)
    assert np.array_equal(xa1, xb1)
    assert np.linalg.norm(xa1 - xa2) > 0.1 * np.linalg.norm(xa1)
    assert np.allclose(a.get_state(), x0, rtol=0, atol=0)
    a.close()
    b.close()


def test_exact_sampler_needs_an_m_matrix_stencil():
    """A stencil with a positive off-diagonal weight has no edge
    decomposition: MGMC_ERR_UNSUPPORTED."""
    st = np.zeros(27)
    st[12], st[13], st[14] = 0.5, 4.0, 0.5
    op = M.LinearOperator((8,), st)
    s = M.MultigridMCSampler(op, M.MultigridParameters(nlevel=1))
    with pytest.raises(M.MGMCError) as e:
        s.exact_sample(np.zeros(op.n))
    assert e.value.name == "MGMC_ERR_UNSUPPORTED"
    s.close()
