"""Problem builders shared by the tests: the same operator for the oracle
(CPU restatement) and for the GB300 library."""
import numpy as np

import multigridmc_gb300 as M
import oracle as O


def operator_1d(lowrank):
    """TestOperator1d of the reference (src/sampler/test_sampler.hh:47-89):
    tridiagonal (6, -1) on Lattice1d(8), optional B = 10 (e_3, e_4),
    Sigma = diag(4.2, 9.3)."""
    st = np.zeros(27)
    st[12], st[13], st[14] = -1.0, 6.0, -1.0
    op_o = O.Operator.from_stencil([8], st)
    op_p = M.LinearOperator((8,), st)
    if lowrank:
        B = np.zeros((7, 2))
        B[3, 0] = 10.0
        B[4, 1] = 10.0
        sig = [4.2, 9.3]
        op_o.set_lowrank(B, sig)
        op_p = op_p.with_lowrank(B, sig)
    return op_o, op_p


def posterior(shape, kappa_sq=10.0, m=0, radius=0.05, variance=1e-4, seed=1, lo=0.1, hi=0.9):
    """Shifted-Laplace FD prior with m ball measurements (centres uniform in
    [lo, hi]^d, Sigma = variance * I)."""
    dim = len(shape)
    op_o = O.Operator.fd(list(shape), kappa_sq)
    op_p = M.LinearOperator.shifted_laplace_fd(shape, kappa_sq)
    if m > 0:
        rng = np.random.default_rng(seed)
        loc = rng.uniform(lo, hi, size=(m, dim))
        var = np.ones(m)
        op_o.add_measurements(loc, var, variance_scaling=variance, radius=radius)
        op_p = op_p.with_measurements(loc, var, variance_scaling=variance, radius=radius)
    return op_o, op_p


def rhs(op_p, seed=7):
    """f = B Sigma^{-1} y with y ~ N(0, 1) (posterior mean field) plus a
    random prior part so that every level sees a non-trivial residual."""
    rng = np.random.default_rng(seed)
    f = 0.1 * rng.standard_normal(op_p.n)
    if op_p.m > 0:
        y = rng.standard_normal(op_p.m)
        f += op_p.B_dense() @ (y / op_p.Sigma)
    return f


def periodic_posterior(shape, Lambda_min=0.12, Lambda_max=0.23, m=0, radius=0.05, variance=1e-4, seed=1, lo=0.1,
                       hi=0.9):
    """Shifted-Laplace FD prior with the periodic correlation length
    (correlationlength_model.hh:83-112: a per-vertex diagonal) and m ball
    measurements, for the oracle and the GB300 library."""
    dim = len(shape)
    op_p = M.LinearOperator.shifted_laplace_fd_periodic(shape, Lambda_min, Lambda_max)
    op_o = O.Operator.from_stencil(list(shape), op_p.stencil)
    op_o.set_diagonal(op_p.centre)
    if m > 0:
        rng = np.random.default_rng(seed)
        loc = rng.uniform(lo, hi, size=(m, dim))
        var = np.ones(m)
        op_o.add_measurements(loc, var, variance_scaling=variance, radius=radius)
        op_p = op_p.with_measurements(loc, var, variance_scaling=variance, radius=radius)
    return op_o, op_p


def fem_posterior(shape, periodic=True, kappa_sq=10.0, Lambda_min=0.12, Lambda_max=0.23, m=0, radius=0.05,
                  variance=1e-4, seed=1, lo=0.1, hi=0.9):
    """Shifted-Laplace FEM prior (constant kappa^2 or the periodic
    correlation length) with m ball measurements."""
    dim = len(shape)
    if periodic:
        op_p = M.LinearOperator.shifted_laplace_fem_periodic(shape, Lambda_min, Lambda_max)
        op_o = O.Operator.fem(list(shape), 1, Lambda_min, Lambda_max)
    else:
        op_p = M.LinearOperator.shifted_laplace_fem(shape, kappa_sq)
        op_o = O.Operator.fem(list(shape), 0, kappa_sq)
    if m > 0:
        rng = np.random.default_rng(seed)
        loc = rng.uniform(lo, hi, size=(m, dim))
        var = np.ones(m)
        op_o.add_measurements(loc, var, variance_scaling=variance, radius=radius)
        op_p = op_p.with_measurements(loc, var, variance_scaling=variance, radius=radius)
    return op_o, op_p


# Config 1 of the benchmark suite: the 2D prior on 64^2 cells (63^2 = 3,969
# unknowns), kappa^2 = 10, no measurements, V(1,1) SSOR (omega = 1) on 4
# levels with the Cholesky sampler on the 8^2-cell coarse level; 10^4 samples
# after 100 burn-in steps.
CONFIG1_SHAPE = (64, 64)
CONFIG1_NLEVEL = 4
CONFIG1_BURNIN = 100
CONFIG1_NSAMPLES = 10000


def config1_mean():
    """Exact mean of the config-1 run: mu uniform in [0, 1] per vertex, and
    f = Q mu (the reference's test right hand side, test_sampler.hh:113-130)."""
    n = int(np.prod([c - 1 for c in CONFIG1_SHAPE]))
    return np.random.default_rng(1342517).uniform(0.0, 1.0, n)


def config1_check(X, mu, C, z, tau_bound=1.5):
    """Sample moments of the chain X (nsamples x n) against the exact mean mu
    and covariance C within Monte Carlo error, and the IACT of the observable
    series z; `tau_bound` bounds the integrated autocorrelation time of the
    per-vertex series in the error model.  Returns a dict of the figures;
    raises AssertionError when one is outside its bound:
    - per-vertex variance z-scores (v - C_pp) / (C_pp sqrt(2 tau / N)):
      maximum below 5, root mean square below 1.25;
    - per-vertex mean z-scores (m - mu_p) / sqrt(tau C_pp / N): the same;
    - relative Frobenius error of the sample covariance below 1.3 times its
      expected Monte Carlo size sqrt(tau sum(C_pq^2 + C_pp C_qq) / N) / |C|;
    - the observable's IACT (window 50) between 0.7 and 2.0 (the reference
      publishes 1.2-1.3 for MGMC)."""
    import multigridmc_gb300 as M
    N = X.shape[0]
    d = np.diag(C)
    m, v = X.mean(0), X.var(0)
    zm = (m - mu) / np.sqrt(tau_bound * d / N)
    zv = (v - d) / (d * np.sqrt(2.0 * tau_bound / N))
    Ch = np.cov(X.T, bias=True)
    rel = np.linalg.norm(Ch - C) / np.linalg.norm(C)
    expected = np.sqrt(tau_bound * np.sum(C ** 2 + np.outer(d, d)) / N) / np.linalg.norm(C)
    tau = M.statistics.tau_int(z, 50)
    out = {"mean_z_max": float(np.abs(zm).max()), "mean_z_rms": float(np.sqrt(np.mean(zm ** 2))),
           "var_z_max": float(np.abs(zv).max()), "var_z_rms": float(np.sqrt(np.mean(zv ** 2))),
           "cov_rel_frobenius": float(rel), "cov_rel_frobenius_expected": float(expected), "iact": float(tau),
           "var_max_abs_err": float(np.abs(v - d).max())}
    assert out["mean_z_max"] < 5.0 and out["mean_z_rms"] < 1.25, out
    assert out["var_z_max"] < 5.0 and out["var_z_rms"] < 1.25, out
    assert rel < 1.3 * expected, out
    assert 0.7 < tau < 2.0, out
    return out
