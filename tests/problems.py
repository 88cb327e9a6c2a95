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
