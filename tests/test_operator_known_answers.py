"""The reference's operator tests (src/linear_operator/test_linear_operator.hh:
176-245), restated: the shifted-Laplace FD and FEM operators with the
periodic correlation length (Lambda in [1.3, 2.3]) applied to
u = prod_d f(x_d), f(z) = 100 z^2 (1 - z) exp(-6 z), against the exact
(kappa^2(x) u - Laplace u) times the cell volume; relative error below
2e-4 on 512^2 cells and 7e-3 on 64^3.  Checked for the library's host
assembly (the constant stencil with per-vertex centre weights, and the
per-vertex FEM stencils, exactly as the samplers upload them; applied on the
host through LinearOperator.to_scipy) and for the oracle's FEM operator."""
import numpy as np
import pytest

import multigridmc_gb300 as M
import oracle as O

LAMBDA_MIN, LAMBDA_MAX = 1.3, 2.3


def _f(z):
    return 100.0 * z * z * (1.0 - z) * np.exp(-6.0 * z)


def _d2f(z):
    return 100.0 * (2.0 + z * (-30.0 + z * (72.0 - 36.0 * z))) * np.exp(-6.0 * z)


def _exact(shape):
    """u_exact and the exact right hand side (test_linear_operator.hh:73-101)
    in the reference's vertex order (x fastest; vertex i at (i + 1) / n)."""
    dim = len(shape)
    axes = [(np.arange(c - 1) + 1.0) / c for c in shape]
    mesh = np.meshgrid(*axes[::-1], indexing="ij")
    x = [mesh[dim - 1 - d].ravel() for d in range(dim)]
    lam = 0.5 * (LAMBDA_MAX - LAMBDA_MIN) * np.prod([np.cos(np.pi * xd) for xd in x], axis=0)
    kappa_sq = 1.0 / (0.5 * (LAMBDA_MAX + LAMBDA_MIN) + lam) ** 2
    u = np.prod([_f(xd) for xd in x], axis=0)
    lap = sum(np.prod([_d2f(x[d]) if d == j else _f(x[d]) for d in range(dim)], axis=0) for j in range(dim))
    volume = np.prod([1.0 / c for c in shape])
    return u, (kappa_sq * u - lap) * volume


CASES = [((512, 512), 2e-4), ((64, 64, 64), 7e-3)]


@pytest.mark.parametrize("shape,tol", CASES, ids=["2d-512", "3d-64"])
@pytest.mark.parametrize("kind", ["fd", "fem"])
def test_shifted_laplace_operator(kind, shape, tol):
    """TestShiftedLaplace{FD,FEM}Operator{2d,3d} on the library's operators."""
    if kind == "fd":
        op = M.LinearOperator.shifted_laplace_fd_periodic(shape, LAMBDA_MIN, LAMBDA_MAX)
    else:
        op = M.LinearOperator.shifted_laplace_fem_periodic(shape, LAMBDA_MIN, LAMBDA_MAX)
    u, rhs_exact = _exact(shape)
    rhs = op.to_scipy() @ u
    assert np.linalg.norm(rhs - rhs_exact) / np.linalg.norm(rhs) < tol


@pytest.mark.parametrize("shape,tol", CASES, ids=["2d-512", "3d-64"])
def test_shifted_laplace_fem_operator_oracle(shape, tol):
    """The same known answer for the oracle's FEM assembly, which the GPU
    parity tests compare against."""
    op = O.Operator.fem(list(shape), 1, LAMBDA_MIN, LAMBDA_MAX)
    u, rhs_exact = _exact(shape)
    rhs = op.apply(u)
    assert np.linalg.norm(rhs - rhs_exact) / np.linalg.norm(rhs) < tol


def _csr(op_o):
    import scipy.sparse as sp
    ptr, col, val = op_o.csr()
    return sp.csr_matrix((val, col, ptr), shape=(op_o.n, op_o.n))


@pytest.mark.parametrize("shape", [(8, 8), (8, 8, 8)], ids=["2d", "3d"])
def test_coarsen_fem_operator(shape):
    """TestCoarsenOperator2d / 3d (test_intergrid.hh:179-207): the Galerkin
    coarsening of the FEM operator with Lambda = 1 is the FEM operator of the
    coarse lattice, |difference|_F < 1e-12 -- for the library's
    LinearOperator.coarsen and for the oracle's sparse triple product."""
    import scipy.sparse.linalg as spl
    coarse = tuple(s // 2 for s in shape)
    fine_p = M.LinearOperator.shifted_laplace_fem(shape, Lambda=1.0)
    direct_p = M.LinearOperator.shifted_laplace_fem(coarse, Lambda=1.0)
    assert spl.norm(fine_p.coarsen().to_scipy() - direct_p.to_scipy()) < 1e-12
    fine_o = O.Operator.fem(list(shape), 0, 1.0)
    direct_o = O.Operator.fem(list(coarse), 0, 1.0)
    assert spl.norm(_csr(fine_o.coarsen()) - _csr(direct_o)) < 1e-12
