"""Oracle pins for the deterministic solvers: the reference's
src/solver/test_solver.hh (CholeskySolver, multigrid-preconditioned
LoopSolver with and without measurements) on its operator, the
shifted-Laplace FEM operator with the periodic correlation length
(Lambda in [0.12, 0.23]), with numpy-seeded exact solutions and measurement
locations, plus the oracle's two coarse-solve forms against each other."""
import numpy as np
import pytest

import oracle as O


def _measured(shape, n_meas=10, variance_scaling=1e-6, radius=0.05, seed=1212417):
    """test_solver.hh:22-80: FEM operator, periodic correlation length, 10
    ball measurements at uniform locations with variance 1 + 2 U, scaled by
    1e-6."""
    rng = np.random.default_rng(seed)
    op = _prior(shape)
    loc = rng.uniform(size=(n_meas, len(shape)))
    var = 1.0 + 2.0 * rng.uniform(size=n_meas)
    op.add_measurements(loc, var, variance_scaling=variance_scaling, radius=radius)
    return op


def _prior(shape):
    return O.Operator.fem(list(shape), 1, 0.12, 0.23)


def _exact(op, seed=3):
    x = np.random.default_rng(seed).standard_normal(op.n)
    return x, op.apply(x)


def test_cholesky_solver():
    """TestCholesky (test_solver.hh:91-105): |x - x_exact| / |x_exact| < 1e-11
    with the Woodbury form, on a 48^2 lattice (the oracle's factor is dense)."""
    op = _measured((48, 48))
    x_exact, b = _exact(op)
    x = O.cholesky_solve(op, b)
    assert np.linalg.norm(x - x_exact) / np.linalg.norm(x_exact) < 1e-11


@pytest.mark.parametrize("lowrank", [False, True], ids=["prior", "measured"])
def test_multigrid_loop_solver(lowrank):
    """TestMultigrid / TestMultigridLowRank (test_solver.hh:112-170): 256^2,
    5 levels, SSOR V(1,1), rtol 1e-13, atol 1e-12 (1e-11 with measurements),
    at most 100 iterations; relative error below 1e-10."""
    op = _measured((256, 256)) if lowrank else _prior((256, 256))
    x_exact, b = _exact(op)
    P = O.MGPreconditioner(op, 5, "SSOR")
    x, it, rn, conv = P.loop_solve(b, 1e-13, 1e-11 if lowrank else 1e-12, 100)
    assert conv and it < 100
    assert np.linalg.norm(x - x_exact) / np.linalg.norm(x_exact) < 1e-10


def test_coarse_forms_agree():
    """The Woodbury coarse solve (the reference's CholeskySolver) and the
    dense factor of the full coarse precision (the GPU's form) give the same
    preconditioner to rounding."""
    op = _measured((32, 32), n_meas=4, variance_scaling=1e-4)
    b = np.random.default_rng(5).standard_normal(op.n)
    pw = O.MGPreconditioner(op, 3, "SSOR", woodbury=True).apply(b)
    pd = O.MGPreconditioner(op, 3, "SSOR", woodbury=False).apply(b)
    assert np.linalg.norm(pw - pd) <= 1e-11 * np.linalg.norm(pw)


def test_sor_smoother_nsmooth_quirk():
    """SORSmoother::apply with nsmooth > 1 runs nsmooth rounds of nsmooth
    sparse sweeps and one low-rank correction (sor_smoother.cc:40-78): with
    npresmooth = npostsmooth = 2 the preconditioner differs from one with
    four single sweeps but still converges as a loop-solver preconditioner."""
    op = _measured((32, 32), n_meas=3, variance_scaling=1e-3)
    x_exact, b = _exact(op)
    P2 = O.MGPreconditioner(op, 3, "SOR", npresmooth=2, npostsmooth=2, woodbury=False)
    x, it, rn, conv = P2.loop_solve(b, 1e-12, 1e-9, 200)
    assert conv
    assert np.linalg.norm(x - x_exact) / np.linalg.norm(x_exact) < 1e-9


def test_preconditioner_symmetric():
    """SSOR pre- and post-smoothing with an exact coarse solve make the
    V-cycle preconditioner symmetric: <P u, v> = <u, P v>."""
    op = _measured((32, 32), n_meas=4, variance_scaling=1e-3)
    rng = np.random.default_rng(8)
    u, v = rng.standard_normal(op.n), rng.standard_normal(op.n)
    P = O.MGPreconditioner(op, 4, "SSOR", omega=1.2, woodbury=False)
    lhs, rhs = P.apply(u) @ v, u @ P.apply(v)
    assert abs(lhs - rhs) <= 1e-12 * np.linalg.norm(P.apply(u)) * np.linalg.norm(v)


def _tridiagonal16():
    """The matrix of CholeskyWrapperTest (test_cholesky_wrapper.hh:14-42):
    16 x 16, 6 on the diagonal, -1 beside it, with x_exact ~ N(0, 1)
    (numpy-seeded here) and b = A x_exact."""
    st = np.zeros(27)
    st[12], st[13], st[14] = -1.0, 6.0, -1.0
    x_exact = np.random.default_rng(1212957).standard_normal(16)
    return st, x_exact


def test_cholesky_wrapper_dense_solve():
    """TestEigenDenseSolve / TestEigenDenseSolveLLT (test_cholesky_wrapper.hh:
    120-143): |x - x_exact| < 1e-12 for the oracle's dense factor."""
    st, x_exact = _tridiagonal16()
    op = O.Operator.from_stencil([17], st)
    b = op.apply(x_exact)
    x = O.cholesky_solve(op, b)
    assert np.linalg.norm(x - x_exact) < 1e-12
