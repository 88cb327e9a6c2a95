"""Variable coefficients: the FD prior with the periodic correlation length
(src/linear_operator/correlationlength_model.hh:83-112, a per-vertex
diagonal of shiftedlaplace_fd_operator.cc:33-52) and its Galerkin coarse
levels with per-point 27-point stencils.  Pathwise parity with the oracle
(whose sparse triple product coarsens the same operator), the operator on
every level, the FP32-mixed chain, the solver, the exact sampler, and the
combinations that are refused."""
import numpy as np
import pytest

import multigridmc_gb300 as M
import oracle as O
from problems import fem_posterior, periodic_posterior, rhs
from test_gpu_parity import _mg, _run_parity

pytestmark = pytest.mark.gpu

CASES = [
    ("2d-prior-32", lambda: periodic_posterior((32, 32)), _mg(4)),
    ("2d-post-32", lambda: periodic_posterior((32, 32), m=3, radius=0.1), _mg(4, omega=1.2)),
    ("3d-post-16", lambda: periodic_posterior((16, 16, 16), m=4), _mg(3)),
    ("3d-post-16-sor-w-coarse-ssor", lambda: periodic_posterior((16, 16, 16), m=4),
     _mg(3, omega=0.9, cycle=2, smoother="SOR", coarse="SSOR")),
    ("3d-post-32", lambda: periodic_posterior((32, 32, 32), m=8), _mg(4)),
    # the FEM prior: a per-vertex 27-point (9-point in 2D) stencil on the fine level
    ("2d-fem-periodic-32", lambda: fem_posterior((32, 32), m=3, radius=0.1), _mg(4)),
    ("3d-fem-periodic-16", lambda: fem_posterior((16, 16, 16), m=4), _mg(3)),
    ("3d-fem-constant-16", lambda: fem_posterior((16, 16, 16), periodic=False, m=4), _mg(3)),
]


@pytest.mark.parametrize("name,mk,prm", CASES, ids=[c[0] for c in CASES])
def test_chain_parity_fp64(name, mk, prm):
    """FP64 chain against the oracle with the same injected noise, within
    1e-12 relative after every step."""
    op_o, op_p = mk()
    nsteps = 40 if op_p.n < 5000 else 10
    worst = _run_parity(op_o, op_p, prm, M.MULTICOLOUR, nsteps)
    assert worst < 1e-12, f"{name}: max relative deviation {worst:.3e}"


FP32_CASES = CASES[1:3] + [
    # weak measurements: the low-rank correction depends on the scale of
    # C = M^{-1} B (with Sigma = 1e-4 it nearly does not), so this case
    # checks the FP64 set-up sweeps of an FP32 chain on the variable field
    ("3d-post-16-weak", lambda: periodic_posterior((16, 16, 16), m=4, variance=1e-1), _mg(3)),
]


@pytest.mark.parametrize("name,mk,prm", FP32_CASES, ids=[c[0] for c in FP32_CASES])
def test_chain_parity_fp32(name, mk, prm):
    """FP32-mixed chain (the fine sweep with the centre field in float4
    spans) against the FP64 oracle: FP32 rounding only."""
    op_o, op_p = mk()
    worst = _run_parity(op_o, op_p, prm, M.MULTICOLOUR, 20, precision=M.FP32_MIXED)
    assert worst < 1e-4, f"{name}: max relative deviation {worst:.3e}"


@pytest.mark.parametrize("precision", [M.FP64, M.FP32_MIXED], ids=["fp64", "fp32-mixed"])
def test_operator_on_every_level(precision):
    """y = A x on every level (the GPU's per-point Galerkin fields) against
    the oracle's sparse triple products."""
    op_o, op_p = periodic_posterior((32, 32, 32), m=4)
    s = M.MultigridMCSampler(op_p, _mg(4), precision=precision)
    rng = np.random.default_rng(4)
    o = op_o
    tol = 1e-13 if precision == M.FP64 else 1e-5
    for lev in range(4):
        x = rng.standard_normal(o.n)
        ref = o.apply(x)
        got = s.level_apply(lev, x)
        assert np.linalg.norm(got - ref) <= tol * np.linalg.norm(ref), f"level {lev}"
        if lev < 3:
            o = o.coarsen()
    s.close()


def test_loop_solver_matches_oracle():
    """The multigrid loop solver on the variable operator: the oracle's
    iteration count and solution."""
    op_o, op_p = periodic_posterior((32, 32, 32), m=4)
    x_exact = np.random.default_rng(4).standard_normal(op_p.n)
    b = op_o.apply(x_exact)
    ref, it_o, _, conv_o = O.MGPreconditioner(op_o, 4, "SSOR", ordering=1, woodbury=False).loop_solve(b, 1e-11, 1e-9, 60)
    s = M.MultigridMCSampler(op_p, _mg(4), noise=M.INJECTED)
    x, it, rn, conv = s.solve(b, 1e-11, 1e-9, 60)
    s.close()
    assert conv and conv_o and abs(it - it_o) <= 1
    assert np.linalg.norm(x - ref) <= 1e-10 * np.linalg.norm(ref)


def test_exact_sampler_moments():
    """Exact draws on the variable prior: per-vertex c_0 in the
    perturbation; mean and covariance within Monte Carlo error."""
    _, op = periodic_posterior((8, 8), m=2, radius=0.2, variance=1e-2)
    Q = op.to_scipy().toarray()
    C = np.linalg.inv(Q)
    f = np.random.default_rng(1).standard_normal(op.n)
    s = M.MultigridMCSampler(op, _mg(2), seed=5)
    N = 4000
    X = np.array([s.exact_sample(f, rtol=1e-11)[0] for _ in range(N)])
    s.close()
    assert np.linalg.norm(X.mean(0) - C @ f) <= 4.5 * np.sqrt(np.trace(C) / N)
    se = np.sqrt(np.sum(C ** 2 + np.outer(np.diag(C), np.diag(C))) / N)
    assert np.linalg.norm(np.cov(X.T) - C) <= 4.5 * se


def test_refused_combinations():
    """A per-vertex centre needs dim >= 2 and the multicolour order; the
    parameter adjoint needs a constant stencil."""
    _, op = periodic_posterior((16, 16))
    with pytest.raises(M.MGMCError) as e:
        M.MultigridMCSampler(op, _mg(3), ordering=M.LEXICOGRAPHIC)
    assert e.value.name == "MGMC_ERR_UNSUPPORTED"
    op1 = M.LinearOperator((8,), M.fd_stencil((8,), 10.0), centre=np.full(7, 5.0))
    with pytest.raises(M.MGMCError) as e:
        M.MultigridMCSampler(op1, _mg(2))
    assert e.value.name == "MGMC_ERR_UNSUPPORTED"
    s = M.MultigridMCSampler(op, _mg(3), noise=M.INJECTED)
    s.inject_noise(np.zeros(s.noise_per_step))
    with pytest.raises(M.MGMCError) as e:
        s.adjoint_params(np.zeros(op.n), np.ones(op.n), np.zeros(op.n))
    assert e.value.name == "MGMC_ERR_UNSUPPORTED"
    s.close()


@pytest.mark.parametrize("lowrank", [False, True], ids=["prior", "measured"])
@pytest.mark.parametrize("precision", [M.FP64, M.FP32_MIXED], ids=["fp64", "fp32-mixed"])
def test_reference_solver_tests_fem(lowrank, precision):
    """TestMultigrid / TestMultigridLowRank of test_solver.hh:112-170 on their
    operator: the FEM prior with the periodic correlation length (Lambda in
    [0.12, 0.23]) on 256^2, 10 measurements with variance 1 + 2U scaled by
    1e-6 for the low-rank case; 5 levels, SSOR V(1,1), rtol 1e-13, atol 1e-12
    (1e-11), maxiter 100; relative error below 1e-10."""
    rng = np.random.default_rng(1212417)
    op = M.LinearOperator.shifted_laplace_fem_periodic((256, 256), 0.12, 0.23)
    if lowrank:
        loc = rng.uniform(size=(10, 2))
        var = 1.0 + 2.0 * rng.uniform(size=10)
        op = op.with_measurements(loc, var, variance_scaling=1e-6, radius=0.05)
    x_exact = np.random.default_rng(3).standard_normal(op.n)
    b = op.to_scipy() @ x_exact
    P = M.MultigridPreconditioner(op, _mg(5), precision=precision)
    S = M.LoopSolver(op, P, M.IterativeSolverParameters(rtol=1e-13, atol=1e-11 if lowrank else 1e-12, maxiter=100))
    x = S.apply(b)
    P.close()
    assert S.converged
    assert np.linalg.norm(x - x_exact) / np.linalg.norm(x_exact) < 1e-10
