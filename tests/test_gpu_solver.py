"""The deterministic multigrid solver on the GPU (MultigridPreconditioner +
LoopSolver of the reference, src/preconditioner/multigrid_preconditioner.cc
and src/solver/loop_solver.cc) against the oracle's restatement, the
reference's own solver tests (test_solver.hh) on the FD operator, FP32
iterative refinement, and that a solve leaves the chain untouched."""
import numpy as np
import pytest

import multigridmc_gb300 as M
import oracle as O
from problems import operator_1d, posterior

pytestmark = pytest.mark.gpu


def _mg(nlevel, smoother="SSOR", npre=1, npost=1, omega=1.0, cycle=1, alpha=1.0, coarse="Cholesky"):
    return M.MultigridParameters(nlevel=nlevel, smoother=smoother, coarse_solver=coarse, npresmooth=npre,
                                 npostsmooth=npost, omega=omega, cycle=cycle, coarse_scaling=alpha)


def _oracle_prec(op_o, prm, ordering):
    return O.MGPreconditioner(op_o, prm.nlevel, prm.smoother, prm.npresmooth, prm.npostsmooth, prm.omega, prm.cycle,
                              prm.coarse_scaling, ordering, woodbury=False)


CASES = [
    ("1d-lowrank", lambda: operator_1d(True), _mg(3)),
    ("2d-prior-64", lambda: posterior((64, 64)), _mg(4)),
    ("2d-post-64-sor2", lambda: posterior((64, 64), m=4, radius=0.1), _mg(4, "SOR", npre=2, npost=2)),
    ("2d-post-32-w", lambda: posterior((32, 32), m=3, radius=0.1), _mg(3, omega=1.3, cycle=2, alpha=1.4)),
    ("3d-post-16", lambda: posterior((16, 16, 16), m=6), _mg(3)),
    ("3d-post-32-coarse-ssor", lambda: posterior((32, 32, 32), m=8), _mg(4, coarse="SSOR")),
]


def _exact_sampler(op_p, prm, ordering):
    """FP64 with injected noise: the parity kernels (one rounding per
    operation, substitution coarse solve); the noise is not used here."""
    return M.MultigridMCSampler(op_p, prm, ordering=ordering, precision=M.FP64, noise=M.INJECTED)


@pytest.mark.parametrize("name,mk,prm", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("ordering", [M.LEXICOGRAPHIC, M.MULTICOLOUR], ids=["lex", "multicolour"])
def test_preconditioner_matches_oracle(name, mk, prm, ordering):
    """x = P b on the GPU (FP64 parity kernels) against the oracle's
    restatement with the same sweep order, 1e-12 relative."""
    op_o, op_p = mk()
    b = np.random.default_rng(2).standard_normal(op_p.n)
    ref = _oracle_prec(op_o, prm, ordering).apply(b)
    s = _exact_sampler(op_p, prm, ordering)
    got = s.precondition(b)
    s.close()
    assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref), name


@pytest.mark.parametrize("name,mk,prm", CASES, ids=[c[0] for c in CASES])
def test_throughput_preconditioner(name, mk, prm):
    """The throughput kernels (FMA contraction, explicit inverse coarse
    factors; MultigridPreconditioner's default) give the parity kernels'
    P b to 1e-9 relative."""
    _, op_p = mk()
    b = np.random.default_rng(2).standard_normal(op_p.n)
    s = _exact_sampler(op_p, prm, M.MULTICOLOUR)
    ref = s.precondition(b)
    s.close()
    P = M.MultigridPreconditioner(op_p, prm)
    got = P.apply(b)
    P.close()
    assert np.linalg.norm(got - ref) <= 1e-9 * np.linalg.norm(ref), name


@pytest.mark.parametrize("name,mk,prm", CASES[1:5], ids=[c[0] for c in CASES[1:5]])
def test_loop_solver_matches_oracle(name, mk, prm):
    """LoopSolver on the GPU: the oracle's outcome and iteration count
    (within one) and its iterate to 1e-10.  With SOR and nsmooth = 2 the
    reference's smoother (two sparse sweeps, then one low-rank correction)
    makes a weak preconditioner that does not reach the tolerance in 40
    iterations; both stop there with the same iterate."""
    op_o, op_p = mk()
    x_exact = np.random.default_rng(4).standard_normal(op_p.n)
    b = op_o.apply(x_exact)
    ref, it_o, _, conv_o = _oracle_prec(op_o, prm, M.LEXICOGRAPHIC).loop_solve(b, 1e-11, 1e-9, 40)
    s = _exact_sampler(op_p, prm, M.LEXICOGRAPHIC)
    x, it, rn, conv = s.solve(b, 1e-11, 1e-9, 40)
    s.close()
    assert conv == conv_o and conv_o == (prm.npresmooth == 1)
    assert abs(it - it_o) <= 1
    assert np.linalg.norm(x - ref) <= 1e-10 * np.linalg.norm(ref)


@pytest.mark.parametrize("lowrank", [False, True], ids=["prior", "measured"])
@pytest.mark.parametrize("precision", [M.FP64, M.FP32_MIXED], ids=["fp64", "fp32-mixed"])
def test_reference_multigrid_solver_tests(lowrank, precision):
    """TestMultigrid / TestMultigridLowRank (test_solver.hh:112-170) on the
    FD operator: 256^2, 5 levels, SSOR V(1,1), rtol 1e-13, atol 1e-12
    (1e-11 with measurements), maxiter 100; relative error below 1e-10.  The
    FP32-mixed hierarchy reaches it too: the loop keeps x and r in FP64
    (iterative refinement)."""
    rng = np.random.default_rng(1212417)
    op = M.LinearOperator.shifted_laplace_fd((256, 256), 1.0 / 0.15 ** 2)
    if lowrank:
        loc = rng.uniform(size=(10, 2))
        var = 1.0 + 2.0 * rng.uniform(size=10)
        op = op.with_measurements(loc, var, variance_scaling=1e-6, radius=0.05)
    x_exact = np.random.default_rng(3).standard_normal(op.n)
    s = M.MultigridMCSampler(op, _mg(5), precision=M.FP64)
    b = s.level_apply(0, x_exact)
    s.close()
    P = M.MultigridPreconditioner(op, _mg(5), precision=precision)
    S = M.LoopSolver(op, P, M.IterativeSolverParameters(rtol=1e-13, atol=1e-11 if lowrank else 1e-12, maxiter=100))
    x = S.apply(b)
    P.close()
    assert S.converged
    assert np.linalg.norm(x - x_exact) / np.linalg.norm(x_exact) < 1e-10


def test_precondition_symmetric_3d():
    """SSOR V-cycle with the exact coarse solve is symmetric: <P u, v> =
    <u, P v> at 64^3 with measurements (FP64, multicolour)."""
    _, op = posterior((64, 64, 64), m=16)
    rng = np.random.default_rng(6)
    u, v = rng.standard_normal(op.n), rng.standard_normal(op.n)
    P = M.MultigridPreconditioner(op, _mg(4, omega=1.1))
    pu, pv = P.apply(u), P.apply(v)
    P.close()
    assert abs(pu @ v - u @ pv) <= 1e-12 * np.linalg.norm(pu) * np.linalg.norm(v)


def test_solve_leaves_the_chain():
    """A solve between steps changes nothing in the chain: the states after
    2 + 3 steps with a solve in between equal those of 5 steps, bit for bit."""
    _, op = posterior((32, 32, 32), m=8)
    f = np.random.default_rng(1).standard_normal(op.n)
    a = M.MultigridMCSampler(op, _mg(4), seed=5)
    c = M.MultigridMCSampler(op, _mg(4), seed=5)
    for s in (a, c):
        s.fix_rhs(f)
    a.step(5)
    c.step(2)
    x, it, rn, conv = c.solve(f, 1e-10, 1e-6, 50)
    assert conv
    c.step(3)
    assert np.array_equal(a.get_state(), c.get_state())
    a.close()
    c.close()


def test_maxiter_zero_and_zero_rhs():
    """maxiter = 0 returns x = 0, not converged, no residual; b = 0 never
    passes the relative test (|r| / |b| is not a number), as in the
    reference, and returns x = 0 after maxiter iterations."""
    _, op = posterior((16, 16))
    s = M.MultigridMCSampler(op, _mg(3))
    x, it, rn, conv = s.solve(np.ones(op.n), maxiter=0)
    assert not conv and it == 0 and rn == -1.0 and not x.any()
    x, it, rn, conv = s.solve(np.zeros(op.n), maxiter=3)
    assert not conv and it == 3 and rn == 0.0 and not x.any()
    s.close()


def test_cholesky_wrapper_dense_solve():
    """TestEigenDenseSolve / TestEigenDenseSolveLLT (test_cholesky_wrapper.hh:
    14-42, 120-143) on the GPU's coarse Cholesky: the 16 x 16 (6, -1)
    tridiagonal matrix, |x - x_exact| < 1e-12, through the one-level
    preconditioner (the factor's two triangular solves, throughput kernels)
    and through the Cholesky sampler fed zero noise (x = L^-T (0 + L^-1 b),
    the parity kernels)."""
    st = np.zeros(27)
    st[12], st[13], st[14] = -1.0, 6.0, -1.0
    op = M.LinearOperator((17,), st)
    x_exact = np.random.default_rng(1212957).standard_normal(16)
    s = M.CholeskySampler(op, noise=M.INJECTED)
    b = s.level_apply(0, x_exact)
    P = M.MultigridPreconditioner(op, M.MultigridParameters(nlevel=1, coarse_solver="Cholesky"))
    assert np.linalg.norm(P.apply(b) - x_exact) < 1e-12
    P.close()
    s.inject_noise(np.zeros(s.noise_per_step))
    x = np.zeros(16)
    s.apply(b, x)
    s.close()
    assert np.linalg.norm(x - x_exact) < 1e-12
