"""Host-side set-up of the GB300 library (no GPU needed): FD stencil,
measurement vectors and Galerkin coarse stencils against the oracle, and the
C ABI's exported symbols against include/mgmc_gb300.h."""
import os
import re

import numpy as np
import pytest

import multigridmc_gb300 as M
import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol():
    lib = M.load()
    hdr = open(os.path.join(ROOT, "include", "mgmc_gb300.h")).read()
    names = set(re.findall(r"\b(mgmc_[a-z0-9_]+)\s*\(", hdr))
    assert names, "no declarations found"
    for n in sorted(names):
        assert hasattr(lib, n), n
    assert names == set(M.SIGNATURES), "binding table and header differ"
    assert lib.mgmc_abi_version() == 2


@pytest.mark.parametrize("shape", [(8,), (64, 64), (16, 16, 16), (6, 10, 4), (256, 256, 256)])
def test_fd_stencil_bitwise(shape):
    assert np.array_equal(M.fd_stencil(shape, 10.0), O.fd_stencil(shape, 10.0))


@pytest.mark.parametrize("shape", [(32, 32), (16, 16, 16), (64, 64, 64), (24, 40, 32)])
def test_measurement_vector_bitwise(shape):
    rng = np.random.default_rng(11)
    for _ in range(4):
        x0 = rng.uniform(0.1, 0.9, len(shape))
        for r in (0.05, 0.0, 0.13):
            i1, v1 = M.measurement_vector(shape, x0, r)
            i2, v2 = O.measurement_vector(shape, x0, r)
            assert np.array_equal(i1, i2) and np.array_equal(v1, v2)


def test_measurement_vector_integrates_to_one():
    # B columns approximate the ball average: sum of weights ~ 1 for R >> h
    i, v = M.measurement_vector((128, 128, 128), [0.5, 0.5, 0.5], 0.05)
    assert abs(v.sum() - 1.0) < 2e-2


@pytest.mark.parametrize("shape", [(16,), (16, 16), (8, 8, 8), (8, 12, 16)])
def test_galerkin_stencil_matches_sparse_rap(shape):
    op = O.Operator.fd(list(shape), 10.0)
    st = M.fd_stencil(shape, 10.0)
    for _ in range(2):
        cop = op.coarsen()
        st = M.galerkin_stencil(len(shape), st)
        ref = O.Operator.from_stencil(cop.shape, st)
        A, R = cop.dense(), ref.dense()
        assert np.abs(A - R).max() <= 4e-15 * np.abs(A).max()
        op = cop


def test_operator_description():
    op = M.LinearOperator.shifted_laplace_fd((16, 16, 16), Lambda=0.31622776601683794)
    assert abs(op.stencil[13] - (10.0 + 6 * 256) / 4096) < 1e-12
    loc = np.array([[0.3, 0.4, 0.5], [0.6, 0.5, 0.4]])
    op = op.with_measurements(loc, [1.0, 2.0], variance_scaling=1e-4, radius=0.1)
    assert op.m == 2 and np.allclose(op.Sigma, [1e-4, 2e-4])
    oo = O.Operator.fd([16, 16, 16], 10.0)
    oo.add_measurements(loc, [1.0, 2.0], variance_scaling=1e-4, radius=0.1)
    Bd, sig = oo.B_dense()
    assert np.array_equal(Bd, op.B_dense()) and np.array_equal(sig, op.Sigma)


def test_sparse_operator_and_exact_observable_moments():
    """LinearOperator.to_scipy assembles A_0 + B Sigma^{-1} B^T (A_0 equal to
    the oracle's CSR operator), and the exact moments of z = b^T x used by the
    convergence measurement agree with a dense solve."""
    from multigridmc_gb300.measurements import exact_observable_moments
    from problems import posterior, rhs
    for shape, m in [((16, 16, 16), 4), ((12, 10), 2), ((9,), 0)]:
        op_o, op_p = posterior(shape, m=m, radius=0.1)
        A = op_p.to_scipy().toarray()
        B = op_p.B_dense()
        A0 = A - (B / op_p.Sigma) @ B.T if m else A
        assert np.abs(A0 - op_o.dense()).max() <= 1e-12 * np.abs(A0).max()
    _, op = posterior((12, 12), m=3, radius=0.1)
    f = rhs(op)
    bidx, bval = M.measurement_vector((12, 12), [0.5, 0.5], 0.1)
    mu, var = exact_observable_moments(op, f, bidx, bval)
    A = op.to_scipy().toarray()
    b = np.zeros(op.n)
    b[bidx] = bval
    assert abs(mu - b @ np.linalg.solve(A, f)) <= 1e-9 * abs(mu)
    assert abs(var - b @ np.linalg.solve(A, b)) <= 1e-9 * var


def test_periodic_correlation_length_model():
    """kappa^2(x) of PeriodicCorrelationLengthModel (correlationlength_model.hh:83-112)
    at the vertex coordinates, and the variable FD diagonal in to_scipy."""
    shape = (6, 5, 4)
    k = M.LinearOperator.periodic_kappa_sq(shape, 0.1, 0.3)
    ref = []
    for c in range(3):
        for b in range(4):
            for a in range(5):
                lam = 0.1
                for xd in ((a + 1) / 6, (b + 1) / 5, (c + 1) / 4):
                    lam *= np.cos(np.pi * xd)
                ref.append(1.0 / (lam + 0.2) ** 2)
    assert np.allclose(k, ref, rtol=1e-14)
    op = M.LinearOperator.shifted_laplace_fd_periodic(shape, 0.1, 0.3)
    hd = 1.0 / (6 * 5 * 4)
    assert np.allclose(op.centre, hd * k + 2 * hd * (36 + 25 + 16), rtol=1e-14)
    A = op.to_scipy()
    assert np.allclose(A.diagonal(), op.centre)
    assert np.allclose(A[0, 1], -hd * 36)


@pytest.mark.parametrize("shape", [(8, 8), (6, 10), (8, 8, 8), (6, 4, 10)])
@pytest.mark.parametrize("model", [0, 1], ids=["constant", "periodic"])
def test_fem_operator_equals_oracle(shape, model):
    """ShiftedLaplaceFEMOperator (shiftedlaplace_fem_operator.cc:9-152): the
    library's per-vertex stencils equal the oracle's assembled matrix bit for
    bit, constant and periodic correlation length."""
    p0, p1 = (10.0, 0.0) if model == 0 else (0.12, 0.23)
    A = O.Operator.fem(list(shape), model, p0, p1).dense()
    if model == 0:
        op = M.LinearOperator.shifted_laplace_fem(shape, p0)
    else:
        op = M.LinearOperator.shifted_laplace_fem_periodic(shape, p0, p1)
    assert np.array_equal(op.to_scipy().toarray(), A)


@pytest.mark.parametrize("kind", ["fd-1d-lowrank", "fd-2d", "fd-3d", "fd-periodic-2d", "fem-periodic-3d"])
def test_operator_coarsen_matches_oracle(kind):
    """LinearOperator.coarsen (mgmc_operator_coarsen; linear_operator.cc:10-23)
    twice: the coarse operators R A R^T + (R B) Sigma^{-1} (R B)^T equal the
    oracle's sparse triple products on random vectors to 1e-13, for a
    constant stencil, the per-vertex centre of the periodic FD prior and the
    per-vertex stencils of the periodic FEM prior."""
    from problems import fem_posterior, operator_1d, periodic_posterior, posterior
    if kind == "fd-1d-lowrank":
        op_o, op_p = operator_1d(True)
        depth = 1
    elif kind == "fd-2d":
        op_o, op_p = posterior((32, 32), m=4, radius=0.1)
        depth = 2
    elif kind == "fd-3d":
        op_o, op_p = posterior((16, 16, 16), m=6, radius=0.1)
        depth = 2
    elif kind == "fd-periodic-2d":
        op_o, op_p = periodic_posterior((32, 32), m=3, radius=0.1)
        depth = 2
    else:
        op_o, op_p = fem_posterior((16, 16, 16), m=3, radius=0.1)
        depth = 2
    rng = np.random.default_rng(11)
    for _ in range(depth):
        op_o, op_p = op_o.coarsen(), op_p.coarsen()
        assert op_p.n == op_o.n and op_p.m == op_o.m
        x = rng.standard_normal(op_p.n)
        yo = op_o.apply(x)
        yp = op_p.to_scipy() @ x
        assert np.linalg.norm(yp - yo) <= 1e-13 * np.linalg.norm(yo), kind


def test_operator_coarsen_errors():
    """An odd lattice cannot be coarsened: a status code, not an exit."""
    op = M.LinearOperator.shifted_laplace_fd((10, 10), 10.0)
    op2 = op.coarsen()
    assert op2.shape == (5, 5)
    with pytest.raises(M.MGMCError) as e:
        op2.coarsen()
    assert e.value.status == 2


@pytest.mark.parametrize("shape", [(16,), (16, 8), (8, 16, 32)])
def test_intergrid_to_sparse(shape):
    """IntergridOperator::to_sparse (intergrid_operator.hh:122-144): R x and
    R^T x_c equal the oracle's restrict and prolongate_add."""
    R = M.intergrid_to_sparse(shape)
    rng = np.random.default_rng(2)
    x = rng.standard_normal(R.shape[1])
    xc = rng.standard_normal(R.shape[0])
    assert np.allclose(R @ x, O.restrict(shape, x), rtol=0, atol=1e-14)
    xp = np.zeros(R.shape[1])
    O.prolongate_add(shape, 1.0, xc, xp)
    assert np.allclose(R.T @ xc, xp, rtol=0, atol=1e-14)


@pytest.mark.parametrize("kind", ["fem-periodic", "fd-periodic"])
def test_noalloc_apply_refuses_variable_coefficients(kind):
    """mgmc_measured_apply_noalloc takes one constant stencil; the wrapper
    refuses operators with a per-vertex centre or stencil field (the call
    never reaches the library, so no GPU is needed)."""
    if kind == "fem-periodic":
        op = M.LinearOperator.shifted_laplace_fem_periodic((8, 8), 0.12, 0.23)
    else:
        op = M.LinearOperator.shifted_laplace_fd_periodic((8, 8), 0.12, 0.23)
    with pytest.raises(M.MGMCError) as e:
        M.measured_apply_noalloc(op, 0, 0, 0, 0, 0, 0, 0)
    assert e.value.status == 1 and "constant stencil" in str(e.value)
