"""Statistical and algebraic pins of the oracle, restating the reference's
own tests: samplers (src/sampler/test_sampler.hh:113-334), smoother fixed
point (src/smoother/test_smoother.hh:90-114) and intergrid operators
(src/intergrid/test_intergrid.hh:87-171)."""
import numpy as np
import pytest

import oracle as O
from problems import operator_1d, posterior


def _mean_cov_error(op, sampler, nsamples, nwarmup=1000):
    rng = np.random.default_rng(1342517)
    mu = rng.uniform(0.0, 1.0, op.n)
    Q = op.precision()
    f = Q @ mu
    x = np.zeros(op.n)
    Ex, C = sampler.mean_cov(f, x, nwarmup, nsamples)
    return np.abs(Ex - mu).max(), np.abs(C - np.linalg.inv(Q)).max()


@pytest.mark.parametrize("lowrank", [False, True])
@pytest.mark.parametrize("kind", ["cholesky", "lowrank-cholesky", "ssor", "mgmc", "mgmc-multicolour"])
def test_sampler_1d(kind, lowrank):
    op, _ = operator_1d(lowrank)
    src = O.Source()
    if kind == "cholesky":
        s = O.cholesky_sampler(op, src)
    elif kind == "lowrank-cholesky":  # TestLowRankCholeskySampler1d, test_sampler.hh:177-190
        s = O.lowrank_cholesky_sampler(op, src)
    elif kind == "ssor":
        s = O.ssor_sampler(op, src, 0.8)
    elif kind == "mgmc":
        s = O.mgmc_sampler(op, src, 3)
    else:
        s = O.mgmc_sampler(op, src, 3, ordering=1)
    n = 1000000 if kind.startswith("mgmc") else 500000
    em, ec = _mean_cov_error(op, s, n)
    assert em < 2e-3 and ec < 2e-3


def test_mgmc_2d_measured():
    """TestMultigridMCSampler2d (8x8 cells, 4 measurements, radius 0.05,
    variance scaling 1e-4) with the FD prior in place of the FEM one."""
    op, _ = posterior((8, 8), kappa_sq=1.0 / 1.2 ** 2)
    rng = np.random.default_rng(1212417)
    sig = 1.0 + 2.0 * rng.uniform(size=4)
    loc = np.array([[0.25, 0.25], [0.25, 0.75], [0.75, 0.25], [0.75, 0.75]])
    op.add_measurements(loc, sig, variance_scaling=1e-4, radius=0.05)
    s = O.mgmc_sampler(op, O.Source(), 3)
    em, ec = _mean_cov_error(op, s, 10000)
    assert em < 2e-2 and ec < 2e-2


@pytest.mark.parametrize("ordering", [0, 1])
def test_ssor_smoother_fixed_point(ordering):
    """SSOR with and without the low-rank update leaves A x = b invariant."""
    op, _ = posterior((32, 32), kappa_sq=2.0)
    rng = np.random.default_rng(1212417)
    loc = rng.uniform(size=(10, 2))
    var = 1e-6 * (1.0 + 2.0 * rng.uniform(size=10))
    op_lr, _ = posterior((32, 32), kappa_sq=2.0)
    op_lr.add_measurements(loc, var, variance_scaling=1.0, radius=0.05)
    for o in (op, op_lr):
        x_exact = rng.standard_normal(o.n)
        b = o.apply(x_exact)
        x = x_exact.copy()
        O.ssor_smoother_apply(o, 0.8, b, x, ordering=ordering)
        assert np.linalg.norm(x - x_exact) / np.linalg.norm(x_exact) < 1e-12


def test_prolongation_is_linear_interpolation():
    rng = np.random.default_rng(1212417)
    xc = rng.standard_normal(3)
    x = np.zeros(7)
    O.prolongate_add([8], 1.0, xc, x)
    ref = np.zeros(7)
    lat = O.Lattice(4)
    for ic in range(3):
        f = lat.fine_vertex_idx(ic)
        ref[f] += xc[ic]
        ref[f - 1] += 0.5 * xc[ic]
        ref[f + 1] += 0.5 * xc[ic]
    assert np.linalg.norm(x - ref) < 1e-12
    xc = rng.standard_normal(9)
    x = np.zeros(49)
    O.prolongate_add([8, 8], 1.0, xc, x)
    ref = np.zeros(49)
    clat, flat = O.Lattice(4, 4), O.Lattice(8, 8)
    for ic in range(9):
        f = clat.fine_vertex_idx(ic)
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                w = (0.5 if dx else 1.0) * (0.5 if dy else 1.0)
                ref[flat.shift_vertexidx(f, (dx, dy))] += w * xc[ic]
    assert np.linalg.norm(x - ref) < 1e-12


@pytest.mark.parametrize("shape", [(8,), (8, 8), (8, 8, 8)])
def test_restriction_is_transpose_of_prolongation(shape):
    rng = np.random.default_rng(1212417)
    nf = int(np.prod([s - 1 for s in shape]))
    nc = int(np.prod([s // 2 - 1 for s in shape]))
    xc = rng.standard_normal(nc)
    r = rng.standard_normal(nf)
    xp = np.zeros(nf)
    O.prolongate_add(list(shape), 1.0, xc, xp)
    rr = O.restrict(list(shape), r)
    assert abs(xc @ rr - xp @ r) < 1e-12


def test_galerkin_coarse_operator_is_27_point_translation_invariant():
    """The sparse R A P of the FD operator has the same 27 weights at every
    coarse vertex (zero-extension at the Dirichlet boundary)."""
    op, _ = posterior((16, 16, 16))
    cop = op.coarsen()
    ptr, col, val = cop.csr()
    lat = O.Lattice(8, 8, 8)
    seen = {}
    for i in range(cop.n):
        a = lat.vertexidx_linear2euclidean(i)
        for k in range(ptr[i], ptr[i + 1]):
            b = lat.vertexidx_linear2euclidean(col[k])
            off = tuple(b[d] - a[d] for d in range(3))
            seen.setdefault(off, []).append(val[k])
    assert len(seen) == 27
    for off, v in seen.items():
        assert np.ptp(v) <= 1e-15 * max(abs(np.max(v)), 1.0)


def test_injected_noise_reproduces_clcg_chain():
    """A sampler fed the CLCG's normals through the injection hook follows
    the same chain as one drawing them itself."""
    op, _ = posterior((16, 16), m=0)
    f = np.random.default_rng(2).standard_normal(op.n)
    a = O.mgmc_sampler(op, O.Source(), 3)
    xa = np.zeros(op.n)
    a.apply(f, xa, 5)
    noise = O.CLCG().draw_normal(200000)
    src = O.Source(noise)
    b = O.mgmc_sampler(op, src, 3)
    xb = np.zeros(op.n)
    b.apply(f, xb, 5)
    assert np.array_equal(xa, xb)


def test_config1_2d_prior_variance():
    """Config 1 on the oracle (the reference's algorithm: lexicographic SSOR,
    dense Cholesky coarse sampler, CLCG noise): 10^4 samples after 100
    burn-in steps; sample mean, per-vertex variance and covariance against
    the exact Cholesky covariance within Monte Carlo error, and the IACT of
    the ball average at the centre."""
    from problems import (CONFIG1_BURNIN, CONFIG1_NLEVEL, CONFIG1_NSAMPLES, CONFIG1_SHAPE, config1_check,
                          config1_mean)
    op = O.Operator.fd(list(CONFIG1_SHAPE), 10.0)
    C = op.covariance()
    mu = config1_mean()
    f = op.precision() @ mu
    s = O.mgmc_sampler(op, O.Source(), CONFIG1_NLEVEL)
    x = np.zeros(op.n)
    s.apply(f, x, CONFIG1_BURNIN)
    X = np.zeros((CONFIG1_NSAMPLES, op.n))
    for k in range(CONFIG1_NSAMPLES):
        s.apply(f, x, 1)
        X[k] = x
    bidx, bval = O.measurement_vector(list(CONFIG1_SHAPE), [0.5, 0.5], 0.05)
    config1_check(X, mu, C, X[:, bidx] @ bval)


def test_lowrank_cholesky_equals_dense_cholesky_covariance():
    """The low-rank Cholesky sampler's linear map has covariance exactly
    Q^{-1} (A_0 = L L^T, A = L (Id + V Sigma^{-1} V^T) L^T): the sample it
    draws from unit normals e_k, minus its mean, is column k of a square root
    of Q^{-1} -- checked on a 2D posterior with 3 measurements to 1e-12."""
    op, _ = posterior((8, 8), m=3, radius=0.2, variance=1e-2)
    n = op.n
    f = np.zeros(n)
    cols = []
    for k in range(n + 1):
        xi = np.zeros(n)
        if k < n:
            xi[k] = 1.0
        s = O.lowrank_cholesky_sampler(op, O.Source(xi))
        x = np.zeros(n)
        s.apply(f, x)
        cols.append(x)
    Fm = np.array(cols[:n]).T - cols[n][:, None]
    C = np.linalg.inv(op.precision())
    assert np.abs(Fm @ Fm.T - C).max() <= 1e-12 * np.abs(C).max()
