"""Statistical checks of the throughput mode (in-kernel Philox noise) and
size-independent properties at the benchmark size.

* Philox4x32-10 equals cuRAND's implementation bit for bit; the FP32
  Box-Muller normals follow N(0,1) (CDF within 2e-4 over 2^24 draws, the
  reference's test_random.hh:78-110 criterion).
* Sampler mean and covariance against the exact ones (test_sampler.hh:113-153)
  for TestOperator1d and a 2D posterior, FP64 and FP32-mixed.
* At 256^3: a noise-free SOR sweep leaves the exact solution of A x = b
  invariant (test_smoother.hh:90-114), through the fused fine-level kernel
  and the low-rank update.
"""
import ctypes as C
from math import erf, sqrt

import numpy as np
import pytest

import multigridmc_gb300 as M
from problems import operator_1d, posterior

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def philox_lib():
    from gpu_helpers import build as hb
    lib = C.CDLL(hb.build())
    lib.philox_check.restype = C.c_int
    return lib


def test_philox_matches_curand(philox_lib):
    n = 1 << 20
    rng = np.random.default_rng(5)
    ctr = rng.integers(0, 2 ** 32, size=(n, 4), dtype=np.uint64).astype(np.uint32)
    key = rng.integers(0, 2 ** 32, size=(n, 2), dtype=np.uint64).astype(np.uint32)
    mine = np.zeros((n, 4), np.uint32)
    ref = np.zeros((n, 4), np.uint32)
    nrm = np.zeros((n, 4), np.float32)
    P = lambda a: a.ctypes.data_as(C.c_void_p)
    assert philox_lib.philox_check(P(ctr), P(key), P(mine), P(ref), P(nrm), n) == 0
    assert np.array_equal(mine, ref)


def test_normals_cdf(philox_lib):
    n = 1 << 22  # 2^24 normals
    ctr = np.zeros((n, 4), np.uint32)
    ctr[:, 0] = np.arange(n, dtype=np.uint32)
    ctr[:, 1] = 7
    key = np.tile(np.array([[12345, 678]], np.uint32), (n, 1))
    mine = np.zeros((n, 4), np.uint32)
    ref = np.zeros((n, 4), np.uint32)
    nrm = np.zeros((n, 4), np.float32)
    P = lambda a: a.ctypes.data_as(C.c_void_p)
    assert philox_lib.philox_check(P(ctr), P(key), P(mine), P(ref), P(nrm), n) == 0
    z = nrm.astype(np.float64).ravel()
    assert np.all(np.isfinite(z))
    nbins = 64
    idx = np.maximum(np.floor((z + 10.0) / 20.0 * nbins).astype(int), 0)
    cdf = np.cumsum(np.bincount(idx, minlength=nbins)[:nbins] / len(z))
    xs = -10.0 + (np.arange(nbins) + 1) / nbins * 20.0
    true = np.array([0.5 * (1 + erf(x / sqrt(2.0))) for x in xs])
    assert np.max(np.abs(cdf - true)) < 2e-4
    assert abs(z.mean()) < 2e-3 and abs(z.var() - 1.0) < 2e-3


def _mean_cov(sampler, Q, nwarm, nsamp, seed=1342517):
    n = Q.shape[0]
    rng = np.random.default_rng(seed)
    mu = rng.uniform(0.0, 1.0, n)
    f = Q @ mu
    sampler.fix_rhs(f)
    sampler.set_state(np.zeros(n))
    sampler.step(nwarm)
    X = np.zeros((nsamp, n))
    for k in range(nsamp):
        sampler.step(1)
        X[k] = sampler.get_state()
    return mu, X


def _exact(op_p):
    import oracle as O
    shape = op_p.shape
    oo = O.Operator.from_stencil(list(shape), op_p.stencil)
    if op_p.m:
        oo.set_lowrank(op_p.B_dense(), op_p.Sigma)
    return oo.precision()


@pytest.mark.parametrize("kind", ["mgmc", "ssor", "cholesky"])
@pytest.mark.parametrize("lowrank", [False, True])
def test_sampler_1d_statistics(kind, lowrank):
    _, op = operator_1d(lowrank)
    Q = _exact(op)
    if kind == "mgmc":
        s = M.MultigridMCSampler(op, M.MultigridParameters(nlevel=3), precision=M.FP64, seed=11)
    elif kind == "ssor":
        s = M.SSORSampler(op, omega=0.8, precision=M.FP64, seed=12)
    else:
        s = M.CholeskySampler(op, precision=M.FP64, seed=13)
    mu, X = _mean_cov(s, Q, 1000, 100000)
    C_exact = np.linalg.inv(Q)
    err_m = np.abs(X.mean(0) - mu).max()
    err_c = np.abs(np.cov(X.T, bias=True) - C_exact).max()
    # 1e5 samples: Monte Carlo error ~ 1/sqrt(N) of the O(0.2) variances
    assert err_m < 6e-3 and err_c < 6e-3, (err_m, err_c)


@pytest.mark.parametrize("precision", [M.FP64, M.FP32_MIXED])
def test_mgmc_2d_posterior_statistics(precision):
    _, op = posterior((16, 16), kappa_sq=10.0, m=3, radius=0.1, variance=1e-2)
    Q = _exact(op)
    s = M.MultigridMCSampler(op, M.MultigridParameters(nlevel=3), precision=precision, seed=21)
    mu, X = _mean_cov(s, Q, 200, 40000)
    C_exact = np.linalg.inv(Q)
    sd = np.sqrt(np.diag(C_exact))
    z_mean = np.abs(X.mean(0) - mu) / sd
    assert z_mean.max() < 0.05  # 5 sigma of the 1/sqrt(N) * sqrt(tau) error
    err_c = np.abs(np.cov(X.T, bias=True) - C_exact).max() / C_exact.max()
    assert err_c < 0.04, err_c


def test_iact_2d_prior():
    """Config 1: 2D prior 64^2 cells, kappa^2 = 10, V(1,1) SSOR, 4 levels,
    coarse Cholesky at 8^2 cells: the MGMC chain decorrelates within ~1-2
    steps (reference: IACT 1.2-1.3), the single-level SSOR chain does not."""
    _, op = posterior((64, 64), kappa_sq=10.0)
    b_idx, b_val = M.measurement_vector((64, 64), [0.5, 0.5], 0.05)
    taus = {}
    for name, s in (("mgmc", M.MultigridMCSampler(op, M.MultigridParameters(nlevel=4), precision=M.FP64, seed=3)),
                    ("ssor", M.SSORSampler(op, omega=1.0, precision=M.FP64, seed=4))):
        s.fix_rhs(np.zeros(op.n))
        s.set_observable(b_idx, b_val, 20100)
        s.step(20100)
        z = s.read_observations(20100)[100:]
        taus[name] = M.statistics.tau_int(z, 50)
    assert 0.7 < taus["mgmc"] < 2.0, taus
    assert taus["ssor"] > taus["mgmc"] + 1.0, taus


@pytest.mark.parametrize("precision,tol", [(M.FP64, 1e-12), (M.FP32_MIXED, 2e-5)])
def test_fixed_point_256cubed(precision, tol):
    """A noise-free SOR sweep with the low-rank update maps the exact
    solution of A x = b to itself, at the benchmark size."""
    import bench
    op, _, _, _, _ = bench.problem()
    s = M.MultigridMCSampler(op, M.MultigridParameters(nlevel=5), precision=precision, seed=1)
    rng = np.random.default_rng(9)
    x = rng.standard_normal(op.n)
    b = s.level_apply(0, x)
    for direction in (M.FORWARD, M.BACKWARD):
        y = s.sor(0, direction, b, x.copy(), with_noise=False)
        assert np.linalg.norm(y - x) / np.linalg.norm(x) < tol


def test_convergence_of_observable_moments():
    """measure_convergence (convergence.cc:4-161) over 400 batched FP64
    chains from x = 0: after a few MGMC steps the mean and variance of the
    observable z = b^T x agree with the exact ones within 5 standard errors."""
    from multigridmc_gb300.measurements import exact_observable_moments, measure_convergence
    from problems import posterior, rhs
    shape = (16, 16, 16)
    _, op = posterior(shape, m=4, radius=0.1)
    f = rhs(op)
    bidx, bval = M.measurement_vector(shape, [0.5, 0.5, 0.5], 0.1)
    mu, var = exact_observable_moments(op, f, bidx, bval)
    res = measure_convergence(op, M.MultigridParameters(nlevel=3), f, bidx, bval, nchain=400, nsteps=10,
                              seed=900, precision=M.FP64)
    for k in range(4, 11):
        assert abs(res["mean"][k] - mu) <= 5 * res["err_mean"][k], (k, res["mean"][k], mu)
        assert abs(res["variance"][k] - var) <= 5 * res["err_variance"][k], (k, res["variance"][k], var)


def test_mean_squared_error_of_running_average():
    """measure_mean_squared_error (mean_squared_error.cc:4-65) over 400
    batched FP64 chains: the squared error of the running average falls like
    the bias (mean / (j + 1))^2 plus tau Var / (j + 1) predicts."""
    from multigridmc_gb300.measurements import exact_observable_moments, measure_mean_squared_error
    from problems import posterior, rhs
    shape = (16, 16, 16)
    _, op = posterior(shape, m=4, radius=0.1)
    f = rhs(op)
    bidx, bval = M.measurement_vector(shape, [0.5, 0.5, 0.5], 0.1)
    mu, var = exact_observable_moments(op, f, bidx, bval)
    res = measure_mean_squared_error(op, M.MultigridParameters(nlevel=3), f, bidx, bval, mu, nchain=400, nsteps=12,
                                     seed=1900, precision=M.FP64)
    mse = res["mse"]
    assert mse[0] == pytest.approx(mu * mu)  # the running average starts at z^0 = 0
    for j in (6, 11):
        model = (mu / (j + 1)) ** 2 + 2.0 * var / (j + 1)
        assert mse[j] < model, (j, mse[j], model)
        assert mse[j] > 0.25 * var / (j + 1), (j, mse[j])


@pytest.mark.parametrize("precision", [M.FP64, M.FP32_MIXED], ids=["fp64", "fp32-mixed"])
def test_config1_2d_prior_variance(precision):
    """Config 1 in full on the GPU: 2D prior on 64^2 cells, kappa^2 = 10,
    V(1,1) SSOR on 4 levels, Cholesky sampler on the 8^2-cell coarse level,
    Philox noise; 10^4 samples after 100 burn-in steps.  Sample mean,
    per-vertex variance and covariance against the exact covariance (dense
    inverse of the precision) within Monte Carlo error, as the reference's
    measured 2D MGMC test checks them (test_sampler.hh:271-334), and the IACT
    of the centre ball average."""
    import oracle as O
    from problems import (CONFIG1_BURNIN, CONFIG1_NLEVEL, CONFIG1_NSAMPLES, CONFIG1_SHAPE, config1_check,
                          config1_mean)
    _, op = posterior(CONFIG1_SHAPE, kappa_sq=10.0)
    oo = O.Operator.fd(list(CONFIG1_SHAPE), 10.0)
    C = oo.covariance()
    mu = config1_mean()
    s = M.MultigridMCSampler(op, M.MultigridParameters(nlevel=CONFIG1_NLEVEL), precision=precision, seed=31)
    s.fix_rhs(oo.precision() @ mu)
    s.set_state(np.zeros(op.n))
    s.step(CONFIG1_BURNIN)
    X = np.zeros((CONFIG1_NSAMPLES, op.n))
    for k in range(CONFIG1_NSAMPLES):
        s.step(1)
        X[k] = s.get_state()
    s.close()
    bidx, bval = M.measurement_vector(CONFIG1_SHAPE, [0.5, 0.5], 0.05)
    config1_check(X, mu, C, X[:, bidx] @ bval)
