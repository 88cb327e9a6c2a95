"""Chain experiments of the reference's measurement drivers, run as batched
GPU chains.

``measure_convergence`` follows src/measurements/convergence.cc:4-161: many
chains of one sampler start from x = 0 with the same right hand side, the
observable z = b^T x is recorded at every step, and the sample moments of
z^k across chains are compared with the exact mean and variance of z.
``measure_mean_squared_error`` follows mean_squared_error.cc:4-65: the
squared error of each chain's running average of z against the exact mean,
averaged over chains.  The reference runs the chains one after another or on
OpenMP threads; here they advance together in one CUDA graph
(``MultigridMCBatch``).
"""
import numpy as np

from . import MultigridMCBatch, MultigridMCSampler


def exact_observable_moments(op, f, bidx, bval):
    """Exact E[z] = b^T A^{-1} f and Var[z] = b^T A^{-1} b of z = b^T x for
    x ~ N(A^{-1} f, A^{-1}) (LinearOperator::observed_mean_and_variance),
    by conjugate gradients on the assembled sparse A (FP64)."""
    import scipy.sparse.linalg as spla
    A = op.to_scipy()
    b = np.zeros(op.n)
    b[np.asarray(bidx, np.int64)] = bval
    diag = A.diagonal()
    M = spla.LinearOperator(A.shape, matvec=lambda v: v / diag)
    kw = {"rtol": 1e-13} if "rtol" in spla.cg.__code__.co_varnames else {"tol": 1e-13}
    mu, info1 = spla.cg(A, f, M=M, maxiter=20000, **kw)
    w, info2 = spla.cg(A, b, M=M, maxiter=20000, **kw)
    if info1 or info2:
        raise RuntimeError("CG did not converge")
    return float(b @ mu), float(b @ w)


def batched_observations(op, params, f, bidx, bval, nchain, nsteps, seed=0, **sampler_kw):
    """z^k = b^T x^k for k = 0 .. nsteps of `nchain` chains (seeds seed ..
    seed + nchain - 1) started at x^0 = 0 and advanced together; returns an
    (nchain, nsteps + 1) array."""
    chains = []
    for i in range(nchain):
        s = MultigridMCSampler(op, params, seed=seed + i, **sampler_kw)
        s.fix_rhs(f)
        s.set_observable(bidx, bval, nsteps + 8)
        chains.append(s)
    batch = MultigridMCBatch(chains)
    batch.step(nsteps)
    batch.synchronize()
    Z = np.zeros((nchain, nsteps + 1))  # z^0 = 0: the chains start at x = 0
    for i, s in enumerate(chains):
        Z[i, 1:] = s.read_observations(nsteps + 8)[:nsteps]
    batch.close()
    for s in chains:
        s.close()
    return Z


def measure_convergence(op, params, f, bidx, bval, nchain, nsteps, seed=0, **sampler_kw):
    """Moments of z^k = b^T x^k over `nchain` chains started at x^0 = 0, for
    k = 0 .. nsteps (convergence.cc:44-64).  Returns a dict of per-step
    arrays: mean, variance (biased, as the reference's x2_avg - x_avg^2),
    and the statistical errors of both (convergence.cc:96-99)."""
    Z = batched_observations(op, params, f, bidx, bval, nchain, nsteps, seed, **sampler_kw)
    m1 = Z.mean(0)
    m2 = (Z ** 2).mean(0)
    m3 = (Z ** 3).mean(0)
    m4 = (Z ** 4).mean(0)
    var = m2 - m1 ** 2
    sigma_sq = nchain / (nchain - 1.0) * var
    mu4 = m4 - 4 * m1 * m3 + 6 * m1 ** 2 * m2 - 3 * m1 ** 4
    err_mean = np.sqrt(sigma_sq / nchain)
    err_var = np.sqrt(np.maximum(mu4 - (nchain - 3.0) / (nchain - 1.0) * sigma_sq ** 2, 0.0) / nchain)
    return {"mean": m1, "variance": var, "err_mean": err_mean, "err_variance": err_var, "nchain": nchain,
            "nsteps": nsteps}


def measure_mean_squared_error(op, params, f, bidx, bval, mean_exact, nchain, nsteps, seed=0, **sampler_kw):
    """Mean squared error of the running average of z over steps 0 .. j
    (including the start x^0 = 0) against the exact mean, averaged over
    `nchain` chains, for j = 0 .. nsteps - 1, with the reference's error
    estimate (mean_squared_error.cc:44-64)."""
    Z = batched_observations(op, params, f, bidx, bval, nchain, max(nsteps - 1, 0), seed, **sampler_kw)
    running = np.cumsum(Z, axis=1) / np.arange(1, Z.shape[1] + 1)
    se = (running - mean_exact) ** 2
    mse = se.mean(0)
    mse_error = ((se ** 2).mean(0) - mse ** 2) / (nchain - 1.0)
    return {"mse": mse, "mse_error": mse_error, "nchain": nchain, "nsteps": nsteps}
