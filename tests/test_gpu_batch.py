"""Batched independent chains (mgmc_batch_*): a chain stepped inside a batch
follows exactly the chain it follows when stepped alone (same Philox
streams, same kernels; the coarse cooperative sweeps only change their CTA
count, not their arithmetic)."""
import numpy as np
import pytest

import multigridmc_gb300 as M
from problems import posterior

pytestmark = pytest.mark.gpu


def _chains(seed0):
    cfgs = [((16, 16, 16), 10.0, 3), ((24, 24, 24), 3.0, 0), ((32, 32, 32), 50.0, 5), ((16, 16), 10.0, 2)]
    out = []
    for k, (shape, ksq, m) in enumerate(cfgs):
        _, op = posterior(shape, kappa_sq=ksq, m=m, radius=0.1, seed=k + 1)
        nlev = 3
        s = M.MultigridMCSampler(op, M.MultigridParameters(nlevel=nlev), precision=M.FP32_MIXED, seed=seed0 + k)
        f = np.random.default_rng(k).standard_normal(op.n) * 0.1
        s.fix_rhs(f)
        out.append(s)
    return out


def test_batch_equals_individual_chains():
    solo = _chains(100)
    for s in solo:
        s.step(7)
    batched = _chains(100)
    batch = M.MultigridMCBatch(batched)
    batch.step(7)
    batch.synchronize()
    for a, b in zip(solo, batched):
        xa, xb = a.get_state(), b.get_state()
        assert np.all(np.isfinite(xb))
        assert np.array_equal(xa, xb)
    batch.close()


def test_batch_observables():
    chains = _chains(7)
    for s in chains:
        bidx = np.arange(min(10, s.n), dtype=np.int64)
        s.set_observable(bidx, np.ones(len(bidx)), 50)
    batch = M.MultigridMCBatch(chains)
    batch.step(20)
    batch.synchronize()
    for s in chains:
        z = s.read_observations(50)
        assert len(z) == 20 and np.all(np.isfinite(z)) and np.std(z) > 0


def _uneven_chains(seed0, n=32):
    """n FP32-mixed chains alternating between 48^3 cells (5 levels, down to
    3^3 cells) and 96^3 cells (6 levels, down to 3^3 cells), kappa^2
    log-uniform in [1, 100], 0-8 ball measurements, each with its own f."""
    rng = np.random.default_rng(11)
    out = []
    for k in range(n):
        N, nlev = (48, 5) if k % 2 == 0 else (96, 6)
        ksq = float(np.exp(rng.uniform(0.0, np.log(100.0))))
        m = int(rng.integers(0, 9))
        op = M.LinearOperator.shifted_laplace_fd((N, N, N), ksq)
        if m > 0:
            op = op.with_measurements(rng.uniform(0.1, 0.9, size=(m, 3)), np.ones(m), 1e-4, 0.05)
        s = M.MultigridMCSampler(op, M.MultigridParameters(nlevel=nlev), precision=M.FP32_MIXED, seed=seed0 + k)
        s.fix_rhs(rng.standard_normal(op.n) * 0.1)
        bidx, bval = M.measurement_vector((N, N, N), [0.5, 0.5, 0.5], 0.1)
        s.set_observable(bidx, bval, 16)
        out.append(s)
    return out


def test_batched_kernels_equal_individual_chains():
    """32 chains of uneven depth (48^3 and 96^3) step through the batched
    kernels -- one launch per kernel of the step for all chains of a lattice
    size -- and every state and observable equals, bit for bit, the same
    chain stepped alone."""
    solo = _uneven_chains(500)
    for s in solo:
        s.step(5)
    chains = _uneven_chains(500)
    batch = M.MultigridMCBatch(chains)
    ngroups, ngrouped = batch.groups
    assert ngroups == 2 and ngrouped == 32, batch.groups
    batch.step(5)
    batch.synchronize()
    for k, (a, b) in enumerate(zip(solo, chains)):
        xa, xb = a.get_state(), b.get_state()
        assert np.all(np.isfinite(xb))
        assert np.array_equal(xa, xb), f"chain {k}: max |diff| {np.abs(xa - xb).max():.3e}"
        za, zb = a.read_observations(16), b.read_observations(16)
        assert len(zb) == 5 and np.array_equal(za, zb), f"chain {k} observables"
    batch.close()
    for s in solo + chains:
        s.close()
