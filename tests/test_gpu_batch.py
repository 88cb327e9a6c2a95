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
