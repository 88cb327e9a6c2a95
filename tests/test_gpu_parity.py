"""Pathwise parity of the GB300 sampler with the CPU oracle.

Both chains consume the same injected N(0,1) stream (the reference's CLCG +
polar-method normals, drawn in the reference's order); the FP64 GPU chain
must stay within 1e-12 relative of the oracle's after every step.  The
lexicographic runs reproduce the reference's sweep order with the wavefront
kernel; the multicolour runs check the throughput kernels against the
oracle run in the same colour order.
"""
import numpy as np
import pytest

import multigridmc_gb300 as M
import oracle as O
from problems import operator_1d, posterior, rhs

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12


def _mg(nlevel, omega=1.0, cycle=1, smoother="SSOR", coarse="Cholesky"):
    return M.MultigridParameters(nlevel=nlevel, smoother=smoother, coarse_solver=coarse, omega=omega, cycle=cycle)


def _run_parity(op_o, op_p, prm, ordering, nsteps, precision=M.FP64):
    gpu = M.MultigridMCSampler(op_p, prm, ordering=ordering, precision=precision, noise=M.INJECTED)
    nps = gpu.noise_per_step
    noise = O.CLCG().draw_normal(nps * nsteps)
    src = O.Source(noise)
    orc = O.mgmc_sampler(op_o, src, prm.nlevel, smoother=prm.smoother, coarse_solver=prm.coarse_solver,
                         npresmooth=prm.npresmooth, npostsmooth=prm.npostsmooth, ncoarsesmooth=prm.ncoarsesmooth,
                         omega=prm.omega, cycle=prm.cycle, coarse_scaling=prm.coarse_scaling, ordering=ordering)
    f = rhs(op_p)
    xo = np.zeros(op_p.n)
    xg = np.zeros(op_p.n)
    worst = 0.0
    for k in range(nsteps):
        orc.apply(f, xo)
        gpu.inject_noise(noise[k * nps:(k + 1) * nps])
        gpu.apply(f, xg)
        err = np.linalg.norm(xg - xo) / np.linalg.norm(xo)
        worst = max(worst, err)
    assert src.position == nps * nsteps, "GPU and oracle consume different numbers of normals per step"
    return worst


def _run_parity_streamed(op_o, op_p, prm, ordering, nsteps):
    """_run_parity for chains whose noise does not fit in memory at once
    (about 1.2e6 normals per step at 64^3, 9.5e6 at 128^3): the oracle draws from its own
    CLCG (the reference's generator, seed 1), the GPU chain is fed each
    step's normals from a second CLCG with the same seed, so both consume the
    same stream in the same order."""
    gpu = M.MultigridMCSampler(op_p, prm, ordering=ordering, precision=M.FP64, noise=M.INJECTED)
    nps = gpu.noise_per_step
    gen = O.CLCG()
    orc = O.mgmc_sampler(op_o, O.Source(), prm.nlevel, smoother=prm.smoother, coarse_solver=prm.coarse_solver,
                         npresmooth=prm.npresmooth, npostsmooth=prm.npostsmooth, ncoarsesmooth=prm.ncoarsesmooth,
                         omega=prm.omega, cycle=prm.cycle, coarse_scaling=prm.coarse_scaling, ordering=ordering)
    f = rhs(op_p)
    xo = np.zeros(op_p.n)
    xg = np.zeros(op_p.n)
    worst = 0.0
    for _ in range(nsteps):
        orc.apply(f, xo)
        gpu.inject_noise(gen.draw_normal(nps))
        gpu.apply(f, xg)
        worst = max(worst, np.linalg.norm(xg - xo) / np.linalg.norm(xo))
    gpu.close()
    return worst


CASES = [
    ("1d", lambda: operator_1d(False), _mg(3)),
    ("1d-lowrank", lambda: operator_1d(True), _mg(3)),
    ("1d-lowrank-sor-w", lambda: operator_1d(True), _mg(3, omega=0.8, cycle=2, smoother="SOR")),
    ("2d-prior-16", lambda: posterior((16, 16)), _mg(3)),
    ("2d-prior-64-config1", lambda: posterior((64, 64)), _mg(4)),
    ("2d-post-32", lambda: posterior((32, 32), m=4, radius=0.1), _mg(4, omega=1.2)),
    ("3d-post-16", lambda: posterior((16, 16, 16), m=8), _mg(3)),
    ("3d-post-16-coarse-ssor", lambda: posterior((16, 16, 16), m=4), _mg(3, coarse="SSOR")),
    ("3d-post-32", lambda: posterior((32, 32, 32), m=16), _mg(4)),
]


@pytest.mark.parametrize("name,mk,prm", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("ordering", [M.LEXICOGRAPHIC, M.MULTICOLOUR], ids=["lex", "multicolour"])
def test_chain_parity_fp64(name, mk, prm, ordering):
    op_o, op_p = mk()
    worst = _run_parity(op_o, op_p, prm, ordering, 100)
    assert worst < TOL_FP64, f"{name}: max relative deviation {worst:.3e}"


def test_chain_parity_many_measurements():
    """More than 64 measurement columns: the m x m low-rank system is formed
    by the general solve (S^{-1} columns loaded in batches, not the
    preloaded slice of m <= 64), in FP64 against the oracle after each of 50
    steps and in the FP32-mixed chain's float-float arithmetic within FP32
    rounding."""
    op_o, op_p = posterior((16, 16, 16), m=80, radius=0.1)
    worst = _run_parity(op_o, op_p, _mg(3), M.MULTICOLOUR, 50)
    assert worst < TOL_FP64, f"FP64: max relative deviation {worst:.3e}"
    worst = _run_parity(op_o, op_p, _mg(3), M.MULTICOLOUR, 20, precision=M.FP32_MIXED)
    assert worst < 1e-4, f"FP32-mixed: {worst:.3e}"


@pytest.mark.parametrize("ordering", [M.LEXICOGRAPHIC, M.MULTICOLOUR], ids=["lex", "multicolour"])
def test_chain_parity_64cubed(ordering):
    """The 64^3 posterior with 32 measurements, five levels: FP64 chain
    against the oracle after each of 100 steps, in the reference's
    lexicographic order (hyperplane wavefront) and in multicolour order."""
    op_o, op_p = posterior((64, 64, 64), m=32)
    worst = _run_parity_streamed(op_o, op_p, _mg(5), ordering, 100)
    assert worst < TOL_FP64, f"max relative deviation {worst:.3e}"


@pytest.mark.parametrize("ordering", [M.LEXICOGRAPHIC, M.MULTICOLOUR], ids=["lex", "multicolour"])
def test_chain_parity_128cubed(ordering):
    """The 128^3 posterior with 32 measurements (kappa^2 = 10, radius 0.05,
    Sigma = 1e-4; five levels down to 8^3 cells, coarse Cholesky): FP64
    chain against the oracle after each of 100 steps, in the reference's
    lexicographic order and in multicolour order."""
    op_o, op_p = posterior((128, 128, 128), m=32)
    worst = _run_parity_streamed(op_o, op_p, _mg(5), ordering, 100)
    assert worst < TOL_FP64, f"max relative deviation {worst:.3e}"


@pytest.mark.parametrize("name,mk,prm", CASES[3:7], ids=[c[0] for c in CASES[3:7]])
def test_chain_parity_fp32(name, mk, prm):
    """FP32-mixed chain against the FP64 oracle on the same noise: the
    deviation is FP32 rounding, not a different chain."""
    op_o, op_p = mk()
    worst = _run_parity(op_o, op_p, prm, M.MULTICOLOUR, 20, precision=M.FP32_MIXED)
    assert worst < 1e-4, f"{name}: {worst:.3e}"


@pytest.mark.parametrize("shape,m", [((8,), 0), ((16, 16), 3), ((16, 16, 16), 6), ((16, 8, 32), 4)])
def test_building_blocks(shape, m):
    """LinearOperator::apply, restrict, prolongate_add and single SOR sweeps
    on every level against the oracle (coarse levels from its sparse RAP)."""
    op_o, op_p = posterior(shape, m=m, radius=0.1)
    nlev = 3 if len(shape) > 1 else 2
    gpu = M.MultigridMCSampler(op_p, _mg(nlev), ordering=M.LEXICOGRAPHIC, noise=M.INJECTED)
    rng = np.random.default_rng(3)
    ops = [op_o]
    for lev in range(1, nlev):
        ops.append(ops[-1].coarsen())
    for lev in range(nlev):
        oo = ops[lev]
        x = rng.standard_normal(oo.n)
        y_o = oo.apply(x)
        y_g = gpu.level_apply(lev, x)
        assert np.linalg.norm(y_g - y_o) <= 1e-13 * np.linalg.norm(y_o)
        if lev + 1 < nlev:
            xc_o = O.restrict(oo.shape, x)
            xc_g = gpu.restrict(lev, x)
            assert np.linalg.norm(xc_g - xc_o) <= 1e-14 * np.linalg.norm(xc_o)
            xc = rng.standard_normal(ops[lev + 1].n)
            xp_o = x.copy()
            O.prolongate_add(oo.shape, 0.7, xc, xp_o)
            xp_g = gpu.prolongate_add(lev, 0.7, xc, x.copy())
            assert np.linalg.norm(xp_g - xp_o) <= 1e-14 * np.linalg.norm(xp_o)
        # one noise-free forward and backward SOR sweep (SORSmoother::apply)
        f = rng.standard_normal(oo.n)
        for fwd in (True, False):
            xo = x.copy()
            # a sampler fed zero noise is the smoother
            src = O.Source(np.zeros(oo.n + oo.m))
            sm = O.sor_sampler(oo, src, 1.0, forward=fwd)
            sm.apply(f, xo)
            xg = gpu.sor(lev, M.FORWARD if fwd else M.BACKWARD, f, x.copy(), with_noise=False)
            assert np.linalg.norm(xg - xo) <= 1e-12 * np.linalg.norm(xo)


def test_errors_are_status_codes():
    """Odd extents, bad parameters and exhausted noise come back as status
    codes, never as an exit (the reference calls exit(-1))."""
    _, op_p = posterior((10, 10, 10))
    with pytest.raises(M.MGMCError) as e:
        M.MultigridMCSampler(op_p, _mg(3))
    assert e.value.status == 2
    _, op_p = posterior((8, 8, 8))
    with pytest.raises(M.MGMCError) as e:
        M.MultigridMCSampler(op_p, M.MultigridParameters(nlevel=2, omega=2.5))
    assert e.value.status == 1
    gpu = M.MultigridMCSampler(op_p, _mg(2), noise=M.INJECTED)
    x = np.zeros(op_p.n)
    with pytest.raises(M.MGMCError) as e:
        gpu.apply(np.zeros(op_p.n), x)
    assert e.value.status == 6
    # negative kappa^2 large enough to make the coarse matrix indefinite
    op_bad = M.LinearOperator.shifted_laplace_fd((8, 8, 8), kappa_sq=-2000.0)
    with pytest.raises(M.MGMCError) as e:
        M.MultigridMCSampler(op_bad, _mg(2))
    assert e.value.status == 3


def test_autotuned_shapes_do_not_change_the_chain(monkeypatch):
    """The colour passes' CTA shapes chosen by the autotuner leave every
    value of the chain unchanged (FP32-mixed, Philox noise, bitwise)."""
    _, op_p = posterior((32, 32, 32), m=8)
    f = np.random.default_rng(4).standard_normal(op_p.n)
    states = []
    for tune in ("0", "1"):
        monkeypatch.setenv("MGMC_AUTOTUNE", tune)
        s = M.MultigridMCSampler(op_p, _mg(4), ordering=M.MULTICOLOUR, precision=M.FP32_MIXED, seed=5)
        s.fix_rhs(f)
        s.step(5)
        states.append(s.get_state())
        s.close()
    assert np.array_equal(states[0], states[1])


def test_sampler_surface_deep_copy():
    """Sampler::deep_copy / get_linear_operator / unfix_rhs (sampler.hh:40-71):
    a deep copy with the original's seed runs the original's chain bit for bit
    from zero, whatever state the original is in; another seed gives another
    chain; the copy shares the operator and nothing on the device."""
    _, op = posterior((32, 32, 32), m=8)
    f = rhs(op)
    a = M.MultigridMCSampler(op, _mg(4), precision=M.FP32_MIXED, seed=11)
    xa = np.zeros(op.n)
    for _ in range(3):
        a.apply(f, xa)
    b, c = a.deep_copy(11), a.deep_copy(12)
    assert b.get_linear_operator() is op and c.params is a.params
    xb, xc = np.zeros(op.n), np.zeros(op.n)
    for _ in range(3):
        b.apply(f, xb)
        c.apply(f, xc)
    assert np.array_equal(xa, xb)
    assert not np.array_equal(xa, xc)
    a.unfix_rhs()
    a.apply(f, xa)
    assert np.array_equal(b.get_state(), xb)
    for s in (a, b, c):
        s.close()


@pytest.mark.parametrize("ordering", [M.LEXICOGRAPHIC, M.MULTICOLOUR], ids=["lex", "multicolour"])
def test_ssor_smoother(ordering):
    """SSORSmoother::apply (ssor_smoother.cc:9-16) with nsmooth = 2 on the
    fine and the first coarse level of a 2D posterior against the oracle's
    forward / backward SOR sweeps fed zero noise (the smoother), 1e-12."""
    op_o, op_p = posterior((32, 32), m=4, radius=0.1)
    gpu = M.MultigridMCSampler(op_p, _mg(3, omega=1.2), ordering=ordering, noise=M.INJECTED)
    ops = [op_o, op_o.coarsen()]
    rng = np.random.default_rng(5)
    for lev, oo in enumerate(ops):
        b = rng.standard_normal(oo.n)
        x0 = rng.standard_normal(oo.n)
        xo = x0.copy()
        for _ in range(2):
            for fwd in (True, False):
                src = O.Source(np.zeros(oo.n + oo.m))
                O.sor_sampler(oo, src, 1.2, forward=fwd, ordering=ordering).apply(b, xo)
        xg = M.SSORSmoother(gpu, lev, nsmooth=2).apply(b, x0.copy())
        assert np.linalg.norm(xg - xo) <= 1e-12 * np.linalg.norm(xo), lev
    gpu.close()
