"""Driver configurations in libconfig syntax (src/auxilliary/parameters.cc)
become the operator, right hand side and multigrid parameters of the GPU
sampler."""
import os

import numpy as np
import pytest

import multigridmc_gb300 as M
import oracle as O
from multigridmc_gb300.config import load_run, parse_libconfig

PARAMS = """
// a driver configuration
general = {
    dim = 2;
    do_cholesky = false;  do_ssor = true;  do_multigridmc = true;
    measure_time_per_sample = true;
    operator = "posterior";
}
lattice = { nx = 32; ny = 16; nz = 8; }
smoother = { nsmooth = 1; omega = 1.0; }
multigrid = {
    smoother = "SSOR"; coarse_solver = "Cholesky";
    npresmooth = 1; npostsmooth = 2; ncoarsesmooth = 1;
    omega = 1.2; nlevel = 3; cycle = 2; coarse_scaling = 1.0; verbose = 2;
}
sampling = { timeseries = { nsamples = 100; nwarmup = 10; }
             convergence = { nthreads = 2; nsteps = 4; nsamples = 8; } }
prior = { pdemodel = "shiftedlaplace_fd"; correlationlengthmodel = "constant"; }
constantcorrelationlengthmodel = { Lambda = 0.25; }
/* measurements */
measurements = {
    radius = 0.1;
    sample_location = [0.5, 0.5];
    variance_scaling = 1.E-2;
    measure_global = true;
    mean_global = 1.5;
    variance_global = 0.01;
    filename = "meas.cfg";
}
"""

MEAS = """
dim = 2;
n = 3;
measurement_locations = [0.25, 0.3, 0.6, 0.7, 0.8, 0.2];
mean = [1.0, -2.0, 0.5];
variance = [1e-4, 2e-4, 1.5e-4];
"""


def test_parse_libconfig_syntax():
    r = parse_libconfig('a = 1; b = -2.5e-3; c = "x\\ty"; d = true; g = { h = [1, 2.0]; i = (3, "s"); }; # c\n')
    assert r == {"a": 1, "b": -2.5e-3, "c": "x\ty", "d": True, "g": {"h": [1, 2.0], "i": [3, "s"]}}


def test_run_config_builds_the_posterior(tmp_path):
    (tmp_path / "params.cfg").write_text(PARAMS)
    (tmp_path / "meas.cfg").write_text(MEAS)
    cfg = load_run(str(tmp_path / "params.cfg"))
    assert cfg.shape == (32, 16) and cfg.operator == "posterior"
    assert cfg.kappa_sq == pytest.approx(16.0)
    prm = cfg.multigrid_parameters()
    assert (prm.nlevel, prm.npostsmooth, prm.cycle, prm.omega) == (3, 2, 2, 1.2)
    op = cfg.linear_operator()
    assert op.m == 4  # three balls and the global average
    np.testing.assert_allclose(op.Sigma, [1e-6, 2e-6, 1.5e-6, 0.01])
    ref = M.LinearOperator.shifted_laplace_fd((32, 16), 16.0).with_measurements(
        [[0.25, 0.3], [0.6, 0.7], [0.8, 0.2]], [1e-4, 2e-4, 1.5e-4], variance_scaling=1e-2, radius=0.1,
        measure_global=True, variance_global=0.01)
    assert np.array_equal(op.B_idx, ref.B_idx) and np.allclose(op.B_val, ref.B_val)
    f = cfg.rhs(op)
    y = np.array([1.0, -2.0, 0.5, 1.5])
    np.testing.assert_allclose(f, op.B_dense() @ (y / op.Sigma), rtol=1e-12)
    assert cfg.sample_location() == [0.5, 0.5]


def test_periodic_correlation_length(tmp_path):
    """prior.correlationlengthmodel = "periodic" (parameters.cc:236-256)
    gives the FD prior with the per-vertex diagonal of the periodic model."""
    text = PARAMS.replace('correlationlengthmodel = "constant"', 'correlationlengthmodel = "periodic"').replace(
        'operator = "posterior"', 'operator = "prior"') + \
        "periodiccorrelationlengthmodel = { Lambda_min = 0.12; Lambda_max = 0.23; };\n"
    (tmp_path / "params.cfg").write_text(text)
    cfg = load_run(str(tmp_path / "params.cfg"))
    assert cfg.correlation == "periodic" and (cfg.Lambda_min, cfg.Lambda_max) == (0.12, 0.23)
    op = cfg.linear_operator()
    ref = M.LinearOperator.shifted_laplace_fd_periodic((32, 16), 0.12, 0.23)
    assert np.array_equal(op.centre, ref.centre) and np.array_equal(op.stencil, ref.stencil)
    with pytest.raises(ValueError):
        cfg.kappa_sq


def test_fem_prior(tmp_path):
    """prior.pdemodel = "shiftedlaplace_fem" gives the FEM operator
    (constant or periodic correlation length)."""
    text = PARAMS.replace('pdemodel = "shiftedlaplace_fd"', 'pdemodel = "shiftedlaplace_fem"').replace(
        'operator = "posterior"', 'operator = "prior"')
    (tmp_path / "params.cfg").write_text(text)
    op = load_run(str(tmp_path / "params.cfg")).linear_operator()
    ref = M.LinearOperator.shifted_laplace_fem((32, 16), 16.0)
    assert np.array_equal(op.stencil, ref.stencil) and op.field is None
    text = text.replace('correlationlengthmodel = "constant"', 'correlationlengthmodel = "periodic"') + \
        "periodiccorrelationlengthmodel = { Lambda_min = 0.12; Lambda_max = 0.23; };\n"
    (tmp_path / "params.cfg").write_text(text)
    op = load_run(str(tmp_path / "params.cfg")).linear_operator()
    ref = M.LinearOperator.shifted_laplace_fem_periodic((32, 16), 0.12, 0.23)
    assert np.array_equal(op.field, ref.field)


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _template():
    return load_run(os.path.join(GOLDEN, "parameters_template.cfg"))


def test_reference_templates_parse():
    """The reference's own parameters_template.cfg and the measurement file
    it names (copies in tests/golden/, made by make_fixtures.py) give the run
    the reference's driver would set up: 2D posterior on 32^2 cells,
    Lambda = 0.2, eight point measurements (radius 0: nearest vertex), a
    W-cycle with SOR smoother and SSOR coarse solver on 4 levels."""
    cfg = _template()
    assert cfg.dim == 2 and cfg.shape == (32, 32) and cfg.operator == "posterior"
    assert cfg.pdemodel == "shiftedlaplace_fd" and cfg.correlation == "constant"
    assert cfg.kappa_sq == pytest.approx(25.0)
    prm = cfg.multigrid_parameters()
    assert (prm.smoother, prm.coarse_solver, prm.nlevel, prm.cycle) == ("SOR", "SSOR", 4, 2)
    assert (prm.npresmooth, prm.npostsmooth, prm.ncoarsesmooth, prm.omega, prm.coarse_scaling) == (1, 1, 1, 1.0, 1.0)
    assert cfg.sampling["timeseries"] == {"nsamples": 10000, "nwarmup": 1000}
    assert cfg.sampling["convergence"]["nthreads"] == 6
    assert cfg.sample_location() == [0.5, 0.5]
    md = cfg.measurement_data
    assert md["n"] == 8 and len(md["measurement_locations"]) == 16 and len(md["mean"]) == 8


def test_reference_template_operator_equals_oracle():
    """The template's posterior (FD prior, kappa^2 = 25, nearest-vertex
    measurements, Sigma = variance) equals the oracle's MeasuredOperator
    built from the same numbers: B bit for bit, A x to 1e-14."""
    cfg = _template()
    op = cfg.linear_operator()
    md = cfg.measurement_data
    loc = np.asarray(md["measurement_locations"], np.float64).reshape(8, 2)
    op_o = O.Operator.fd([32, 32], 25.0)
    op_o.add_measurements(loc, np.asarray(md["variance"], np.float64), variance_scaling=1.0, radius=0.0)
    assert op.m == 8 and op_o.m == 8
    Bo, sig_o = op_o.B_dense()
    assert np.array_equal(op.B_dense(), Bo) and np.array_equal(op.Sigma, sig_o)
    np.testing.assert_array_equal(op.Sigma, np.asarray(md["variance"], np.float64))
    x = np.random.default_rng(3).standard_normal(op.n)
    B = op.B_dense()
    y = M.LinearOperator(op.shape, op.stencil).to_scipy() @ x + B @ ((B.T @ x) / op.Sigma)
    want = op_o.apply(x)
    assert np.linalg.norm(y - want) <= 1e-14 * np.linalg.norm(want)
    f = cfg.rhs(op)
    np.testing.assert_allclose(f, B @ (np.asarray(md["mean"]) / op.Sigma), rtol=1e-14)


@pytest.mark.gpu
@pytest.mark.parametrize("ordering", [M.LEXICOGRAPHIC, M.MULTICOLOUR], ids=["lex", "multicolour"])
def test_reference_template_chain_equals_oracle(ordering):
    """MGMC as the template configures it (SOR smoother, SSOR coarse solver,
    W-cycle, 4 levels) on the template's posterior: the FP64 GPU chain
    against the oracle's on the same injected noise, 100 steps.

    The template's point measurements have Sigma ~ 1.2e-6, so f = B Sigma^-1 y
    reaches 3.4e6 at the measured vertices against states of order 4: every
    sweep's value there cancels from ~1e6 down to O(1), and a rounding
    difference of one ulp anywhere in f moves the chain by ~3e-12 relative
    (measured below on the oracle itself).  The GPU's solve-form low-rank
    correction and the oracle's explicit Bbar = M^-1 B S^-1 round
    differently, so the bound is 100 such one-ulp perturbations instead of
    the 1e-12 of the well-conditioned configurations (Sigma = 1e-4,
    ball averages)."""
    cfg = _template()
    op = cfg.linear_operator()
    prm = cfg.multigrid_parameters()
    md = cfg.measurement_data
    op_o = O.Operator.fd([32, 32], 25.0)
    op_o.add_measurements(np.asarray(md["measurement_locations"], np.float64).reshape(8, 2),
                          np.asarray(md["variance"], np.float64), variance_scaling=1.0, radius=0.0)
    gpu = M.MultigridMCSampler(op, prm, ordering=ordering, precision=M.FP64, noise=M.INJECTED)
    nps = gpu.noise_per_step
    nsteps = 100
    noise = O.CLCG().draw_normal(nps * nsteps)
    src = O.Source(noise)
    orc = O.mgmc_sampler(op_o, src, prm.nlevel, smoother=prm.smoother, coarse_solver=prm.coarse_solver,
                         npresmooth=prm.npresmooth, npostsmooth=prm.npostsmooth, ncoarsesmooth=prm.ncoarsesmooth,
                         omega=prm.omega, cycle=prm.cycle, coarse_scaling=prm.coarse_scaling, ordering=ordering)
    f = cfg.rhs(op)
    # sensitivity of the oracle's chain to a one-ulp change of f
    orc2 = O.mgmc_sampler(op_o, O.Source(noise), prm.nlevel, smoother=prm.smoother,
                          coarse_solver=prm.coarse_solver, npresmooth=prm.npresmooth, npostsmooth=prm.npostsmooth,
                          ncoarsesmooth=prm.ncoarsesmooth, omega=prm.omega, cycle=prm.cycle,
                          coarse_scaling=prm.coarse_scaling, ordering=ordering)
    f_ulp = np.nextafter(f, np.inf)
    xo, xg, xu = np.zeros(op.n), np.zeros(op.n), np.zeros(op.n)
    gpu.inject_noise(noise)
    worst, ulp = 0.0, 0.0
    for _ in range(nsteps):
        orc.apply(f, xo)
        orc2.apply(f_ulp, xu)
        gpu.apply(f, xg)
        worst = max(worst, np.linalg.norm(xg - xo) / np.linalg.norm(xo))
        ulp = max(ulp, np.linalg.norm(xu - xo) / np.linalg.norm(xo))
    assert src.position == nps * nsteps
    assert 0.0 < ulp < 1e-11, ulp
    assert worst < 100.0 * ulp, (worst, ulp)
    gpu.close()
