"""Adjoint of an MGMC step with its noise held fixed (no counterpart in the
reference): the transpose identity on every configuration the sampler
supports, pathwise gradients of a chain functional with respect to the
measurement values against central finite differences, and a checkpointed
torch.autograd.Function (test-only wrapper) over a longer chain."""
import numpy as np
import pytest

import multigridmc_gb300 as M
from problems import operator_1d, posterior

pytestmark = pytest.mark.gpu


def _mg(nlevel, omega=1.0, cycle=1, smoother="SSOR", coarse="Cholesky"):
    return M.MultigridParameters(nlevel=nlevel, smoother=smoother, coarse_solver=coarse, omega=omega, cycle=cycle)


def _sampler(op, prm, ordering=M.MULTICOLOUR, precision=M.FP64):
    return M.MultigridMCSampler(op, prm, ordering=ordering, precision=precision, noise=M.INJECTED)


CASES = [
    ("1d-lowrank", lambda: operator_1d(True)[1], _mg(3)),
    ("2d-post-16-one-level-ssor", lambda: posterior((16, 16), m=3, radius=0.1)[1], _mg(1, coarse="SSOR")),
    ("1d-lowrank-sor-w", lambda: operator_1d(True)[1], _mg(3, omega=0.8, cycle=2, smoother="SOR")),
    ("2d-post-32", lambda: posterior((32, 32), m=4, radius=0.1)[1], _mg(4, omega=1.2)),
    ("3d-post-16", lambda: posterior((16, 16, 16), m=8)[1], _mg(3)),
    ("3d-post-16-coarse-ssor", lambda: posterior((16, 16, 16), m=4)[1], _mg(3, coarse="SSOR")),
    ("3d-post-32", lambda: posterior((32, 32, 32), m=16)[1], _mg(4)),
]


@pytest.mark.parametrize("name,mk,prm", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("ordering", [M.LEXICOGRAPHIC, M.MULTICOLOUR], ids=["lex", "multicolour"])
def test_adjoint_transpose_identity(name, mk, prm, ordering):
    """<Phi u + K f, v> = <u, Phi^T v> + <f, K^T v> for the noise-free step
    (zero noise injected), FP64, to rounding."""
    op = mk()
    s = _sampler(op, prm, ordering)
    rng = np.random.default_rng(3)
    u, f, v = (rng.standard_normal(op.n) for _ in range(3))
    s.inject_noise(np.zeros(s.noise_per_step))
    x = u.copy()
    s.apply(f, x)
    xbar, fbar = v.copy(), np.zeros(op.n)
    s.adjoint_step(xbar, fbar)
    lhs = float(x @ v)
    rhs = float(u @ xbar + f @ fbar)
    scale = np.linalg.norm(x) * np.linalg.norm(v)
    assert abs(lhs - rhs) <= 1e-12 * scale, f"{name}: {lhs} vs {rhs}"
    s.close()


def _subcube_mask(shape):
    """Vertices of the sub-cube [0.25, 0.75]^d (vertex i at (i + 1) / cells)."""
    axes = [((np.arange(c - 1) + 1.0) / c) for c in shape]
    grids = np.meshgrid(*axes[::-1], indexing="ij")  # slowest first; x fastest in the flat order
    inside = np.ones(grids[0].shape, bool)
    for g in grids:
        inside &= (g >= 0.25) & (g <= 0.75)
    return inside.reshape(-1).astype(np.float64)


class Chain:
    """J(y) = (1/T) sum_t ||x_t restricted to the sub-cube||^2 over T steps
    from x_0 = 0 with injected (fixed) noise and f = B Sigma^{-1} y."""

    def __init__(self, op, prm, nsteps, seed=11):
        self.op, self.T = op, nsteps
        self.s = _sampler(op, prm)
        self.nps = self.s.noise_per_step
        self.noise = np.random.default_rng(seed).standard_normal(nsteps * self.nps)
        self.B = op.B_dense()
        self.mask = _subcube_mask(op.shape)

    def f_of(self, y):
        return self.B @ (np.asarray(y, np.float64) / self.op.Sigma)

    def run(self, y, t0=0, t1=None, x0=None):
        """States x_{t0+1} .. x_{t1} from x_{t0} (default: the whole chain)."""
        t1 = self.T if t1 is None else t1
        f = self.f_of(y)
        x = np.zeros(self.op.n) if x0 is None else x0.copy()
        out = []
        for t in range(t0, t1):
            self.s.inject_noise(self.noise[t * self.nps:(t + 1) * self.nps])
            self.s.apply(f, x)
            out.append(x.copy())
        return out

    def J(self, y):
        return sum(float((self.mask * xt) @ xt) for xt in self.run(y)) / self.T

    def grad(self, y):
        xs = self.run(y)
        lam = (2.0 / self.T) * self.mask * xs[-1]
        fbar = np.zeros(self.op.n)
        for t in range(self.T - 1, -1, -1):  # lam = adjoint of x_{t+1}
            self.s.adjoint_step(lam, fbar)
            if t >= 1:
                lam += (2.0 / self.T) * self.mask * xs[t - 1]
        return (self.B.T @ fbar) / self.op.Sigma


def test_gradient_matches_finite_differences():
    """dJ/dy by the adjoint against central differences of the FP64 chain
    (step 1e-6 relative), within 1e-5 relative."""
    _, op = posterior((16, 16, 16), m=6)
    ch = Chain(op, _mg(3), nsteps=12)
    y = np.random.default_rng(5).standard_normal(op.m)
    g = ch.grad(y)
    for k in range(op.m):
        h = 1e-6 * max(1.0, abs(y[k]))
        yp, ym = y.copy(), y.copy()
        yp[k] += h
        ym[k] -= h
        fd = (ch.J(yp) - ch.J(ym)) / (2 * h)
        assert abs(g[k] - fd) <= 1e-5 * max(abs(fd), 1e-3 * np.abs(g).max()), f"y[{k}]: adjoint {g[k]} vs FD {fd}"


def test_checkpointed_autograd_function():
    """A torch.autograd.Function over a 40-step chain that keeps only every
    10th state and recomputes each segment in the backward pass gives the
    gradient of the full-storage adjoint loop."""
    torch = pytest.importorskip("torch")
    _, op = posterior((16, 16, 16), m=4)
    ch = Chain(op, _mg(3), nsteps=40)
    every = 10

    class ChainJ(torch.autograd.Function):
        @staticmethod
        def forward(ctx, y):
            yv = y.detach().numpy()
            x = np.zeros(op.n)
            checkpoints, J = {0: x.copy()}, 0.0
            for t0 in range(0, ch.T, every):
                seg = ch.run(yv, t0, min(ch.T, t0 + every), x)
                J += sum(float((ch.mask * xt) @ xt) for xt in seg)
                x = seg[-1]
                checkpoints[t0 + len(seg)] = x.copy()
            ctx.y, ctx.cp = yv, checkpoints
            return torch.tensor(J / ch.T, dtype=torch.float64)

        @staticmethod
        def backward(ctx, gJ):
            lam = np.zeros(op.n)
            fbar = np.zeros(op.n)
            starts = list(range(0, ch.T, every))
            for t0 in reversed(starts):
                t1 = min(ch.T, t0 + every)
                seg = ch.run(ctx.y, t0, t1, ctx.cp[t0])  # x_{t0+1} .. x_{t1}
                for i in range(len(seg) - 1, -1, -1):
                    lam += (2.0 / ch.T) * ch.mask * seg[i]  # dJ/dx_{t0+i+1}
                    ch.s.adjoint_step(lam, fbar)           # -> adjoint of x_{t0+i}
            g = (ch.B.T @ fbar) / op.Sigma
            return gJ * torch.from_numpy(g)

    y = torch.from_numpy(np.random.default_rng(9).standard_normal(op.m)).requires_grad_(True)
    J = ChainJ.apply(y)
    (gy,) = torch.autograd.grad(J, y)
    assert abs(J.item() - ch.J(y.detach().numpy())) <= 1e-12 * abs(J.item())
    ref = ch.grad(y.detach().numpy())
    assert np.allclose(gy.numpy(), ref, rtol=1e-10, atol=1e-14 * np.abs(ref).max())


# ------------------------------------------------- parameter derivatives
class ParamChain:
    """J(kappa^2, log Sigma, y) = (1/T) sum_t ||x_t on the sub-cube||^2 over
    T steps from x_0 = 0 with f = B Sigma^{-1} y, for the FD prior with the
    measurement columns of `locs` (fixed B), injected noise fixed by seed or
    Philox noise fixed by the sampler seed."""

    def __init__(self, shape, locs, prm, nsteps, kappa_sq=10.0, variance=1e-3, radius=0.1, ordering=M.MULTICOLOUR,
                 precision=M.FP64, noise=M.INJECTED, seed=11):
        self.shape, self.prm, self.T = tuple(shape), prm, nsteps
        self.ordering, self.precision, self.noise, self.seed = ordering, precision, noise, seed
        self.cols = [M.measurement_vector(self.shape, x0, radius) for x0 in locs]
        self.m = len(self.cols)
        self.theta0 = (kappa_sq, np.full(self.m, np.log(variance)))
        self.y = np.random.default_rng(seed + 1).standard_normal(self.m)
        op = self.op(*self.theta0)
        self.n = op.n
        self.B = op.B_dense()
        self.mask = _subcube_mask(self.shape)
        self.hd = float(np.prod([1.0 / c for c in self.shape]))
        s = self.sampler(op)
        self.nps = s.noise_per_step
        s.close()
        self.normals = np.random.default_rng(seed).standard_normal(nsteps * self.nps)

    def op(self, kappa_sq, logsig):
        return M.LinearOperator.shifted_laplace_fd(self.shape, kappa_sq).with_lowrank(self.cols, np.exp(logsig))

    def sampler(self, op):
        return M.MultigridMCSampler(op, self.prm, ordering=self.ordering, precision=self.precision, noise=self.noise,
                                    seed=self.seed)

    def f_of(self, logsig):
        return self.B @ (self.y / np.exp(logsig))

    def run(self, kappa_sq, logsig):
        s = self.sampler(self.op(kappa_sq, logsig))
        f = self.f_of(logsig)
        x = np.zeros(self.n)
        xs = [x.copy()]
        for t in range(self.T):
            if self.noise == M.INJECTED:
                s.inject_noise(self.normals[t * self.nps:(t + 1) * self.nps])
            s.apply(f, x)
            xs.append(x.copy())
        return s, f, xs

    def J(self, kappa_sq, logsig):
        s, _, xs = self.run(kappa_sq, logsig)
        s.close()
        return sum(float((self.mask * xt) @ xt) for xt in xs[1:]) / self.T

    def grad(self, kappa_sq, logsig):
        """(dJ/dkappa^2, dJ/dlog Sigma, dJ/dy) by the parameter adjoint."""
        s, f, xs = self.run(kappa_sq, logsig)
        lam = (2.0 / self.T) * self.mask * xs[-1]
        fbar = np.zeros(self.n)
        gc, gsig = 0.0, np.zeros(self.m)
        for t in range(self.T - 1, -1, -1):  # lam = adjoint of x_{t+1}
            if self.noise == M.INJECTED:
                s.inject_noise(self.normals[t * self.nps:(t + 1) * self.nps])
            c, g = s.adjoint_params(xs[t], lam, fbar, step_index=t)
            gc += c
            gsig += g
            if t >= 1:
                lam += (2.0 / self.T) * self.mask * xs[t]
        s.close()
        sig = np.exp(logsig)
        Btf = self.B.T @ fbar
        return self.hd * gc, gsig - Btf * self.y / sig, Btf / sig


def _check_fd(ch, gk, gs):
    """Two checks per parameter: central differences with step 1e-6
    (relative for kappa^2, absolute for log Sigma) within 1e-5 relative, the
    error judged against the larger of |FD| and a tenth of the largest
    gradient entry (the chain's rounding, ~1e-13 relative, divided by the
    step is ~1e-7 of the gradient's scale); and the fourth-order central
    difference with step 1e-4, whose truncation (~1e-16) and rounding
    (~1e-9) errors are both small, within 1e-7 of the gradient's scale."""
    k2, ls = ch.theta0
    scale = max(abs(gk), np.abs(gs).max())

    def J_at(i, t):
        if i < 0:
            return ch.J(k2 * (1.0 + t), ls)
        e = np.zeros(ch.m)
        e[i] = t
        return ch.J(k2, ls + e)

    for i, g in [(-1, gk)] + list(enumerate(gs)):
        unit = k2 if i < 0 else 1.0
        h = 1e-6
        fd2 = (J_at(i, h) - J_at(i, -h)) / (2 * h * unit)
        assert abs(g - fd2) <= 1e-5 * max(abs(fd2), 0.1 * scale), f"parameter {i}: adjoint {g} vs FD {fd2}"
        h = 1e-4
        fd4 = (8 * (J_at(i, h) - J_at(i, -h)) - (J_at(i, 2 * h) - J_at(i, -2 * h))) / (12 * h * unit)
        assert abs(g - fd4) <= 1e-7 * scale, f"parameter {i}: adjoint {g} vs fourth-order FD {fd4}"


_LOCS3 = [(0.3, 0.4, 0.5), (0.6, 0.55, 0.4), (0.45, 0.7, 0.65), (0.5, 0.3, 0.35)]
PARAM_CASES = [
    ("3d-16-ssor", (16, 16, 16), _LOCS3, _mg(3), M.MULTICOLOUR),
    ("3d-16-ssor-lex", (16, 16, 16), _LOCS3[:3], _mg(3), M.LEXICOGRAPHIC),
    ("3d-16-coarse-ssor", (16, 16, 16), _LOCS3[:2], _mg(3, coarse="SSOR"), M.MULTICOLOUR),
    ("2d-32-sor-w", (32, 32), [(0.3, 0.6), (0.7, 0.4), (0.5, 0.5)], _mg(3, omega=1.2, cycle=2, smoother="SOR"),
     M.MULTICOLOUR),
    ("2d-32-ssor-w-lex", (32, 32), [(0.3, 0.6), (0.7, 0.4)], _mg(3, omega=0.9, cycle=2), M.LEXICOGRAPHIC),
    ("2d-16-one-level-ssor", (16, 16), [(0.3, 0.6), (0.7, 0.4)], _mg(1, coarse="SSOR"), M.MULTICOLOUR),
]


@pytest.mark.parametrize("name,shape,locs,prm,ordering", PARAM_CASES, ids=[c[0] for c in PARAM_CASES])
def test_parameter_gradients_match_finite_differences(name, shape, locs, prm, ordering):
    """dJ/dkappa^2 and dJ/dlog Sigma_k (with f = B Sigma^{-1} y following
    Sigma) by the parameter adjoint against finite differences of the FP64
    chain with the same injected noise."""
    ch = ParamChain(shape, locs, prm, nsteps=8, ordering=ordering)
    gk, gs, _ = ch.grad(*ch.theta0)
    _check_fd(ch, gk, gs)


def test_parameter_gradients_philox_noise():
    """The same with in-kernel Philox noise: the adjoint replays each step
    with the noise of its step counter, and the finite differences rebuild
    the sampler with the same seed."""
    ch = ParamChain((16, 16, 16), _LOCS3, _mg(3), nsteps=6, noise=M.PHILOX, seed=21)
    gk, gs, _ = ch.grad(*ch.theta0)
    _check_fd(ch, gk, gs)


def test_measurement_value_gradient_of_parameter_adjoint():
    """The y-gradient of the parameter adjoint equals the plain adjoint's
    (the linear part is the same computation)."""
    ch = ParamChain((16, 16, 16), _LOCS3, _mg(3), nsteps=5)
    _, _, gy = ch.grad(*ch.theta0)
    s, f, xs = ch.run(*ch.theta0)
    lam = (2.0 / ch.T) * ch.mask * xs[-1]
    fbar = np.zeros(ch.n)
    for t in range(ch.T - 1, -1, -1):
        s.adjoint_step(lam, fbar)
        if t >= 1:
            lam += (2.0 / ch.T) * ch.mask * xs[t]
    s.close()
    ref = (ch.B.T @ fbar) / np.exp(ch.theta0[1])
    assert np.allclose(gy, ref, rtol=1e-12, atol=1e-14 * np.abs(ref).max())


def test_fp32_parameter_gradients_against_fp64():
    """FP32-mixed parameter gradients against the FP64 ones of the coupled
    chain (Philox noise, same seed), within 1e-3 relative."""
    kw = dict(shape=(16, 16, 16), locs=_LOCS3, prm=_mg(3), nsteps=6, noise=M.PHILOX, seed=31)
    g64 = ParamChain(precision=M.FP64, **kw).grad(*ParamChain(**kw).theta0)
    c32 = ParamChain(precision=M.FP32_MIXED, **kw)
    g32 = c32.grad(*c32.theta0)
    for a, b in zip(g32, g64):
        a, b = np.atleast_1d(a), np.atleast_1d(b)
        assert np.linalg.norm(a - b) <= 1e-3 * np.linalg.norm(b)


def test_parameter_gradient_against_oracle_chain():
    """dJ/dkappa^2 against central differences of the oracle's CPU chain (the
    reference algorithm, lexicographic order) with the same injected noise."""
    import oracle as O
    ch = ParamChain((16, 16, 16), _LOCS3[:2], _mg(3), nsteps=6, ordering=M.LEXICOGRAPHIC)
    gk, _, _ = ch.grad(*ch.theta0)
    k2, ls = ch.theta0

    def J_oracle(kappa_sq):
        op = O.Operator.fd(list(ch.shape), kappa_sq)
        op.set_lowrank(ch.B, np.exp(ls))
        src = O.Source(ch.normals)
        s = O.mgmc_sampler(op, src, 3, "SSOR", "Cholesky", ordering=0)
        f = ch.f_of(ls)
        x = np.zeros(ch.n)
        J = 0.0
        for _ in range(ch.T):
            s.apply(f, x)
            J += float((ch.mask * x) @ x)
        return J / ch.T

    dk = 1e-6 * k2
    fd = (J_oracle(k2 + dk) - J_oracle(k2 - dk)) / (2 * dk)
    assert abs(gk - fd) <= 1e-5 * abs(fd)
