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
