"""ctypes front end of the CPU oracle (test infrastructure only).

The oracle restates the reference's sampling path on the CPU; see the header
of ``mgmc_oracle.cc`` for what it follows and how it is pinned.  Only the
tests, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` leg of
``bench.py`` import this package -- the library under test never does.
"""
import ctypes as C

import numpy as np

from . import build as _build

_lib = None

_P = C.c_void_p
_D = C.POINTER(C.c_double)
_I64 = C.POINTER(C.c_int64)
_I32 = C.POINTER(C.c_int32)
_INT = C.POINTER(C.c_int)


def _dp(a):
    return a.ctypes.data_as(_D)


def _ip(a):
    return a.ctypes.data_as(_I64)


def lib():
    """Load (building if needed) the oracle shared library."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build()
    L = C.CDLL(path)
    sig = {
        "orc_lattice_nvertex": (C.c_int64, [C.c_int] * 4),
        "orc_lattice_vertex_euclid": (None, [C.c_int] * 4 + [C.c_int64, _INT]),
        "orc_lattice_vertex_linear": (C.c_int64, [C.c_int] * 4 + [_INT]),
        "orc_lattice_shift_vertex": (C.c_int64, [C.c_int] * 4 + [C.c_int64, _INT]),
        "orc_lattice_cell_euclid": (None, [C.c_int] * 4 + [C.c_int64, _INT]),
        "orc_lattice_cell_linear": (C.c_int64, [C.c_int] * 4 + [_INT]),
        "orc_lattice_fine_vertex_idx": (C.c_int64, [C.c_int] * 4 + [C.c_int64]),
        "orc_lattice_vertex_coordinates": (None, [C.c_int] * 4 + [C.c_int64, _D]),
        "orc_quadrature": (C.c_int, [C.c_int, C.c_int, _D, _D]),
        "orc_fd_stencil": (None, [C.c_int] * 4 + [C.c_double, _D]),
        "orc_stencil_operator": (_P, [C.c_int] * 4 + [_D]),
        "orc_fd_operator": (_P, [C.c_int] * 4 + [C.c_double]),
        "orc_op_destroy": (None, [_P]),
        "orc_op_n": (C.c_int64, [_P]),
        "orc_op_m": (C.c_int, [_P]),
        "orc_op_nnz": (C.c_int64, [_P]),
        "orc_op_get_csr": (None, [_P, _I64, _I64, _D]),
        "orc_op_B_nnz": (C.c_int64, [_P]),
        "orc_op_get_B": (None, [_P, _I64, _I64, _D, _D]),
        "orc_op_set_lowrank": (None, [_P, C.c_int, _I64, _I64, _D, _D]),
        "orc_op_add_measurements": (None, [_P, C.c_int, _D, _D, C.c_double, C.c_double, C.c_int, C.c_double]),
        "orc_measurement_vector": (C.c_int64, [C.c_int] * 4 + [_D, C.c_double, _I64, _D, C.c_int64]),
        "orc_op_apply": (None, [_P, _D, _D]),
        "orc_op_precision": (None, [_P, _D]),
        "orc_op_coarsen": (_P, [_P]),
        "orc_op_coarsenable": (C.c_int, [_P]),
        "orc_restrict": (None, [C.c_int] * 4 + [_D, _D]),
        "orc_prolongate_add": (None, [C.c_int] * 4 + [C.c_double, _D, _D]),
        "orc_rng_create": (_P, [C.c_int, C.c_int]),
        "orc_rng_destroy": (None, [_P]),
        "orc_rng_draw_int": (None, [_P, C.c_int64, _I32]),
        "orc_rng_draw_uniform": (None, [_P, C.c_int64, _D]),
        "orc_rng_draw_normal": (None, [_P, C.c_int64, _D]),
        "orc_source_clcg": (_P, []),
        "orc_source_buffer": (_P, [_D, C.c_int64]),
        "orc_source_position": (C.c_int64, [_P]),
        "orc_source_destroy": (None, [_P]),
        "orc_sor_sampler": (_P, [_P, _P, C.c_double, C.c_int, C.c_int, C.c_int]),
        "orc_ssor_sampler": (_P, [_P, _P, C.c_double, C.c_int, C.c_int]),
        "orc_cholesky_sampler": (_P, [_P, _P]),
        "orc_lowrank_cholesky_sampler": (_P, [_P, _P]),
        "orc_mgmc_sampler": (_P, [_P, _P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                  C.c_double, C.c_int, C.c_double, C.c_int]),
        "orc_sampler_destroy": (None, [_P]),
        "orc_sampler_apply": (C.c_int, [_P, _D, _D, C.c_int]),
        "orc_sampler_observe": (C.c_int, [_P, _D, _D, C.c_int64, C.c_int64, _I64, _D, _D]),
        "orc_sampler_mean_cov": (C.c_int, [_P, C.c_int64, _D, _D, C.c_int64, C.c_int64, _D, _D]),
        "orc_ssor_smoother_apply": (None, [_P, C.c_double, C.c_int, C.c_int, _D, _D]),
        "orc_dense_cholesky": (C.c_int, [_D, C.c_int64]),
        "orc_op_set_diagonal": (None, [_P, _D]),
        "orc_fem_operator": (_P, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double]),
        "orc_mg_create": (_P, [_P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_double, C.c_int,
                               C.c_int]),
        "orc_mg_destroy": (None, [_P]),
        "orc_mg_apply": (None, [_P, _D, _D]),
        "orc_loop_solve": (C.c_int, [_P, _D, _D, C.c_double, C.c_double, C.c_int, _D, _INT]),
        "orc_cholesky_solve": (C.c_int, [_P, _D, _D]),
        "orc_stats_create": (_P, [C.c_int, C.c_uint]),
        "orc_stats_destroy": (None, [_P]),
        "orc_stats_record": (None, [_P, _D, C.c_int64]),
        "orc_stats_average": (None, [_P, _D]),
        "orc_stats_covariance": (None, [_P, _D]),
        "orc_stats_autocov": (C.c_int, [_P, _D]),
        "orc_stats_tau_int": (C.c_double, [_P, _D]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _dims(dim, shape):
    s = list(shape) + [2] * (3 - len(shape))
    return [dim, int(s[0]), int(s[1]), int(s[2])]


# ---------------------------------------------------------------- lattice
class Lattice:
    """Reference Lattice{1,2,3}d index maps (lattice{1,2,3}d.hh)."""

    def __init__(self, *shape):
        self.shape = tuple(int(s) for s in shape)
        self.dim = len(shape)
        self._a = _dims(self.dim, self.shape)

    @property
    def nvertex(self):
        return lib().orc_lattice_nvertex(*self._a)

    def vertexidx_linear2euclidean(self, ell):
        out = (C.c_int * 3)()
        lib().orc_lattice_vertex_euclid(*self._a, ell, out)
        return tuple(out[: self.dim])

    def vertexidx_euclidean2linear(self, idx):
        a = (C.c_int * 3)(*idx)
        return lib().orc_lattice_vertex_linear(*self._a, a)

    def shift_vertexidx(self, ell, shift):
        a = (C.c_int * 3)(*shift)
        return lib().orc_lattice_shift_vertex(*self._a, ell, a)

    def cellidx_linear2euclidean(self, ell):
        out = (C.c_int * 3)()
        lib().orc_lattice_cell_euclid(*self._a, ell, out)
        return tuple(out[: self.dim])

    def cellidx_euclidean2linear(self, idx):
        a = (C.c_int * 3)(*idx)
        return lib().orc_lattice_cell_linear(*self._a, a)

    def fine_vertex_idx(self, ell):
        return lib().orc_lattice_fine_vertex_idx(*self._a, ell)

    def vertex_coordinates(self, ell):
        out = (C.c_double * 3)()
        lib().orc_lattice_vertex_coordinates(*self._a, ell, out)
        return tuple(out[: self.dim])

    def coarse(self):
        return Lattice(*[s // 2 for s in self.shape])


def quadrature(dim, order):
    npts = (order + 1) ** dim
    w = np.zeros(npts)
    p = np.zeros((npts, dim))
    lib().orc_quadrature(dim, order, _dp(w), _dp(p))
    return w, p


def fd_stencil(shape, kappa_sq):
    st = np.zeros(27)
    lib().orc_fd_stencil(*_dims(len(shape), shape), kappa_sq, _dp(st))
    return st


def measurement_vector(shape, x0, radius):
    dim = len(shape)
    x0 = np.ascontiguousarray(x0, dtype=np.float64)
    n = lib().orc_measurement_vector(*_dims(dim, shape), _dp(x0), radius, None, None, 0)
    idx = np.zeros(n, dtype=np.int64)
    val = np.zeros(n)
    lib().orc_measurement_vector(*_dims(dim, shape), _dp(x0), radius, _ip(idx), _dp(val), n)
    return idx, val


def restrict(shape, x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    nc = Lattice(*[s // 2 for s in shape]).nvertex
    xc = np.zeros(nc)
    lib().orc_restrict(*_dims(len(shape), shape), _dp(x), _dp(xc))
    return xc


def prolongate_add(shape, alpha, xc, x):
    xc = np.ascontiguousarray(xc, dtype=np.float64)
    lib().orc_prolongate_add(*_dims(len(shape), shape), alpha, _dp(xc), _dp(x))


# --------------------------------------------------------------- operators
class Operator:
    """LinearOperator A = A_0 + B Sigma^{-1} B^T on a lattice."""

    def __init__(self, handle, shape):
        self.h = handle
        self.shape = tuple(shape)
        self.dim = len(shape)

    @classmethod
    def fd(cls, shape, kappa_sq):
        return cls(lib().orc_fd_operator(*_dims(len(shape), shape), kappa_sq), shape)

    @classmethod
    def fem(cls, shape, model, p0, p1=0.0):
        """ShiftedLaplaceFEMOperator: model 0 constant kappa^2 = p0, model 1
        periodic correlation length (Lambda_min, Lambda_max)."""
        dim, nx, ny, nz = _dims(len(shape), shape)
        return cls(lib().orc_fem_operator(dim, nx, ny, nz, int(model), float(p0), float(p1)), shape)

    @classmethod
    def from_stencil(cls, shape, stencil27):
        st = np.ascontiguousarray(stencil27, dtype=np.float64)
        return cls(lib().orc_stencil_operator(*_dims(len(shape), shape), _dp(st)), shape)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_op_destroy(self.h)
            self.h = None

    @property
    def n(self):
        return lib().orc_op_n(self.h)

    @property
    def m(self):
        return lib().orc_op_m(self.h)

    def csr(self):
        n, nnz = self.n, lib().orc_op_nnz(self.h)
        ptr = np.zeros(n + 1, np.int64)
        col = np.zeros(nnz, np.int64)
        val = np.zeros(nnz)
        lib().orc_op_get_csr(self.h, _ip(ptr), _ip(col), _dp(val))
        return ptr, col, val

    def dense(self):
        ptr, col, val = self.csr()
        A = np.zeros((self.n, self.n))
        for i in range(self.n):
            A[i, col[ptr[i]:ptr[i + 1]]] = val[ptr[i]:ptr[i + 1]]
        return A

    def B(self):
        m, nnz = self.m, lib().orc_op_B_nnz(self.h)
        ptr = np.zeros(m + 1, np.int64)
        row = np.zeros(nnz, np.int64)
        val = np.zeros(nnz)
        sig = np.zeros(m)
        lib().orc_op_get_B(self.h, _ip(ptr), _ip(row), _dp(val), _dp(sig))
        return ptr, row, val, sig

    def B_dense(self):
        ptr, row, val, sig = self.B()
        Bd = np.zeros((self.n, self.m))
        for j in range(self.m):
            Bd[row[ptr[j]:ptr[j + 1]], j] = val[ptr[j]:ptr[j + 1]]
        return Bd, sig

    def set_diagonal(self, diag):
        """Per-vertex diagonal of A_0 (variable-coefficient FD prior)."""
        self._diag = np.ascontiguousarray(diag, dtype=np.float64)
        lib().orc_op_set_diagonal(self.h, _dp(self._diag))
        return self

    def set_lowrank(self, Bdense, Sigma):
        Bdense = np.asarray(Bdense, dtype=np.float64)
        m = Bdense.shape[1]
        ptr, rows, vals = [0], [], []
        for j in range(m):
            nz = np.nonzero(Bdense[:, j])[0]
            rows.extend(nz.tolist())
            vals.extend(Bdense[nz, j].tolist())
            ptr.append(len(rows))
        ptr = np.array(ptr, np.int64)
        rows = np.array(rows, np.int64)
        vals = np.array(vals)
        sig = np.ascontiguousarray(Sigma, dtype=np.float64)
        lib().orc_op_set_lowrank(self.h, m, _ip(ptr), _ip(rows), _dp(vals), _dp(sig))
        return self

    def add_measurements(self, locations, variance, variance_scaling=1.0, radius=0.05,
                         measure_global=False, variance_global=0.0):
        loc = np.ascontiguousarray(locations, dtype=np.float64).reshape(-1)
        var = np.ascontiguousarray(variance, dtype=np.float64)
        lib().orc_op_add_measurements(self.h, len(var), _dp(loc), _dp(var), variance_scaling,
                                      radius, int(measure_global), variance_global)
        return self

    def apply(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.n)
        lib().orc_op_apply(self.h, _dp(x), _dp(y))
        return y

    def precision(self):
        Q = np.zeros((self.n, self.n))
        lib().orc_op_precision(self.h, _dp(Q))
        return Q

    def covariance(self):
        return np.linalg.inv(self.precision())

    def coarsen(self):
        return Operator(lib().orc_op_coarsen(self.h), [s // 2 for s in self.shape])


# ------------------------------------------------------------------ noise
class CLCG:
    """parallel_random.cc CLCGenerator (seed1 = seed2 = 1)."""

    def __init__(self, n_threads=1, thread_id=0):
        self.h = lib().orc_rng_create(n_threads, thread_id)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_rng_destroy(self.h)

    def draw_int(self, n):
        out = np.zeros(n, np.int32)
        lib().orc_rng_draw_int(self.h, n, out.ctypes.data_as(_I32))
        return out

    def draw_uniform(self, n):
        out = np.zeros(n)
        lib().orc_rng_draw_uniform(self.h, n, _dp(out))
        return out

    def draw_normal(self, n):
        out = np.zeros(n)
        lib().orc_rng_draw_normal(self.h, n, _dp(out))
        return out


class Source:
    """Normal source for the samplers: the CLCG or an injected buffer."""

    def __init__(self, buffer=None):
        if buffer is None:
            self.h = lib().orc_source_clcg()
            self._buf = None
        else:
            self._buf = np.ascontiguousarray(buffer, dtype=np.float64)
            self.h = lib().orc_source_buffer(_dp(self._buf), len(self._buf))

    @property
    def position(self):
        return lib().orc_source_position(self.h)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_source_destroy(self.h)


# ---------------------------------------------------------------- samplers
class Sampler:
    def __init__(self, handle, op, source):
        if not handle:
            raise RuntimeError("oracle sampler construction failed")
        self.h = handle
        self.op = op  # keep alive
        self.source = source
        self.n = op.n

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_sampler_destroy(self.h)

    def apply(self, f, x, nsteps=1):
        f = np.ascontiguousarray(f, dtype=np.float64)
        assert x.dtype == np.float64 and x.flags.c_contiguous
        rc = lib().orc_sampler_apply(self.h, _dp(f), _dp(x), nsteps)
        if rc:
            raise RuntimeError("oracle sampler apply failed (noise exhausted?)")

    def observe(self, f, x, nsteps, bidx, bval):
        f = np.ascontiguousarray(f, dtype=np.float64)
        bidx = np.ascontiguousarray(bidx, dtype=np.int64)
        bval = np.ascontiguousarray(bval, dtype=np.float64)
        obs = np.zeros(nsteps)
        rc = lib().orc_sampler_observe(self.h, _dp(f), _dp(x), nsteps, len(bidx), _ip(bidx), _dp(bval), _dp(obs))
        if rc:
            raise RuntimeError("oracle sampler observe failed")
        return obs

    def mean_cov(self, f, x, nwarmup, nsamples):
        n = self.n
        f = np.ascontiguousarray(f, dtype=np.float64)
        Ex = np.zeros(n)
        Cxx = np.zeros((n, n))
        rc = lib().orc_sampler_mean_cov(self.h, n, _dp(f), _dp(x), nwarmup, nsamples, _dp(Ex), _dp(Cxx))
        if rc:
            raise RuntimeError("oracle sampler failed")
        return Ex, Cxx


def sor_sampler(op, source, omega, nsmooth=1, forward=True, ordering=0):
    return Sampler(lib().orc_sor_sampler(op.h, source.h, omega, nsmooth, int(forward), ordering), op, source)


def ssor_sampler(op, source, omega, nsmooth=1, ordering=0):
    return Sampler(lib().orc_ssor_sampler(op.h, source.h, omega, nsmooth, ordering), op, source)


def cholesky_sampler(op, source):
    return Sampler(lib().orc_cholesky_sampler(op.h, source.h), op, source)


def lowrank_cholesky_sampler(op, source):
    """LowRankCholeskySampler (cholesky_sampler.cc:41-129) with the dense
    natural-order factor of the sparse part."""
    return Sampler(lib().orc_lowrank_cholesky_sampler(op.h, source.h), op, source)


def mgmc_sampler(op, source, nlevel, smoother="SSOR", coarse_solver="Cholesky", npresmooth=1,
                 npostsmooth=1, ncoarsesmooth=1, omega=1.0, cycle=1, coarse_scaling=1.0, ordering=0):
    h = lib().orc_mgmc_sampler(op.h, source.h, nlevel, 1 if smoother == "SSOR" else 0,
                               0 if coarse_solver == "Cholesky" else 1, npresmooth, npostsmooth,
                               ncoarsesmooth, omega, cycle, coarse_scaling, ordering)
    return Sampler(h, op, source)


def ssor_smoother_apply(op, omega, b, x, nsmooth=1, ordering=0):
    b = np.ascontiguousarray(b, dtype=np.float64)
    lib().orc_ssor_smoother_apply(op.h, omega, nsmooth, ordering, _dp(b), _dp(x))


class MGPreconditioner:
    """MultigridPreconditioner (multigrid_preconditioner.cc:8-108); coarse
    solve by the Woodbury CholeskySolver (woodbury=True) or the dense
    natural-order factor of the full coarse precision."""

    def __init__(self, op, nlevel, smoother="SSOR", npresmooth=1, npostsmooth=1, omega=1.0, cycle=1,
                 coarse_scaling=1.0, ordering=0, woodbury=True):
        self.op = op
        self.h = lib().orc_mg_create(op.h, nlevel, 1 if smoother == "SSOR" else 0, npresmooth, npostsmooth,
                                     omega, cycle, coarse_scaling, ordering, int(woodbury))
        if not self.h:
            raise RuntimeError("multigrid preconditioner set-up failed")

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_mg_destroy(self.h)
            self.h = None

    def apply(self, b):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(self.op.n)
        lib().orc_mg_apply(self.h, _dp(b), _dp(x))
        return x

    def loop_solve(self, b, rtol, atol, maxiter):
        """LoopSolver::apply (loop_solver.cc:9-53): (x, niter, rnorm, converged)."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(self.op.n)
        rn = C.c_double(0.0)
        cv = C.c_int(0)
        it = lib().orc_loop_solve(self.h, _dp(b), _dp(x), rtol, atol, maxiter, C.byref(rn), C.byref(cv))
        return x, it, rn.value, bool(cv.value)


def cholesky_solve(op, b):
    """CholeskySolver::apply (cholesky_solver.cc:9-43, Woodbury form)."""
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros(op.n)
    if lib().orc_cholesky_solve(op.h, _dp(b), _dp(x)):
        raise np.linalg.LinAlgError("not SPD")
    return x


def dense_cholesky(A):
    M = np.array(A, dtype=np.float64, order="C")
    if lib().orc_dense_cholesky(_dp(M), M.shape[0]):
        raise np.linalg.LinAlgError("not SPD")
    return M


# -------------------------------------------------------------- statistics
class Statistics:
    """statistics.{hh,cc}: running moments, autocovariance window, tau_int."""

    def __init__(self, dim, window):
        self.dim = dim
        self.h = lib().orc_stats_create(dim, window)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_stats_destroy(self.h)

    def record(self, Q):
        Q = np.ascontiguousarray(Q, dtype=np.float64).reshape(-1, self.dim)
        lib().orc_stats_record(self.h, _dp(Q), Q.shape[0])

    def average(self):
        out = np.zeros(self.dim)
        lib().orc_stats_average(self.h, _dp(out))
        return out

    def covariance(self):
        out = np.zeros((self.dim, self.dim))
        lib().orc_stats_covariance(self.h, _dp(out))
        return out

    def auto_covariance(self, window):
        out = np.zeros((window, self.dim, self.dim))
        k = lib().orc_stats_autocov(self.h, _dp(out))
        return out[:k]

    def tau_int(self, v):
        v = np.ascontiguousarray(v, dtype=np.float64)
        return lib().orc_stats_tau_int(self.h, _dp(v))
