"""GB300 Multigrid Monte Carlo sampler -- Python front end.

Mirrors the reference's class surface for the sampling path:

=======================  ==========================================================
this module              reference (eikehmueller/MultigridMC)
=======================  ==========================================================
``fd_stencil``           ShiftedLaplaceFDOperator (linear_operator/shiftedlaplace_fd_operator.cc:9-57)
``measurement_vector``   MeasuredOperator::measurement_vector (linear_operator/measured_operator.cc:69-171)
``LinearOperator``       LinearOperator / MeasuredOperator (linear_operator/linear_operator.hh:19-213,
                         measured_operator.cc:9-47)
``MultigridParameters``  MultigridParameters (auxilliary/parameters.hh:150-179)
``MultigridMCSampler``   MultigridMCSampler (sampler/multigridmc_sampler.cc:8-145)
``SSORSampler``          SSORSampler (sampler/ssor_sampler.{hh,cc})
``CholeskySampler``      DenseCholeskySampler (sampler/cholesky_sampler.cc:25-37)
``LowRankCholeskySampler``  LowRankCholeskySampler (sampler/cholesky_sampler.cc:41-129)
``MultigridPreconditioner``  MultigridPreconditioner (preconditioner/multigrid_preconditioner.cc:8-108)
``SORSmoother``          SORSmoother (smoother/sor_smoother.cc:9-78), nsmooth = 1
``SSORSmoother``         SSORSmoother (smoother/ssor_smoother.cc:9-16)
``ExactSampler``         exact draws x = Q^{-1}(f + eta), the comparator role of SparseCholeskySampler
                         (sampler/cholesky_sampler.cc:9-23)
``LoopSolver``           LoopSolver (solver/loop_solver.cc:9-53) with IterativeSolverParameters
                         (auxilliary/parameters.hh:130-147)
=======================  ==========================================================

Every call goes through the C ABI of ``libmgmc_gb300.so``
(``include/mgmc_gb300.h``); there is no CPU implementation behind this
module.  If the library cannot be loaded, import of the sampler classes
raises -- nothing falls back to the host.
"""
import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

from . import statistics  # noqa: F401  (tau_int for chain observables)

from . import build as _build

__all__ = [
    "MGMCError", "load", "fd_stencil", "galerkin_stencil", "measurement_vector", "intergrid_to_sparse",
    "LinearOperator",
    "MultigridParameters", "MultigridMCSampler", "MultigridMCBatch", "SSORSampler", "CholeskySampler",
    "LowRankCholeskySampler",
    "IterativeSolverParameters", "MultigridPreconditioner", "LoopSolver", "ExactSampler", "SORSmoother",
    "SSORSmoother",
    "FP64", "FP32_MIXED", "LEXICOGRAPHIC", "MULTICOLOUR", "PHILOX", "INJECTED", "FORWARD", "BACKWARD",
]

OK = 0
STATUS = {0: "MGMC_OK", 1: "MGMC_ERR_INVALID_ARGUMENT", 2: "MGMC_ERR_LATTICE", 3: "MGMC_ERR_NOT_SPD",
          4: "MGMC_ERR_CUDA", 5: "MGMC_ERR_OUT_OF_MEMORY", 6: "MGMC_ERR_NOISE_EXHAUSTED",
          7: "MGMC_ERR_NONFINITE", 8: "MGMC_ERR_UNSUPPORTED"}
LEXICOGRAPHIC, MULTICOLOUR = 0, 1
FP64, FP32_MIXED = 0, 1
PHILOX, INJECTED = 0, 1
FORWARD, BACKWARD = 1, 2


class MGMCError(RuntimeError):
    """A C-ABI call returned a status other than MGMC_OK."""

    def __init__(self, status, message):
        self.status = status
        self.name = STATUS.get(status, str(status))
        super().__init__(f"{self.name}: {message}")


class _OpDesc(C.Structure):
    _fields_ = [("dim", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("stencil", C.c_double * 27), ("m", C.c_int),
                ("B_colptr", C.POINTER(C.c_int64)), ("B_rowidx", C.POINTER(C.c_int64)),
                ("B_val", C.POINTER(C.c_double)), ("Sigma", C.POINTER(C.c_double)),
                ("centre", C.POINTER(C.c_double)), ("field", C.POINTER(C.c_double))]


class _Params(C.Structure):
    _fields_ = [("nlevel", C.c_int), ("smoother", C.c_int), ("coarse_solver", C.c_int),
                ("npresmooth", C.c_int), ("npostsmooth", C.c_int), ("ncoarsesmooth", C.c_int),
                ("omega", C.c_double), ("cycle", C.c_int), ("coarse_scaling", C.c_double),
                ("ordering", C.c_int), ("precision", C.c_int), ("noise", C.c_int),
                ("seed", C.c_uint64), ("device", C.c_int)]


_lib = None
_D = C.POINTER(C.c_double)
_I64 = C.POINTER(C.c_int64)
_P = C.c_void_p

# name -> (restype, argtypes); the list is the complete set of symbols the
# header declares
SIGNATURES = {
    "mgmc_abi_version": (C.c_int, []),
    "mgmc_last_error": (C.c_char_p, []),
    "mgmc_fd_stencil": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, _D]),
    "mgmc_measurement_vector": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, _D, C.c_double, _I64, _D,
                                          C.c_int64, _I64]),
    "mgmc_galerkin_stencil": (C.c_int, [C.c_int, _D, _D]),
    "mgmc_operator_coarsen": (C.c_int, [C.POINTER(_OpDesc), _D, _D, _I64, _I64, _D, C.c_int64, _I64]),
    "mgmc_fem_field": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, _D]),
    "mgmc_sampler_create": (C.c_int, [C.POINTER(_OpDesc), C.POINTER(_Params), C.POINTER(_P)]),
    "mgmc_sampler_destroy": (C.c_int, [_P]),
    "mgmc_sampler_apply": (C.c_int, [_P, _D, _D, C.c_int]),
    "mgmc_sampler_fix_rhs": (C.c_int, [_P, _D, C.c_int]),
    "mgmc_sampler_set_state": (C.c_int, [_P, _D, C.c_int]),
    "mgmc_sampler_get_state": (C.c_int, [_P, _D, C.c_int]),
    "mgmc_sampler_step": (C.c_int, [_P, C.c_int64]),
    "mgmc_sampler_set_step_counter": (C.c_int, [_P, C.c_int64]),
    "mgmc_sampler_get_step_counter": (C.c_int, [_P, _I64]),
    "mgmc_sampler_set_observable": (C.c_int, [_P, C.c_int64, _I64, _D, C.c_int64]),
    "mgmc_sampler_read_observations": (C.c_int, [_P, _D, C.c_int64, _I64]),
    "mgmc_sampler_set_probes": (C.c_int, [_P, C.c_int, _I64, _I64, _D, C.c_int64]),
    "mgmc_sampler_inject_noise": (C.c_int, [_P, _D, C.c_int64, C.c_int]),
    "mgmc_sampler_noise_per_step": (C.c_int, [_P, _I64]),
    "mgmc_sampler_synchronize": (C.c_int, [_P]),
    "mgmc_sampler_stream": (C.c_int, [_P, C.POINTER(_P)]),
    "mgmc_sampler_nlevel": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "mgmc_sampler_level_size": (C.c_int, [_P, C.c_int, _I64]),
    "mgmc_sampler_launches_per_step": (C.c_int, [_P, _I64]),
    "mgmc_sampler_adjoint_step": (C.c_int, [_P, _D, _D, C.c_int]),
    "mgmc_sampler_adjoint_params": (C.c_int, [_P, _D, C.c_int64, _D, _D, _D, _D, C.c_int]),
    "mgmc_sampler_precondition": (C.c_int, [_P, _D, _D, C.c_int]),
    "mgmc_sampler_exact_sample": (C.c_int, [_P, _D, _D, C.c_double, C.c_int, C.c_int, C.POINTER(C.c_int)]),
    "mgmc_sampler_solve": (C.c_int, [_P, _D, _D, C.c_double, C.c_double, C.c_int, C.c_int,
                                     C.POINTER(C.c_int), _D, C.POINTER(C.c_int)]),
    "mgmc_level_stencil": (C.c_int, [_P, C.c_int, _D]),
    "mgmc_level_apply": (C.c_int, [_P, C.c_int, _D, _D]),
    "mgmc_level_restrict": (C.c_int, [_P, C.c_int, _D, _D]),
    "mgmc_level_prolongate_add": (C.c_int, [_P, C.c_int, C.c_double, _D, _D]),
    "mgmc_level_sor": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, _D, _D]),
    "mgmc_level_sweep_device": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int64]),
    "mgmc_level_transfer_device": (C.c_int, [_P, C.c_int, C.c_int, C.c_int64]),
    "mgmc_batch_create": (C.c_int, [C.c_int, C.POINTER(_P), C.POINTER(_P)]),
    "mgmc_batch_step": (C.c_int, [_P, C.c_int64]),
    "mgmc_batch_info": (C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "mgmc_batch_synchronize": (C.c_int, [_P]),
    "mgmc_batch_stream": (C.c_int, [_P, C.POINTER(_P)]),
    "mgmc_batch_destroy": (C.c_int, [_P]),
    "mgmc_lrchol_create": (C.c_int, [C.POINTER(_OpDesc), C.c_int, C.c_uint64, C.c_int, C.POINTER(_P)]),
    "mgmc_lrchol_destroy": (C.c_int, [_P]),
    "mgmc_lrchol_fix_rhs": (C.c_int, [_P, _D, C.c_int]),
    "mgmc_lrchol_apply": (C.c_int, [_P, _D, _D, C.c_int]),
    "mgmc_lrchol_inject_noise": (C.c_int, [_P, _D, C.c_int64]),
    "mgmc_lrchol_stream": (C.c_int, [_P, C.POINTER(_P)]),
    "mgmc_device_fma_rate": (C.c_int, [C.c_int, _D]),
    "mgmc_measured_apply_noalloc": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, _D, C.c_int, _P, _P, _P, _P,
                                              _P, _P, _P]),
}


def library_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load libmgmc_gb300.so (building it in-tree if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise ImportError(f"{path} is missing; run multigridmc_gb300.build.build()")
        _build.build()
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _check(status):
    if status != OK:
        msg = load().mgmc_last_error()
        raise MGMCError(status, msg.decode() if msg else "")


def _dp(a):
    return a.ctypes.data_as(_D)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _shape3(shape):
    s = list(shape) + [2] * (3 - len(shape))
    return int(s[0]), int(s[1]), int(s[2])


# ------------------------------------------------------------- host set-up
def fd_stencil(shape, kappa_sq):
    """27-entry stencil of ShiftedLaplaceFDOperator on a lattice of `shape` cells."""
    st = np.zeros(27)
    _check(load().mgmc_fd_stencil(len(shape), *_shape3(shape), float(kappa_sq), _dp(st)))
    return st


def fem_field(shape, model, p0, p1=0.0):
    """Per-vertex stencils of ShiftedLaplaceFEMOperator (27 x n, weight-major):
    model 0 constant kappa^2 = p0, model 1 periodic (Lambda_min, Lambda_max)."""
    n = int(np.prod([s - 1 for s in shape]))
    out = np.zeros((27, n))
    _check(load().mgmc_fem_field(len(shape), *_shape3(shape), int(model), float(p0), float(p1), _dp(out)))
    return out


def galerkin_stencil(dim, fine):
    fine = _f64(fine)
    out = np.zeros(27)
    _check(load().mgmc_galerkin_stencil(dim, _dp(fine), _dp(out)))
    return out


def intergrid_to_sparse(shape):
    """IntergridOperator::to_sparse (intergrid/intergrid_operator.hh:122-144)
    of the linear intergrid operator (intergrid_operator_linear.cc:8-31):
    the restriction R from the lattice of `shape` cells to the lattice of
    shape // 2 cells as a scipy.sparse CSR matrix (n_coarse x n_fine); coarse
    vertex a sits on fine vertex 2 a + 1 per direction, with weights
    prod_d {1/2, 1, 1/2} on its 3^d footprint.  The prolongation is R^T.
    Host-side (set-up and checks); the samplers apply R and P with their own
    kernels."""
    import scipy.sparse as sp
    dim = len(shape)
    Nf = [c - 1 for c in shape]
    Nc = [c // 2 - 1 for c in shape]
    cidx = np.indices(Nc[::-1]).reshape(dim, -1)[::-1]  # coarse (a, b, c), x fastest
    ccol = np.arange(int(np.prod(Nc)))
    rows, cols, vals = [], [], []
    for off in np.ndindex(*([3] * dim)):
        o = np.array(off) - 1
        fpos = 2 * cidx + 1 + o[:, None]
        ok = np.all((fpos >= 0) & (fpos < np.array(Nf)[:, None]), axis=0)
        frow = np.zeros(ok.sum(), np.int64)
        stride = 1
        for d in range(dim):
            frow += fpos[d, ok] * stride
            stride *= Nf[d]
        rows.append(frow)
        cols.append(ccol[ok])
        vals.append(np.full(ok.sum(), 0.5 ** int(np.abs(o).sum())))
    n_f, n_c = int(np.prod(Nf)), int(np.prod(Nc))
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(cols), np.concatenate(rows))), shape=(n_c, n_f))


def measured_apply_noalloc(op, B_colptr, B_rowidx, B_val, Sigma, x, y, stream=0):
    """mgmc_measured_apply_noalloc: y = A x with device buffers given as raw
    addresses (integers); nothing is allocated by the library.  Asynchronous
    on `stream` (a cudaStream_t address, 0 = default stream).  A_0 must be
    one constant stencil: an operator with a per-vertex centre or stencil
    field (periodic correlation length, FEM with variable coefficients) is
    refused with MGMC_ERR_INVALID_ARGUMENT rather than applied with the
    wrong weights."""
    if op.centre is not None or op.field is not None:
        raise MGMCError(1, "mgmc_measured_apply_noalloc handles a constant stencil A_0 only; this operator "
                           "has per-vertex coefficients")
    st = _f64(op.stencil)
    _check(load().mgmc_measured_apply_noalloc(op.dim, *_shape3(op.shape), _dp(st), op.m, B_colptr, B_rowidx,
                                              B_val, Sigma, x, y, stream))


def device_fma_rate(precision):
    """mgmc_device_fma_rate: the measured FMA throughput of the current GPU
    in TFLOP/s, FP64 (precision FP64) or FP32 (precision FP32_MIXED)."""
    out = C.c_double(0.0)
    _check(load().mgmc_device_fma_rate(int(precision), C.byref(out)))
    return out.value


def measurement_vector(shape, x0, radius):
    """(indices, values) of MeasuredOperator::measurement_vector."""
    x0 = _f64(x0)
    nnz = C.c_int64(0)
    L = load()
    _check(L.mgmc_measurement_vector(len(shape), *_shape3(shape), _dp(x0), float(radius), None, None, 0,
                                     C.byref(nnz)))
    idx = np.zeros(nnz.value, np.int64)
    val = np.zeros(nnz.value)
    _check(L.mgmc_measurement_vector(len(shape), *_shape3(shape), _dp(x0), float(radius),
                                     idx.ctypes.data_as(_I64), _dp(val), nnz.value, C.byref(nnz)))
    return idx, val


@dataclass
class LinearOperator:
    """A = A_0 + B Sigma^{-1} B^T with a constant stencil A_0 on `shape` cells.

    ``B`` is held column-compressed (``B_ptr``, ``B_idx``, ``B_val``) in the
    reference's vertex order.
    """
    shape: tuple
    stencil: np.ndarray
    B_ptr: np.ndarray = field(default_factory=lambda: np.zeros(1, np.int64))
    B_idx: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    B_val: np.ndarray = field(default_factory=lambda: np.zeros(0))
    Sigma: np.ndarray = field(default_factory=lambda: np.zeros(0))
    centre: np.ndarray = None  # per-vertex centre weight of the stencil (variable coefficients), or None
    field: np.ndarray = None   # per-vertex 27-point stencils, weight-major (27 x n), or None

    @property
    def dim(self):
        return len(self.shape)

    @property
    def m(self):
        return len(self.B_ptr) - 1

    @property
    def n(self):
        return int(np.prod([s - 1 for s in self.shape]))

    @classmethod
    def shifted_laplace_fd(cls, shape, kappa_sq=None, Lambda=None):
        """ShiftedLaplaceFDOperator with kappa^2 = 1/Lambda^2 (correlationlength_model.hh:52)."""
        if kappa_sq is None:
            kappa_sq = 1.0 / Lambda ** 2
        return cls(tuple(int(s) for s in shape), fd_stencil(shape, kappa_sq))

    @classmethod
    def shifted_laplace_fem(cls, shape, kappa_sq=None, Lambda=None):
        """ShiftedLaplaceFEMOperator (shiftedlaplace_fem_operator.cc:9-152) with a
        constant correlation length: a constant 3^d-point stencil."""
        if kappa_sq is None:
            kappa_sq = 1.0 / Lambda ** 2
        shape = tuple(int(s) for s in shape)
        fld = fem_field(shape, 0, kappa_sq, 0.0)
        n = fld.shape[1]
        return cls(shape, fld[:, n // 2].copy())

    @classmethod
    def shifted_laplace_fem_periodic(cls, shape, Lambda_min, Lambda_max):
        """ShiftedLaplaceFEMOperator with the periodic correlation length: a
        per-vertex 3^d-point stencil field (the mass term follows kappa^2(x))."""
        shape = tuple(int(s) for s in shape)
        fld = fem_field(shape, 1, Lambda_min, Lambda_max)
        n = fld.shape[1]
        return cls(shape, fld[:, n // 2].copy(), field=fld)

    @staticmethod
    def periodic_kappa_sq(shape, Lambda_min, Lambda_max):
        """kappa^2(x) = 1 / Lambda(x)^2 at the vertices, Lambda(x) = Lambda_1 +
        Lambda_2 prod_d cos(pi x_d), Lambda_1,2 = (Lambda_max +- Lambda_min) / 2
        (PeriodicCorrelationLengthModel, correlationlength_model.hh:83-112);
        vertex i (0-based) of a direction with n cells at x = (i + 1) / n."""
        L1, L2 = 0.5 * (Lambda_max + Lambda_min), 0.5 * (Lambda_max - Lambda_min)
        axes = [np.cos(np.pi * (np.arange(c - 1) + 1.0) / c) for c in shape]
        lam = np.full([c - 1 for c in shape[::-1]], L2)
        for d, a in enumerate(axes):  # x fastest: the last array axis
            sh = [1] * len(shape)
            sh[len(shape) - 1 - d] = a.size
            lam = lam * a.reshape(sh)
        lam = lam + L1
        return (1.0 / (lam * lam)).reshape(-1)

    @classmethod
    def shifted_laplace_fd_periodic(cls, shape, Lambda_min, Lambda_max):
        """ShiftedLaplaceFDOperator with the periodic correlation length: the
        neighbour weights -h^d / h_d^2 and the per-vertex diagonal
        h^d kappa^2(x) + sum_d 2 h^d / h_d^2 (shiftedlaplace_fd_operator.cc:33-52)."""
        shape = tuple(int(s) for s in shape)
        st = fd_stencil(shape, 0.0)
        hd = 1.0
        for c in shape:
            hd *= 1.0 / c
        diag = hd * cls.periodic_kappa_sq(shape, Lambda_min, Lambda_max)
        for c in shape:
            diag = diag + 2.0 * hd * (c * c)
        return cls(shape, st, centre=diag)

    def with_lowrank(self, Bdense_or_cols, Sigma):
        """Attach B (dense n x m array, or list of (idx, val) columns) and Sigma."""
        cols = Bdense_or_cols
        if isinstance(cols, np.ndarray):
            cols = [(np.nonzero(cols[:, j])[0], cols[np.nonzero(cols[:, j])[0], j]) for j in range(cols.shape[1])]
        ptr, idx, val = [0], [], []
        for (i, v) in cols:
            order = np.argsort(i, kind="stable")
            idx.extend(np.asarray(i, np.int64)[order].tolist())
            val.extend(np.asarray(v, np.float64)[order].tolist())
            ptr.append(len(idx))
        return LinearOperator(self.shape, self.stencil, np.array(ptr, np.int64), np.array(idx, np.int64),
                              np.array(val, np.float64), _f64(Sigma), self.centre, self.field)

    def with_measurements(self, locations, variance, variance_scaling=1.0, radius=0.05, measure_global=False,
                          variance_global=0.0):
        """MeasuredOperator (measured_operator.cc:9-47)."""
        locations = np.asarray(locations, np.float64).reshape(-1, self.dim)
        cols = [measurement_vector(self.shape, x0, radius) for x0 in locations]
        sigma = list(variance_scaling * np.asarray(variance, np.float64))
        if measure_global:
            cv = 1.0
            for s in self.shape:
                cv /= float(s)
            cols.append((np.arange(self.n, dtype=np.int64), np.full(self.n, cv)))
            sigma.append(variance_global)
        return self.with_lowrank(cols, sigma)

    def coarsen(self):
        """LinearOperator::coarsen (linear_operator.cc:10-23): the operator
        R A R^T + (R B) Sigma^{-1} (R B)^T on the lattice with half the cells
        per direction (mgmc_operator_coarsen), with the coarse stencil, the
        coarse per-vertex stencils of a variable operator and B_c = R B."""
        cshape = tuple(s // 2 for s in self.shape)
        nc = int(np.prod([s - 1 for s in cshape]))
        variable = self.centre is not None or self.field is not None
        st = np.zeros(27)
        cf = np.zeros((27, nc)) if variable else None
        ptr = np.zeros(self.m + 1, np.int64)
        nnz = C.c_int64(0)
        desc = self._desc()
        L = load()
        cfp = _dp(cf) if variable else None
        _check(L.mgmc_operator_coarsen(C.byref(desc), _dp(st), cfp, ptr.ctypes.data_as(_I64), None, None, 0,
                                       C.byref(nnz)))
        idx = np.zeros(nnz.value, np.int64)
        val = np.zeros(nnz.value)
        _check(L.mgmc_operator_coarsen(C.byref(desc), _dp(st), cfp, ptr.ctypes.data_as(_I64),
                                       idx.ctypes.data_as(_I64), _dp(val), nnz.value, C.byref(nnz)))
        return LinearOperator(cshape, st, ptr, idx, val, np.array(self.Sigma, dtype=float), field=cf)

    def to_scipy(self):
        """A = A_0 + B Sigma^{-1} B^T as a scipy.sparse CSR matrix in the
        vertex order (the matrix LinearOperator::get_sparse of the reference
        assembles; host-side, for exact comparators at moderate sizes)."""
        import scipy.sparse as sp
        N = [c - 1 for c in self.shape] + [1] * (3 - self.dim)
        n = self.n
        idx = np.arange(n).reshape(N[2], N[1], N[0])
        rows, cols, vals = [], [], []
        for dz in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dx in (-1, 0, 1):
                    k = (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1)
                    w = float(self.stencil[k])
                    if w == 0.0 and (self.field is None or not self.field[k].any()):
                        continue
                    src = idx[max(0, -dz):N[2] - max(0, dz), max(0, -dy):N[1] - max(0, dy), max(0, -dx):N[0] - max(0, dx)]
                    dst = idx[max(0, dz):N[2] + min(0, dz), max(0, dy):N[1] + min(0, dy), max(0, dx):N[0] + min(0, dx)]
                    rows.append(src.ravel())
                    cols.append(dst.ravel())
                    vals.append(np.asarray(self.field[k])[src.ravel()] if self.field is not None else np.full(src.size, w))
        A = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))
        if self.centre is not None and self.field is None:
            A = (A + sp.diags(np.asarray(self.centre, np.float64) - float(self.stencil[13]))).tocsr()
        if self.m > 0:
            Bs = sp.csc_matrix((self.B_val, self.B_idx, self.B_ptr), shape=(n, self.m))
            A = (A + Bs @ sp.diags(1.0 / self.Sigma) @ Bs.T).tocsr()
        return A

    def B_dense(self):
        B = np.zeros((self.n, self.m))
        for j in range(self.m):
            B[self.B_idx[self.B_ptr[j]:self.B_ptr[j + 1]], j] = self.B_val[self.B_ptr[j]:self.B_ptr[j + 1]]
        return B

    def _desc(self):
        d = _OpDesc()
        d.dim = self.dim
        d.nx, d.ny, d.nz = _shape3(self.shape)
        for k in range(27):
            d.stencil[k] = float(self.stencil[k])
        d.m = self.m
        self._keep = (np.ascontiguousarray(self.B_ptr, np.int64), np.ascontiguousarray(self.B_idx, np.int64),
                      _f64(self.B_val), _f64(self.Sigma))
        d.B_colptr = self._keep[0].ctypes.data_as(_I64)
        d.B_rowidx = self._keep[1].ctypes.data_as(_I64)
        d.B_val = self._keep[2].ctypes.data_as(_D)
        d.Sigma = self._keep[3].ctypes.data_as(_D)
        if self.centre is not None:
            c = _f64(self.centre)
            if c.size != self.n:
                raise ValueError("centre needs one weight per vertex")
            self._keep = self._keep + (c,)
            d.centre = c.ctypes.data_as(_D)
        if self.field is not None:
            fl = _f64(self.field)
            if fl.shape != (27, self.n):
                raise ValueError("field needs 27 weights per vertex")
            self._keep = self._keep + (fl,)
            d.field = fl.ctypes.data_as(_D)
        return d


@dataclass
class MultigridParameters:
    """MultigridParameters (auxilliary/parameters.hh:150-179)."""
    nlevel: int = 4
    smoother: str = "SSOR"
    coarse_solver: str = "Cholesky"
    npresmooth: int = 1
    npostsmooth: int = 1
    ncoarsesmooth: int = 1
    omega: float = 1.0
    cycle: int = 1
    coarse_scaling: float = 1.0


# ------------------------------------------------------------------ sampler
class MultigridMCSampler:
    """GPU MultigridMCSampler: the chain state lives on the GPU.

    ``apply(f, x)`` follows Sampler::apply (sampler.hh:52-55): one sample,
    ``x`` (numpy float64, length n) is updated in place.
    """

    def __init__(self, linear_operator, params=None, ordering=MULTICOLOUR, precision=FP64, noise=PHILOX,
                 seed=0, device=0):
        params = params or MultigridParameters()
        self.op = linear_operator
        self.params = params
        self.n = linear_operator.n
        p = _Params()
        p.nlevel = params.nlevel
        p.smoother = {"SOR": 0, "SSOR": 1}[params.smoother]
        p.coarse_solver = {"Cholesky": 0, "SSOR": 1}[params.coarse_solver]
        p.npresmooth, p.npostsmooth, p.ncoarsesmooth = params.npresmooth, params.npostsmooth, params.ncoarsesmooth
        p.omega = params.omega
        p.cycle = params.cycle
        p.coarse_scaling = params.coarse_scaling
        p.ordering, p.precision, p.noise = ordering, precision, noise
        p.seed = seed
        p.device = device
        self._args = dict(ordering=ordering, precision=precision, noise=noise, device=device)
        self._h = C.c_void_p()
        desc = linear_operator._desc()
        self._L = load()
        _check(self._L.mgmc_sampler_create(C.byref(desc), C.byref(p), C.byref(self._h)))

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._L.mgmc_sampler_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- Sampler surface
    def apply(self, f, x):
        """Sampler::apply: x <- one MGMC step with right hand side f.  With
        f = None the step uses the right hand side already on the device
        (fix_rhs, or the last apply), and only x crosses the host link."""
        assert x.dtype == np.float64 and x.flags.c_contiguous and x.size == self.n
        if f is None:
            _check(self._L.mgmc_sampler_apply(self._h, None, _dp(x), 0))
            return x
        f = _f64(f)
        _check(self._L.mgmc_sampler_apply(self._h, _dp(f), _dp(x), 0))
        return x

    def fix_rhs(self, f):
        """The right hand side ``step()`` and ``apply(None, x)`` sample with
        (Sampler::fix_rhs, sampler.hh:64); ``apply(f, x)`` with an f uses
        that f, as in the reference, whose MultigridMCSampler inherits the
        no-op fix_rhs."""
        f = _f64(f)
        _check(self._L.mgmc_sampler_fix_rhs(self._h, _dp(f), 0))

    def unfix_rhs(self):
        """Sampler::unfix_rhs (sampler.hh:71): a no-op for this sampler --
        ``apply(f, x)`` reads its f on every call either way."""

    def get_linear_operator(self):
        """Sampler::get_linear_operator (sampler.hh:51-54)."""
        return self.op

    def deep_copy(self, seed):
        """Sampler::deep_copy (sampler.hh:40, multigridmc_sampler.hh:50-57):
        a new sampler of the same operator and parameters that draws from its
        own noise stream -- the Philox key ``seed`` in place of the
        reference's RandomGenerator -- with its own chain state (zero) and
        no fixed right hand side.  The copy shares nothing on the device."""
        return MultigridMCSampler(self.op, self.params, seed=seed, **self._args)

    def set_state(self, x):
        x = _f64(x)
        _check(self._L.mgmc_sampler_set_state(self._h, _dp(x), 0))

    def get_state(self):
        x = np.zeros(self.n)
        _check(self._L.mgmc_sampler_get_state(self._h, _dp(x), 0))
        return x

    def adjoint_step(self, xbar, fbar):
        """Adjoint of one step with its noise held fixed: xbar (the adjoint of
        the step's output state) becomes the adjoint of its input state, in
        place, and the adjoint with respect to the right hand side f is added
        to fbar.  No counterpart in the reference."""
        assert xbar.dtype == np.float64 and xbar.flags.c_contiguous and xbar.size == self.n
        assert fbar.dtype == np.float64 and fbar.flags.c_contiguous and fbar.size == self.n
        _check(self._L.mgmc_sampler_adjoint_step(self._h, _dp(xbar), _dp(fbar), 0))
        return xbar

    def adjoint_params(self, x_in, xbar, fbar, step_index=0):
        """adjoint_step with the parameters: replays the step from x_in (with
        the step's noise: the next injected values, or the Philox noise of
        step `step_index`), turns xbar into the adjoint of x_in in place, adds
        K^T xbar to fbar and returns (d/dcentre, d/dlog Sigma) of xbar^T x_out
        with the right hand side held fixed.  No counterpart in the
        reference."""
        x_in = _f64(x_in)
        assert xbar.dtype == np.float64 and xbar.flags.c_contiguous and xbar.size == self.n
        assert fbar.dtype == np.float64 and fbar.flags.c_contiguous and fbar.size == self.n
        gc = C.c_double(0.0)
        gs = np.zeros(max(self.op.m, 1))
        _check(self._L.mgmc_sampler_adjoint_params(self._h, _dp(x_in), int(step_index), _dp(xbar), _dp(fbar),
                                                   C.byref(gc), _dp(gs), 0))
        return gc.value, gs[:self.op.m].copy()

    def precondition(self, b):
        """x = P b: one noise-free cycle of this hierarchy from zero
        (MultigridPreconditioner::apply); the chain is left unchanged."""
        b = _f64(b)
        x = np.zeros(self.n)
        _check(self._L.mgmc_sampler_precondition(self._h, _dp(b), _dp(x), 0))
        return x

    def solve(self, b, rtol=1e-10, atol=1e-10, maxiter=100):
        """LoopSolver::apply with this hierarchy as the multigrid
        preconditioner: returns (x, niter, residual norm, converged); the
        chain is left unchanged."""
        b = _f64(b)
        x = np.zeros(self.n)
        it, rn, cv = C.c_int(0), C.c_double(0.0), C.c_int(0)
        _check(self._L.mgmc_sampler_solve(self._h, _dp(b), _dp(x), float(rtol), float(atol), int(maxiter), 0,
                                          C.byref(it), C.byref(rn), C.byref(cv)))
        return x, it.value, rn.value, bool(cv.value)

    def exact_sample(self, f, rtol=1e-10, maxiter=100):
        """An exact draw from N(Q^{-1} f, Q^{-1}): x = Q^{-1}(f + eta) with
        eta ~ N(0, Q) drawn in-kernel, solved by the multigrid loop solver;
        advances the step counter.  Returns (x, iterations)."""
        f = _f64(f)
        x = np.zeros(self.n)
        it = C.c_int(0)
        _check(self._L.mgmc_sampler_exact_sample(self._h, _dp(f), _dp(x), float(rtol), int(maxiter), 0, C.byref(it)))
        return x, it.value

    def exact_sample_device(self, f_ptr, x_ptr, rtol=1e-10, maxiter=100):
        it = C.c_int(0)
        cast = lambda p: C.cast(C.c_void_p(p), _D)
        _check(self._L.mgmc_sampler_exact_sample(self._h, cast(f_ptr), cast(x_ptr), float(rtol), int(maxiter), 1,
                                                 C.byref(it)))
        return it.value

    def solve_device(self, b_ptr, x_ptr, rtol=1e-10, atol=1e-10, maxiter=100):
        """solve() on device vectors given as addresses of n float64 values
        (the solution is written to x_ptr); returns (niter, residual norm,
        converged)."""
        it, rn, cv = C.c_int(0), C.c_double(0.0), C.c_int(0)
        _check(self._L.mgmc_sampler_solve(self._h, C.cast(C.c_void_p(b_ptr), _D), C.cast(C.c_void_p(x_ptr), _D),
                                          float(rtol), float(atol), int(maxiter), 1, C.byref(it), C.byref(rn),
                                          C.byref(cv)))
        return it.value, rn.value, bool(cv.value)

    def step(self, nsteps=1):
        _check(self._L.mgmc_sampler_step(self._h, int(nsteps)))

    @property
    def step_counter(self):
        """The Philox step counter (steps taken since creation)."""
        c = C.c_int64(0)
        _check(self._L.mgmc_sampler_get_step_counter(self._h, C.byref(c)))
        return c.value

    @step_counter.setter
    def step_counter(self, k):
        _check(self._L.mgmc_sampler_set_step_counter(self._h, int(k)))

    # --- device-resident vectors (addresses of n float64 values)
    def set_state_device(self, x_ptr):
        _check(self._L.mgmc_sampler_set_state(self._h, C.cast(C.c_void_p(x_ptr), _D), 1))

    def get_state_device(self, x_ptr):
        """Writes the state to x_ptr and waits for it."""
        _check(self._L.mgmc_sampler_get_state(self._h, C.cast(C.c_void_p(x_ptr), _D), 1))
        self.synchronize()

    def adjoint_params_device(self, x_ptr, xbar_ptr, fbar_ptr, step_index=0):
        """adjoint_params on device vectors; returns (d/dcentre, d/dlog Sigma)."""
        gc = C.c_double(0.0)
        gs = np.zeros(max(self.op.m, 1))
        cast = lambda p: C.cast(C.c_void_p(p), _D)
        _check(self._L.mgmc_sampler_adjoint_params(self._h, cast(x_ptr), int(step_index), cast(xbar_ptr),
                                                   cast(fbar_ptr), C.byref(gc), _dp(gs), 1))
        return gc.value, gs[:self.op.m].copy()

    def synchronize(self):
        _check(self._L.mgmc_sampler_synchronize(self._h))

    @property
    def stream(self):
        s = C.c_void_p()
        _check(self._L.mgmc_sampler_stream(self._h, C.byref(s)))
        return s.value

    def set_observable(self, idx, val, capacity):
        self._nprobe = 1
        idx = np.ascontiguousarray(idx, np.int64)
        val = _f64(val)
        _check(self._L.mgmc_sampler_set_observable(self._h, len(idx), idx.ctypes.data_as(_I64), _dp(val),
                                                   int(capacity)))

    def set_probes(self, probes, capacity):
        """probes: list of (idx, val); after every step all b_p^T x are kept."""
        ptr, idx, val = [0], [], []
        for (i, v) in probes:
            idx.extend(np.asarray(i, np.int64).tolist())
            val.extend(np.asarray(v, np.float64).tolist())
            ptr.append(len(idx))
        ptr = np.array(ptr, np.int64)
        idx = np.array(idx, np.int64)
        val = np.array(val, np.float64)
        self._nprobe = len(probes)
        _check(self._L.mgmc_sampler_set_probes(self._h, len(probes), ptr.ctypes.data_as(_I64),
                                               idx.ctypes.data_as(_I64), _dp(val), int(capacity)))

    def read_observations(self, capacity):
        """Observations since the last read: shape (steps,) for one
        observable, (steps, nprobe) after set_probes."""
        np_ = getattr(self, "_nprobe", 1) or 1
        out = np.zeros(max(int(capacity), 1) * np_)
        cnt = C.c_int64(0)
        _check(self._L.mgmc_sampler_read_observations(self._h, _dp(out), int(capacity) * np_, C.byref(cnt)))
        k = min(cnt.value, capacity)
        return out[:k] if np_ == 1 else out[:k * np_].reshape(k, np_)

    def inject_noise(self, normals):
        normals = _f64(normals)
        _check(self._L.mgmc_sampler_inject_noise(self._h, _dp(normals), len(normals), 0))

    @property
    def noise_per_step(self):
        c = C.c_int64(0)
        _check(self._L.mgmc_sampler_noise_per_step(self._h, C.byref(c)))
        return c.value

    @property
    def nlevel(self):
        c = C.c_int(0)
        _check(self._L.mgmc_sampler_nlevel(self._h, C.byref(c)))
        return c.value

    def level_size(self, level):
        c = C.c_int64(0)
        _check(self._L.mgmc_sampler_level_size(self._h, level, C.byref(c)))
        return c.value

    @property
    def launches_per_step(self):
        c = C.c_int64(0)
        _check(self._L.mgmc_sampler_launches_per_step(self._h, C.byref(c)))
        return c.value

    # --- level building blocks
    def level_stencil(self, level):
        st = np.zeros(27)
        _check(self._L.mgmc_level_stencil(self._h, level, _dp(st)))
        return st

    def level_apply(self, level, x):
        x = _f64(x)
        y = np.zeros(self.level_size(level))
        _check(self._L.mgmc_level_apply(self._h, level, _dp(x), _dp(y)))
        return y

    def restrict(self, level, x):
        x = _f64(x)
        xc = np.zeros(self.level_size(level + 1))
        _check(self._L.mgmc_level_restrict(self._h, level, _dp(x), _dp(xc)))
        return xc

    def prolongate_add(self, level, alpha, xc, x):
        xc = _f64(xc)
        assert x.dtype == np.float64 and x.flags.c_contiguous
        _check(self._L.mgmc_level_prolongate_add(self._h, level, float(alpha), _dp(xc), _dp(x)))
        return x

    def sweep_device(self, level, direction=FORWARD, nrepeat=1, with_noise=True, with_lowrank=True):
        """SOR sweeps on the level's device-resident vectors (asynchronous)."""
        _check(self._L.mgmc_level_sweep_device(self._h, level, direction, int(with_noise), int(with_lowrank),
                                               int(nrepeat)))

    def transfer_device(self, level, which, nrepeat=1):
        """Residual-restrictions (which=0) or prolongations (which=1) between
        `level` and level+1 on the device-resident vectors (asynchronous)."""
        _check(self._L.mgmc_level_transfer_device(self._h, level, int(which), int(nrepeat)))

    def sor(self, level, direction, f, x, with_noise=True):
        f = _f64(f)
        assert x.dtype == np.float64 and x.flags.c_contiguous
        _check(self._L.mgmc_level_sor(self._h, level, direction, int(with_noise), _dp(f), _dp(x)))
        return x


class SORSmoother:
    """SORSmoother::apply (smoother/sor_smoother.cc:40-78) with nsmooth = 1,
    the form every sampler and SSORSmoother builds: one noise-free SOR sweep
    of level ``level`` of ``sampler``'s hierarchy (its operator and omega) in
    ``direction``, then the low-rank correction x -= Bbar B^T x.  ``x`` is
    updated in place."""

    def __init__(self, sampler, level=0, direction=FORWARD):
        self.sampler, self.level, self.direction = sampler, level, direction

    def apply(self, b, x):
        return self.sampler.sor(self.level, self.direction, b, x, with_noise=False)


class SSORSmoother:
    """SSORSmoother::apply (smoother/ssor_smoother.cc:9-16): ``nsmooth``
    times a forward then a backward SORSmoother on one level."""

    def __init__(self, sampler, level=0, nsmooth=1):
        self.forward = SORSmoother(sampler, level, FORWARD)
        self.backward = SORSmoother(sampler, level, BACKWARD)
        self.nsmooth = nsmooth

    def apply(self, b, x):
        for _ in range(self.nsmooth):
            self.forward.apply(b, x)
            self.backward.apply(b, x)
        return x


class MultigridMCBatch:
    """Independent chains stepped together in one CUDA graph (mgmc_batch_*)."""

    def __init__(self, samplers):
        self.samplers = list(samplers)  # keep alive
        self._L = load()
        arr = (C.c_void_p * len(self.samplers))(*[s._h.value for s in self.samplers])
        self._h = C.c_void_p()
        _check(self._L.mgmc_batch_create(len(self.samplers), arr, C.byref(self._h)))

    def step(self, nsteps=1):
        _check(self._L.mgmc_batch_step(self._h, int(nsteps)))

    def synchronize(self):
        _check(self._L.mgmc_batch_synchronize(self._h))

    @property
    def groups(self):
        """(number of batched groups, chains in them): the chains that step
        through the batched kernels rather than their own step graphs."""
        g, n = C.c_int(0), C.c_int(0)
        _check(self._L.mgmc_batch_info(self._h, C.byref(g), C.byref(n)))
        return g.value, n.value

    @property
    def stream(self):
        s = C.c_void_p()
        _check(self._L.mgmc_batch_stream(self._h, C.byref(s)))
        return s.value

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._L.mgmc_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def SSORSampler(linear_operator, omega=1.0, nsmooth=1, **kw):
    """SSORSampler (ssor_sampler.hh:29-37): a one-level hierarchy whose
    coarse solver is SSOR with `nsmooth` forward/backward pairs."""
    p = MultigridParameters(nlevel=1, coarse_solver="SSOR", ncoarsesmooth=nsmooth, omega=omega)
    return MultigridMCSampler(linear_operator, p, **kw)


class ExactSampler:
    """Exact sampler (the role of SparseCholeskySampler, cholesky_sampler.cc:9-23,
    at any lattice size): every apply(f, x) overwrites x with an independent
    draw x = Q^{-1}(f + eta), eta ~ N(0, Q), by a multigrid solve to relative
    residual `rtol` on the hierarchy of `params`."""

    def __init__(self, linear_operator, params=None, precision=FP32_MIXED, seed=0, rtol=1e-10, device=0):
        self.op = linear_operator
        self.rtol = rtol
        self._s = MultigridMCSampler(linear_operator, params, precision=precision, seed=seed, device=device)

    def apply(self, f, x):
        y, _ = self._s.exact_sample(f, self.rtol)
        x[:] = y
        return x

    def close(self):
        self._s.close()


def CholeskySampler(linear_operator, **kw):
    """Exact sampler with the dense natural-order Cholesky factor
    (DenseCholeskySampler, cholesky_sampler.cc:25-37).  Its ``apply(f, x)``
    reads f on every call; the reference's Cholesky samplers, after
    ``fix_rhs(f0)``, sample with f0 whatever f ``apply`` is given
    (cholesky_sampler.hh:52-66; its callers pass the same f)."""
    p = MultigridParameters(nlevel=1, coarse_solver="Cholesky")
    return MultigridMCSampler(linear_operator, p, **kw)


class LowRankCholeskySampler:
    """LowRankCholeskySampler (cholesky_sampler.cc:41-129): A_0 factored once
    on the host (FP64, block by block along the last lattice direction), the
    low-rank term through the thin QR of L^{-1} B; samples drawn on the GPU
    (mgmc_lrchol_*).  ``apply(f, x)`` writes a sample into x; f = None uses
    the f given to ``fix_rhs``."""

    def __init__(self, linear_operator, noise=PHILOX, seed=0, device=0):
        if linear_operator.centre is not None or linear_operator.field is not None:
            raise MGMCError(8, "the low-rank Cholesky sampler takes a constant stencil")
        self.op = linear_operator
        self.n = linear_operator.n
        self._L = load()
        self._h = C.c_void_p()
        desc = linear_operator._desc()
        _check(self._L.mgmc_lrchol_create(C.byref(desc), int(noise), C.c_uint64(seed), int(device),
                                          C.byref(self._h)))

    def fix_rhs(self, f):
        f = _f64(f)
        _check(self._L.mgmc_lrchol_fix_rhs(self._h, _dp(f), 0))

    def apply(self, f, x):
        assert x.dtype == np.float64 and x.flags.c_contiguous and x.size == self.n
        if f is None:
            _check(self._L.mgmc_lrchol_apply(self._h, None, _dp(x), 0))
        else:
            f = _f64(f)
            _check(self._L.mgmc_lrchol_apply(self._h, _dp(f), _dp(x), 0))
        return x

    def apply_device(self, f_ptr, x_ptr):
        """apply on device arrays (raw addresses; f_ptr = 0: the fixed f)."""
        _check(self._L.mgmc_lrchol_apply(self._h, C.cast(C.c_void_p(f_ptr or None), _D),
                                         C.cast(C.c_void_p(x_ptr), _D), 1))

    def inject_noise(self, normals):
        normals = _f64(normals)
        _check(self._L.mgmc_lrchol_inject_noise(self._h, _dp(normals), len(normals)))

    @property
    def stream(self):
        st = C.c_void_p()
        _check(self._L.mgmc_lrchol_stream(self._h, C.byref(st)))
        return st.value

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._L.mgmc_lrchol_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------ deterministic solver
@dataclass
class IterativeSolverParameters:
    """IterativeSolverParameters (auxilliary/parameters.hh:130-147)."""
    rtol: float = 1.0e-10
    atol: float = 1.0e-10
    maxiter: int = 100
    verbose: int = 0


class MultigridPreconditioner:
    """MultigridPreconditioner (multigrid_preconditioner.cc:8-108) on the GPU:
    a noise-free cycle of the sampler hierarchy for ``linear_operator`` with
    the smoothers of ``params`` and a Cholesky coarse solve."""

    def __init__(self, linear_operator, params=None, ordering=MULTICOLOUR, precision=FP64, device=0):
        self.linear_operator = linear_operator
        self._s = MultigridMCSampler(linear_operator, params, ordering=ordering, precision=precision, device=device)

    def apply(self, b, x=None):
        """x = P b (x is filled in place when given)."""
        y = self._s.precondition(b)
        if x is None:
            return y
        x[:] = y
        return x

    def close(self):
        self._s.close()


class LoopSolver:
    """LoopSolver (loop_solver.cc:9-53): x = 0, then x -= P (A x - b) until
    |r| / |b| < rtol and |r| < atol or maxiter iterations."""

    def __init__(self, linear_operator, preconditioner, params=None):
        if not isinstance(preconditioner, MultigridPreconditioner):
            raise TypeError("the GPU loop solver runs with a MultigridPreconditioner")
        if preconditioner.linear_operator is not linear_operator:
            raise ValueError("preconditioner built for another operator")
        self.linear_operator = linear_operator
        self.preconditioner = preconditioner
        self.params = params or IterativeSolverParameters()
        self.niter, self.rnorm, self.converged = 0, -1.0, False

    def apply(self, b, x=None):
        p = self.params
        y, self.niter, self.rnorm, self.converged = self.preconditioner._s.solve(b, p.rtol, p.atol, p.maxiter)
        if p.verbose >= 1:
            if self.converged:
                print(f"Solver converged after {self.niter:5d} iterations\n||r|| = {self.rnorm:8.3e}")
            else:
                print(f"Solver failed to converge after {p.maxiter:5d} iterations")
        if x is None:
            return y
        x[:] = y
        return x
