/*
 * mgmc_gb300.h -- C ABI of the GB300 Multigrid Monte Carlo sampler.
 *
 * The library samples the Gaussian distribution
 *
 *     pi(x) ~ exp(-1/2 x^T A x + f^T x),   A = A_0 + B Sigma^{-1} B^T,
 *
 * where A_0 is a constant-coefficient stencil operator on a structured
 * 1d/2d/3d lattice with homogeneous Dirichlet boundaries and B is a sparse
 * n x m measurement matrix.  It replaces the reference's sampler classes:
 *
 *   mgmc_sampler_create      MultigridMCSampler ctor  src/sampler/multigridmc_sampler.cc:8-106
 *                            (nlevel == 1 with coarse_solver SSOR gives
 *                            SSORSampler, src/sampler/ssor_sampler.hh:29-37;
 *                            with coarse_solver CHOLESKY the dense
 *                            CholeskySampler, src/sampler/cholesky_sampler.cc:25-37)
 *   mgmc_sampler_apply       Sampler::apply(f, x)     src/sampler/sampler.hh:52-55,
 *                                                     multigridmc_sampler.cc:139-145
 *   mgmc_sampler_fix_rhs     Sampler::fix_rhs         src/sampler/sampler.hh:64-71
 *   mgmc_level_apply         LinearOperator::apply    src/linear_operator/linear_operator.hh:78-88
 *   mgmc_level_restrict      IntergridOperator::restrict        src/intergrid/intergrid_operator.hh:74-88
 *   mgmc_level_prolongate_add IntergridOperator::prolongate_add src/intergrid/intergrid_operator.hh:106-120
 *   mgmc_level_sor           SORSampler::apply / SORSmoother::apply
 *                                                     src/sampler/sor_sampler.cc:37-59,
 *                                                     src/smoother/sor_smoother.cc:40-78
 *   mgmc_fd_stencil          ShiftedLaplaceFDOperator src/linear_operator/shiftedlaplace_fd_operator.cc:9-57
 *   mgmc_measurement_vector  MeasuredOperator::measurement_vector
 *                                                     src/linear_operator/measured_operator.cc:69-171
 *   mgmc_galerkin_stencil    LinearOperator::coarsen  src/linear_operator/linear_operator.cc:10-23
 *   mgmc_operator_coarsen    LinearOperator::coarsen  src/linear_operator/linear_operator.cc:10-23
 *                            (the whole operator: stencil or field, B_c = R B)
 *   mgmc_sampler_precondition MultigridPreconditioner::apply src/preconditioner/multigrid_preconditioner.cc:102-108
 *   mgmc_sampler_solve       LoopSolver::apply        src/solver/loop_solver.cc:9-53
 *
 * Conventions
 *  - Every entry point returns an mgmc_status; none exits, throws or traps
 *    (the reference calls exit(-1) on errors).  mgmc_last_error() gives a
 *    message for the calling thread.
 *  - Vectors crossing the ABI are FP64 in the reference's vertex order
 *    (lexicographic, x fastest, interior vertices only,
 *    src/lattice/lattice3d.hh:118-141).  Pointers are host pointers unless the
 *    argument `on_device` is non-zero, in which case they are device
 *    pointers of the GPU the sampler was created on.
 *  - A sampler is not thread-safe (the reference's samplers keep mutable
 *    work vectors too); use one sampler per host thread.  All of a sampler's
 *    GPU work runs on its own CUDA stream (mgmc_sampler_stream).
 */
#ifndef MGMC_GB300_H
#define MGMC_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MGMC_ABI_VERSION 2

typedef enum mgmc_status {
    MGMC_OK = 0,
    MGMC_ERR_INVALID_ARGUMENT = 1,
    MGMC_ERR_LATTICE = 2,          /* extent odd / nothing left to coarsen (lattice3d.hh:248-263) */
    MGMC_ERR_NOT_SPD = 3,          /* coarse precision matrix not positive definite */
    MGMC_ERR_CUDA = 4,             /* a CUDA runtime call failed */
    MGMC_ERR_OUT_OF_MEMORY = 5,
    MGMC_ERR_NOISE_EXHAUSTED = 6,  /* injected-noise mode: not enough normals queued */
    MGMC_ERR_NONFINITE = 7,        /* NaN/Inf seen in the chain state */
    MGMC_ERR_UNSUPPORTED = 8
} mgmc_status;

/* sweep ordering */
enum {
    MGMC_ORDER_LEXICOGRAPHIC = 0, /* the reference's order (sor_smoother.cc:66-76), run as a hyperplane wavefront */
    MGMC_ORDER_MULTICOLOUR = 1    /* 2 colours for axis-only stencils, 2^dim colours otherwise */
};
/* arithmetic */
enum {
    MGMC_FP64 = 0,      /* every level in FP64 */
    MGMC_FP32_MIXED = 1 /* sweeps, residuals, transfers in FP32; coarse Cholesky factor FP64; m x m system float-float */
};
/* noise source */
enum {
    MGMC_NOISE_PHILOX = 0,  /* counter-based Philox4x32-10 normals generated inside the kernels */
    MGMC_NOISE_INJECTED = 1 /* caller-supplied N(0,1) values consumed in the reference's draw order */
};
/* smoother / coarse solver (MultigridParameters, src/auxilliary/parameters.hh:150-179) */
enum { MGMC_SMOOTHER_SOR = 0, MGMC_SMOOTHER_SSOR = 1 };
enum { MGMC_COARSE_CHOLESKY = 0, MGMC_COARSE_SSOR = 1 };
enum { MGMC_FORWARD = 1, MGMC_BACKWARD = 2 }; /* Direction, src/smoother/sor_smoother.hh:14-18 */

/* Problem: lattice, fine-level stencil and the optional low-rank term. */
typedef struct mgmc_operator_desc {
    int dim;            /* 1, 2 or 3 */
    int nx, ny, nz;     /* cells per direction (unused directions ignored); n = prod (n_d - 1) unknowns */
    double stencil[27]; /* constant fine-level stencil, entry (dz+1)*9 + (dy+1)*3 + (dx+1) */
    int m;              /* number of measurement columns, 0 for none */
    const int64_t *B_colptr; /* m+1 column pointers of B (CSC, row indices ascending) */
    const int64_t *B_rowidx; /* vertex indices in the reference's order */
    const double *B_val;
    const double *Sigma;     /* m diagonal entries of the measurement covariance */
    /* Optional per-vertex centre weight of the fine stencil (n values in the
     * reference's vertex order), replacing stencil[13]: the FD prior with a
     * variable correlation length, diagonal h^d kappa^2(x) + sum_d 2 h^d / h_d^2
     * (shiftedlaplace_fd_operator.cc:33-52, correlationlength_model.hh:83-112).
     * The coarse levels then carry per-point 27-point Galerkin stencils.
     * Needs dim >= 2 and MGMC_ORDER_MULTICOLOUR; NULL for a constant stencil. */
    const double *centre;
    /* Optional per-vertex 27-point stencil of the fine level, weight-major
     * (weight k of vertex p at field[k * n + p], k as in `stencil`): the FEM
     * prior with a variable correlation length (mgmc_fem_field).  Takes
     * precedence over stencil and centre; `stencil` should still hold a
     * representative stencil (it sets the colouring).  Needs dim >= 2 and
     * MGMC_ORDER_MULTICOLOUR; NULL otherwise. */
    const double *field;
} mgmc_operator_desc;

/* Sampler parameters: MultigridParameters plus the GB300 execution choices. */
typedef struct mgmc_sampler_params {
    int nlevel;
    int smoother;      /* MGMC_SMOOTHER_SOR | MGMC_SMOOTHER_SSOR */
    int coarse_solver; /* MGMC_COARSE_CHOLESKY | MGMC_COARSE_SSOR */
    int npresmooth;
    int npostsmooth;
    int ncoarsesmooth;
    double omega;
    int cycle;         /* 1 = V-cycle, 2 = W-cycle */
    double coarse_scaling;
    int ordering;      /* MGMC_ORDER_* */
    int precision;     /* MGMC_FP64 | MGMC_FP32_MIXED */
    int noise;         /* MGMC_NOISE_* */
    uint64_t seed;     /* Philox key */
    int device;        /* CUDA device ordinal */
} mgmc_sampler_params;

typedef struct mgmc_sampler mgmc_sampler;

/* ---------------------------------------------------------------- info */
int mgmc_abi_version(void);
const char *mgmc_last_error(void);

/* -------------------------------------------------------- host set-up */
/* ShiftedLaplaceFDOperator stencil (shiftedlaplace_fd_operator.cc:9-57):
 * diag h^d kappa^2 + sum_d 2 h^d / h_d^2, neighbours -h^d / h_d^2. */
mgmc_status mgmc_fd_stencil(int dim, int nx, int ny, int nz, double kappa_sq, double stencil[27]);
/* MeasuredOperator::measurement_vector (measured_operator.cc:69-171): FE
 * quadrature of 1{|x-x0|<R}/V_d(R); radius < 1e-12 selects the nearest
 * vertex.  Writes at most `capacity` entries and sets *nnz to the count. */
mgmc_status mgmc_measurement_vector(int dim, int nx, int ny, int nz, const double *x0, double radius,
                                    int64_t *idx, double *val, int64_t capacity, int64_t *nnz);
/* ShiftedLaplaceFEMOperator (shiftedlaplace_fem_operator.cc:9-152): Q1
 * elements, 2-point Gauss-Legendre quadrature per direction; kappa^2
 * constant (model 0, p0 = kappa^2) or from the periodic correlation length
 * (model 1, p0 = Lambda_min, p1 = Lambda_max).  Writes the weight-major
 * per-vertex stencils (27 x n values) to field. */
mgmc_status mgmc_fem_field(int dim, int nx, int ny, int nz, int model, double p0, double p1, double *field);
/* Galerkin triple product R A R^T of a constant stencil with the linear
 * intergrid operator (linear_operator.cc:10-23, intergrid_operator_linear.cc:8-31). */
mgmc_status mgmc_galerkin_stencil(int dim, const double fine[27], double coarse[27]);
/* LinearOperator::coarsen (linear_operator.cc:10-23) of a whole operator on
 * the host: the coarse lattice has half the cells per direction; its
 * stencil R A R^T goes to coarse_stencil, and for a per-vertex operator
 * (op->centre or op->field set) its per-vertex Galerkin stencils, 27 x n_c
 * weight-major, go to coarse_field (required then, ignored otherwise);
 * B_c = R B (CSC, row indices ascending) goes to Bc_colptr (m+1 entries) and
 * Bc_rowidx / Bc_val (cap entries each).  *nnz receives nnz(B_c); call with
 * Bc_rowidx = Bc_val = NULL to size them.  Sigma is unchanged. */
mgmc_status mgmc_operator_coarsen(const mgmc_operator_desc *op, double coarse_stencil[27], double *coarse_field,
                                  int64_t *Bc_colptr, int64_t *Bc_rowidx, double *Bc_val, int64_t cap,
                                  int64_t *nnz);

/* ------------------------------------------------------------- sampler */
/* The device keeps the low-rank term's indices in 32 bits: with m > 0, a
 * lattice whose padded level array (nx ny (nz + 2) + 32 entries for
 * nx x ny x nz cells, about 4.1e9 for 1600^3 cells) exceeds 2^32 - 1
 * entries is refused with MGMC_ERR_UNSUPPORTED. */
mgmc_status mgmc_sampler_create(const mgmc_operator_desc *op, const mgmc_sampler_params *params,
                                mgmc_sampler **out);
mgmc_status mgmc_sampler_destroy(mgmc_sampler *s);
/* One sample: x <- MGMC step(f, x), both length n.  f == NULL: step with
 * the right hand side already on the device (the last one given to
 * mgmc_sampler_fix_rhs or mgmc_sampler_apply; MGMC_ERR_INVALID_ARGUMENT if
 * there is none), so that only x crosses the host link -- the
 * fix_rhs-then-apply loop of measure_sampling_time
 * (src/measurements/sampling_time.cc:28-41). */
mgmc_status mgmc_sampler_apply(mgmc_sampler *s, const double *f, double *x, int on_device);
/* Keep f on the device for mgmc_sampler_step. */
mgmc_status mgmc_sampler_fix_rhs(mgmc_sampler *s, const double *f, int on_device);
mgmc_status mgmc_sampler_set_state(mgmc_sampler *s, const double *x, int on_device);
mgmc_status mgmc_sampler_get_state(mgmc_sampler *s, double *x, int on_device);
/* nsteps samples with the state and right hand side resident on the GPU;
 * asynchronous on the sampler's stream. */
mgmc_status mgmc_sampler_step(mgmc_sampler *s, int64_t nsteps);
/* Observable z_k = b^T x after every step (measure_sampling_time,
 * src/measurements/sampling_time.cc:37-41); up to `capacity` values are
 * kept on the device until read. */
mgmc_status mgmc_sampler_set_observable(mgmc_sampler *s, int64_t nnz, const int64_t *idx, const double *val,
                                        int64_t capacity);
/* Several observables at once: probe p is b_p (entries ptr[p]..ptr[p+1] of
 * idx/val); after every step the nprobe values are appended, step-major.
 * Replaces any observable set before. */
mgmc_status mgmc_sampler_set_probes(mgmc_sampler *s, int nprobe, const int64_t *ptr, const int64_t *idx,
                                    const double *val, int64_t capacity);
/* Copies min(count, capacity / nprobe) steps of observations into out
 * (step-major, nprobe values per step), sets *count to the number of steps
 * recorded since the last read and starts a new record. */
mgmc_status mgmc_sampler_read_observations(mgmc_sampler *s, double *out, int64_t capacity, int64_t *count);
/* Injected-noise mode: queue `count` N(0,1) values; each step consumes
 * mgmc_sampler_noise_per_step() of them in the reference's draw order. */
mgmc_status mgmc_sampler_inject_noise(mgmc_sampler *s, const double *normals, int64_t count, int on_device);
mgmc_status mgmc_sampler_noise_per_step(mgmc_sampler *s, int64_t *count);
mgmc_status mgmc_sampler_synchronize(mgmc_sampler *s);
mgmc_status mgmc_sampler_stream(mgmc_sampler *s, void **cuda_stream);
mgmc_status mgmc_sampler_nlevel(mgmc_sampler *s, int *nlevel);
mgmc_status mgmc_sampler_level_size(mgmc_sampler *s, int level, int64_t *n);
/* The step counter that keys the Philox noise (the number of steps taken
 * since creation); setting it lets a chain segment be recomputed from a
 * checkpoint with its original noise.  No counterpart in the reference. */
mgmc_status mgmc_sampler_set_step_counter(mgmc_sampler *s, int64_t step);
mgmc_status mgmc_sampler_get_step_counter(mgmc_sampler *s, int64_t *step);
/* Number of kernel launches one step issues (measurement bookkeeping). */
mgmc_status mgmc_sampler_launches_per_step(mgmc_sampler *s, int64_t *count);
/* Adjoint of one step with its noise held fixed (no counterpart in the
 * reference; pathwise differentiation of chain functionals).  A step is
 * affine in the state and the right hand side, x' = Phi x + K f + noise
 * terms; on entry xbar (n values) holds the adjoint of x', on return the
 * adjoint of x, Phi^T xbar, and K^T xbar has been added to fbar (n values).
 * Vectors in the reference's vertex order, host (on_device = 0) or device
 * pointers.  Gradients with respect to the measurement values y follow
 * through f = B Sigma^{-1} y. */
mgmc_status mgmc_sampler_adjoint_step(mgmc_sampler *s, double *xbar, double *fbar, int on_device);
/* Adjoint of one step with respect to the parameters as well (no
 * counterpart in the reference).  Replays the step from x_in (n values)
 * with the sampler's fixed right hand side and the step's noise -- the
 * next mgmc_sampler_noise_per_step() injected values, which it consumes
 * like a step, or with Philox noise the noise of the step taken when the
 * step counter was step_index (0 for the first step after creation) --
 * records its intermediate states, and then, as mgmc_sampler_adjoint_step,
 * turns xbar into the adjoint of x_in and adds K^T xbar to fbar.  It also
 * adds to *g_centre the derivative of xbar^T x_out with respect to the
 * fine stencil's centre weight (the FD prior's centre weight is
 * h^d kappa^2 + const, so d/dkappa^2 = h^d d/dcentre; coarse stencils
 * follow by Galerkin coarsening) and to g_logsigma[k] (m values) the
 * derivative with respect to log Sigma_k, both with the right hand side
 * held fixed (f = B Sigma^{-1} y adds -(B^T fbar)_k y_k / Sigma_k).
 * g_centre and g_logsigma are host pointers; x_in, xbar and fbar follow
 * on_device.  The chain's state is left unchanged. */
mgmc_status mgmc_sampler_adjoint_params(mgmc_sampler *s, const double *x_in, int64_t step_index, double *xbar,
                                        double *fbar, double *g_centre, double *g_logsigma, int on_device);

/* ------------------------------------------------ deterministic solver */
/* MultigridPreconditioner::apply (src/preconditioner/multigrid_preconditioner.cc:102-108):
 * x = P b, one cycle of the sampler's hierarchy with the noise switched off,
 * from x = 0 on every level (:76), with the SOR/SSOR smoothers of
 * multigrid_preconditioner.cc:17-35 and a Cholesky coarse solve whatever
 * the sampler's coarse_solver (:41-46).  Computed in the sampler's
 * precision.  The chain's state and right hand side are left unchanged. */
mgmc_status mgmc_sampler_precondition(mgmc_sampler *s, const double *b, double *x, int on_device);
/* LoopSolver::apply (src/solver/loop_solver.cc:9-53) with that
 * preconditioner: x = 0; for k < maxiter: r = A x - b, stop when
 * |r| / |b| < rtol and |r| < atol, else x -= P r.  The iterate and the
 * residual are FP64 whatever the sampler's precision (an FP32-mixed
 * sampler gives mixed-precision iterative refinement).  On return *niter is
 * the iteration at which the test passed (maxiter when it never did),
 * *rnorm the last residual norm (-1 when maxiter = 0) and *converged 0 or
 * 1; not converging is not an error (the reference only reports it).  The
 * chain's state and right hand side are left unchanged. */
mgmc_status mgmc_sampler_solve(mgmc_sampler *s, const double *b, double *x, double rtol, double atol, int maxiter,
                               int on_device, int *niter, double *rnorm, int *converged);
/* Exact sampler, the comparator of SparseCholeskySampler / DenseCholeskySampler
 * (src/sampler/cholesky_sampler.cc:9-37) at sizes a factorisation does not
 * reach: x = Q^{-1}(f + eta) with eta ~ N(0, Q), Q = A_0 + B Sigma^{-1} B^T,
 * is an exact draw from N(Q^{-1} f, Q^{-1}).  eta is drawn in-kernel (Philox
 * keyed by the sampler's seed and step counter, which the call advances by
 * one) from an edge decomposition of A_0 -- which needs a symmetric stencil
 * with non-positive off-diagonal weights and weak diagonal dominance (the
 * FD prior has it; otherwise MGMC_ERR_UNSUPPORTED) -- plus B Sigma^{-1/2} xi;
 * the system is solved by mgmc_sampler_solve's loop to relative residual
 * rtol (MGMC_ERR_NONFINITE if maxiter iterations do not reach it).  The
 * sample does not depend on the chain's state, which is left unchanged.
 * *niter (may be NULL) receives the iteration count. */
mgmc_status mgmc_sampler_exact_sample(mgmc_sampler *s, const double *f, double *x, double rtol, int maxiter,
                                      int on_device, int *niter);

/* -------------------------------------------- level building blocks */
mgmc_status mgmc_level_stencil(mgmc_sampler *s, int level, double stencil[27]);
/* y = A x on level `level` (including B Sigma^{-1} B^T x). */
mgmc_status mgmc_level_apply(mgmc_sampler *s, int level, const double *x, double *y);
/* xc = R x from `level` to level+1. */
mgmc_status mgmc_level_restrict(mgmc_sampler *s, int level, const double *x, double *xc);
/* x += alpha P xc from level+1 to `level`. */
mgmc_status mgmc_level_prolongate_add(mgmc_sampler *s, int level, double alpha, const double *xc, double *x);
/* One SOR sweep in `direction` with the low-rank update: with_noise != 0
 * is SORSampler::apply (noise from the sampler's source), 0 is
 * SORSmoother::apply with right hand side f. */
mgmc_status mgmc_level_sor(mgmc_sampler *s, int level, int direction, int with_noise, const double *f, double *x);
/* `nrepeat` SOR sweeps on the level's device-resident state and right hand
 * side (SORSampler::apply, sor_sampler.cc:37-59), asynchronous on the
 * sampler's stream; with_lowrank == 0 runs the stencil sweep kernels only.
 * Used to time the sweep kernels in isolation. */
mgmc_status mgmc_level_sweep_device(mgmc_sampler *s, int level, int direction, int with_noise, int with_lowrank,
                                    int64_t nrepeat);
/* `nrepeat` residual-restrictions from `level` to level+1 (which = 0: f_{l+1} =
 * R (f - A x), with the low-rank term; multigridmc_sampler.cc:124-126) or
 * prolongations (which = 1: x += alpha P x_{l+1}, :131) on the levels'
 * device-resident vectors, asynchronous on the sampler's stream.  Used to time
 * the transfer kernels in isolation; the residual-restriction also zeroes
 * the coarse state. */
mgmc_status mgmc_level_transfer_device(mgmc_sampler *s, int level, int which, int64_t nrepeat);

/* ----------------------------------------------------------------- batch */
/* Many independent chains (the reference's only parallel mode: independent
 * chains per OpenMP thread, src/measurements/convergence.cc:29-78) stepped
 * together.  Chains that share a lattice geometry and a step structure
 * (FP32-mixed, MGMC_NOISE_PHILOX, multicolour order, SSOR smoother,
 * Cholesky coarse solver, constant stencils, 3D) form groups whose step is
 * one sequence of batched launches -- every launch covers all chains of
 * the group; every other chain runs its own step graph; all of it is one
 * CUDA graph launch per step.  A chain follows bit for bit the chain it
 * follows when stepped alone.  Chains keep their own state, right hand
 * side and observables; they must use MGMC_NOISE_PHILOX and one device.
 * Set observables (mgmc_sampler_set_observable / _set_probes) before
 * creating the batch.  The samplers must outlive the batch; while it
 * exists, step them only through mgmc_batch_step. */
typedef struct mgmc_batch mgmc_batch;
mgmc_status mgmc_batch_create(int nchain, mgmc_sampler *const *samplers, mgmc_batch **out);
mgmc_status mgmc_batch_step(mgmc_batch *b, int64_t nsteps);
/* No counterpart in the reference: the number of batched groups and of the
 * chains they hold (the rest step through their own graphs). */
mgmc_status mgmc_batch_info(mgmc_batch *b, int *ngroups, int *ngrouped);
mgmc_status mgmc_batch_synchronize(mgmc_batch *b);
mgmc_status mgmc_batch_stream(mgmc_batch *b, void **cuda_stream);
mgmc_status mgmc_batch_destroy(mgmc_batch *b);

/* ------------------------------------------- low-rank Cholesky sampler */
/* LowRankCholeskySampler (src/sampler/cholesky_sampler.cc:41-129,
 * cholesky_sampler.hh:173-267): the exact comparator of the reference's
 * summary study.  Created from an operator with a constant stencil (a
 * per-vertex centre or field: MGMC_ERR_UNSUPPORTED); the Cholesky factor
 * of A_0 is computed once on the host in FP64, block by block along the
 * last lattice direction (A_0 is block tridiagonal there: planes in 3D),
 * with the reference's low-rank correction (V = L^{-1} B = Q R, the factor
 * W of Id - R (Sigma + V^T V)^{-1} R^T); samples are drawn on the GPU in
 * FP64: n normals (noise MGMC_NOISE_PHILOX, key `seed`, or
 * MGMC_NOISE_INJECTED in the reference's draw order), g = L^{-1} f
 * corrected by the low-rank factors, x = L^{-T}(xi + g) corrected likewise.
 * The host set-up costs about 2 nb p^3 flops (nb blocks of p vertices) and
 * the device holds 2 nb p^2 + 3 n m doubles.  apply: x <- a sample (x's
 * input value is not used); f == NULL samples with the fixed f. */
typedef struct mgmc_lrchol mgmc_lrchol;
mgmc_status mgmc_lrchol_create(const mgmc_operator_desc *op, int noise, uint64_t seed, int device, mgmc_lrchol **out);
mgmc_status mgmc_lrchol_destroy(mgmc_lrchol *s);
/* LowRankCholeskySampler::fix_rhs (cholesky_sampler.cc:117-129) */
mgmc_status mgmc_lrchol_fix_rhs(mgmc_lrchol *s, const double *f, int on_device);
/* LowRankCholeskySampler::apply (cholesky_sampler.cc:86-115) */
mgmc_status mgmc_lrchol_apply(mgmc_lrchol *s, const double *f, double *x, int on_device);
mgmc_status mgmc_lrchol_inject_noise(mgmc_lrchol *s, const double *normals, int64_t count);
mgmc_status mgmc_lrchol_stream(mgmc_lrchol *s, void **cuda_stream);

/* ------------------------------------------------------------ diagnostics */
/* No counterpart in the reference.  Measured FMA throughput of the current
 * GPU in TFLOP/s (2 flop per FMA), FP64 (precision = MGMC_FP64) or FP32
 * (MGMC_FP32_MIXED): full occupancy, eight independent FMA chains per
 * thread, about 20 ms per timed launch, best of three, CUDA events.  It
 * bounds the kernels whose flops per byte exceed the HBM roofline's; it
 * changes no clock or other setting of the GPU. */
mgmc_status mgmc_device_fma_rate(int precision, double *tflops);

/* ------------------------------------------- no-allocation operator apply */
/* No counterpart in the reference.  y = A x for A = A_0 + B Sigma^{-1} B^T
 * without allocating device memory, for callers that cannot call
 * cudaMalloc: work captured into a CUDA graph in global capture mode,
 * applications whose device memory is owned by their own pool and lent to
 * the library buffer by buffer, and latency-critical loops that cannot
 * afford cudaMalloc's device-wide synchronisation.
 * A_0 must be one constant 27-point stencil for every vertex (`stencil`, a
 * host array); operators with a per-vertex centre or a per-vertex stencil
 * field are not handled here.  B_colptr/B_rowidx/B_val (column-compressed,
 * as in mgmc_operator_desc), Sigma, x and y are device pointers of the
 * current device, vectors in the reference's vertex order.  Work is queued
 * on `cuda_stream` (NULL = default stream) and the call returns without
 * waiting for it.  A_0 x is summed per row in ascending index order; the
 * low-rank part is added with atomics, so its order, and the last bits of
 * y, can change from run to run.  A CUDA error pending from earlier work is
 * reported (MGMC_ERR_CUDA) and left in place.
 * The only scratch, B^T x, lives in a static device array of
 * MGMC_NOALLOC_MAX_M doubles (32 KiB) that every GPU loading the library
 * holds until the process exits; m > MGMC_NOALLOC_MAX_M is rejected with
 * MGMC_ERR_INVALID_ARGUMENT.  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress) and loads the entry point's
 * kernels; make that first call before any stream capture.  All calls on a
 * device share the array: calls that overlap on the GPU race and must be
 * ordered by the caller. */
#define MGMC_NOALLOC_MAX_M 4096
mgmc_status mgmc_measured_apply_noalloc(int dim, int nx, int ny, int nz, const double stencil[27], int m,
                                        const int64_t *B_colptr, const int64_t *B_rowidx, const double *B_val,
                                        const double *Sigma, const double *x, double *y, void *cuda_stream);

#ifdef __cplusplus
}
#endif

#endif /* MGMC_GB300_H */
