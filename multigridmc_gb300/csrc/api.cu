// api.cu -- C ABI, hierarchy set-up and step orchestration of the GB300
// Multigrid Monte Carlo sampler.
//
// One mgmc_sampler owns one chain: the level hierarchy (stencils, B, the
// low-rank factors C = M^{-1} B, the coarse Cholesky factor) and the chain
// state stay resident in device memory; a step is a fixed sequence of
// kernel launches on the sampler's stream, captured once into a CUDA graph
// when the noise comes from the in-kernel Philox generator.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#include "../../include/mgmc_gb300.h"
#include "kernels.cuh"
#include "setup.h"

namespace mgmc {

static thread_local std::string g_err;

void set_last_error(const std::string &msg) { g_err = msg; }

struct Error {
    mgmc_status st;
    std::string msg;
};

#define CK(call)                                                                                         \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess)                                                                           \
            throw Error{e_ == cudaErrorMemoryAllocation ? MGMC_ERR_OUT_OF_MEMORY : MGMC_ERR_CUDA,          \
                        std::string(#call) + ": " + cudaGetErrorString(e_)};                           \
    } while (0)

static void fail(mgmc_status st, const std::string &msg) { throw Error{st, msg}; }

template <typename P>
static P *dalloc(size_t count) {
    void *p = nullptr;
    if (count == 0) count = 1;
    CK(cudaMalloc(&p, count * sizeof(P)));
    return (P *)p;
}

template <typename P>
static P *dupload(const std::vector<P> &v, cudaStream_t s) {
    P *p = dalloc<P>(v.size());
    if (!v.empty()) CK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(P), cudaMemcpyHostToDevice, s));
    return p;
}

// v as float-float pairs hi + lo: hi = v rounded to FP32, lo = the
// remainder rounded to FP32 (about 48 significant bits in all)
static std::vector<float2> float_float(const std::vector<double> &v) {
    std::vector<float2> r(v.size());
    for (size_t i = 0; i < v.size(); ++i) {
        const float hi = (float)v[i];
        r[i] = make_float2(hi, (float)(v[i] - (double)hi));
    }
    return r;
}

static inline unsigned nblk(i64 n, int bs) { return (unsigned)std::max<i64>(1, (n + bs - 1) / bs); }

// Row-compressed sparse n x m matrix over its support rows (padded indices).
struct RowCsr {
    i64 nrows = 0;
    i64 *rows = nullptr, *ptr = nullptr;
    int *col = nullptr;
    void *val = nullptr;  // T for C, double for B
};

struct Level {
    Geometry geo;
    Grid3 g;
    double st[27];
    int ncol = 2, npt = 7;
    double diag = 0, sd = 0;
    void *x = nullptr, *f = nullptr;    // state and right hand side (T, padded)
    void *s1 = nullptr, *s2 = nullptr;  // scratch for the building-block calls
    SparseCols Bh;                      // B on this level (compact indices)
    i64 *Bptr = nullptr;
    unsigned *Bidx = nullptr;  // padded indices of B's entries
    double *Bval = nullptr;
    RowCsr Br;          // B by rows (double values)
    CorrRows C[2];      // C = M^{-1} B, forward / backward (T values)
    double *SinvT[2] = {nullptr, nullptr};  // S^{-1} transposed, per sweep direction
    float2 *SinvT_ff[2] = {nullptr, nullptr};  // the same as float-float pairs (FP32 chain)
    double *y = nullptr, *z = nullptr, *part = nullptr;
    float *zf = nullptr, *Bvalf = nullptr;
    int bt_split = 1;  // blocks per column of the B^T x reduction
    unsigned *counter = nullptr;  // CTA counter of k_bt_solve
    int sweep_tx = 0;             // CTA width of the colour passes chosen by the autotuner (0: sweep_block())
    int sweep_threads = 0;        // and its thread count, 128 or 256 (0: RBP_THREADS)
    void *adj[4] = {nullptr, nullptr, nullptr, nullptr};  // adjoint: x-bar, f-bar, two work vectors (T, padded)
    CUtensorMap xmap{}, fmap{};  // 3D tile maps of x and f for the residual-restriction
    bool tma = false;            // maps valid (3D, rows of a multiple of 16 bytes)
    // variable coefficients: 0 the constant stencil st; 1 a per-point centre
    // weight (the fine level of a variable-coefficient prior); 2 a per-point
    // 27-point stencil (its Galerkin coarse levels), weight-major with stride nalloc
    int var = 0;
    void *vw = nullptr;        // the field in the level's type (padded, ghosts zero)
    double *vw64 = nullptr;    // the field in FP64 (vw itself for FP64 chains): FP64 kernels of FP32
                               // chains (set-up sweeps, solver residual, exact sampler) read it
    std::vector<double> vh;    // host field, compact: n centre weights or 27 x n weights
};

// the level's field in the kernel's type T
template <typename T>
static VarField<T> var_field(const Level &lv) {
    const void *w = sizeof(T) == sizeof(double) ? (const void *)lv.vw64 : lv.vw;
    return VarField<T>{(const T *)w, lv.geo.nalloc};
}

struct Sampler {
    mgmc_sampler_params P;
    int dim = 3, m = 0;
    bool fp32 = false, exact = false;
    int nsm = 152;    // SMs of the device
    bool pdl = true;  // programmatic dependent launch between step kernels (MGMC_NO_PDL=1 turns it off)
    int noise_mode = NOISE_PHILOX;
    std::vector<Level> L;
    std::vector<double> Sigma;
    double *d_sigma_inv = nullptr, *d_sigma_sqrt = nullptr;
    float2 *d_sigma_sqrt_ff = nullptr;  // Sigma^{1/2} as float-float pairs (FP32 chain)
    // coarse Cholesky
    bool chol = false;
    double *dL = nullptr, *dgv = nullptr;
    void *dLinv = nullptr, *dLinvT = nullptr;  // L^{-1}, L^{-T}: double (FP64 chain) or float (FP32 chain)
    int chol_ld = 0;                           // their leading dimension (16-byte rows)
    size_t chol_smem = 0;
    // bookkeeping
    cudaStream_t stream = nullptr;
    u64 *d_step = nullptr, *d_obs_count = nullptr;
    unsigned *d_err = nullptr;
    double *d_obs = nullptr;
    i64 obs_cap = 0;
    int nprobe = 0;
    i64 *d_bptr = nullptr, *d_bidx = nullptr;
    double *d_bval = nullptr;
    unsigned *d_done = nullptr;
    double *d_cvec = nullptr;  // compact n_0 doubles for transfers
    // injected noise queue
    double *d_noise = nullptr;
    i64 noise_cap = 0, noise_len = 0, noise_pos = 0, noise_per_step = 0;
    // step construction
    unsigned inv = 0;
    i64 noise_off = 0;
    i64 launches = 0;       // kernel launches counted while a sequence is issued
    i64 step_launches = 0;  // ... of the last step issued by launch_step
    bool counting = false;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    // level 0's f split by colour for the FP32 fine sweep (k_split_colours):
    // colour k at fsplit + k * fhalf; refreshed wherever level 0's f changes
    float *fsplit = nullptr;
    i64 fhalf = 0;
    bool rhs_set = false;  // level 0's f was given (fix_rhs or apply): apply may take f = NULL
    void refresh_fsplit();
    // deterministic solver: LoopSolver around MultigridPreconditioner
    bool noisy = true;  // false while the preconditioner's noise-free cycle is recorded
    double *sv_x = nullptr, *sv_b = nullptr, *sv_r = nullptr;  // FP64 iterate, rhs, residual (padded level 0)
    double *sv_part = nullptr, *sv_norm = nullptr;             // |r|^2 partial sums and total
    int sv_np = 0;
    void *sv_keep_x = nullptr, *sv_keep_f = nullptr;  // the chain's x_0 and f_0 while a solve borrows them
    cudaGraph_t rgraph = nullptr, pgraph = nullptr;   // residual + norm; preconditioner cycle
    cudaGraphExec_t rexec = nullptr, pexec = nullptr;
    std::vector<void *> owned;  // every device allocation

    template <typename P_>
    P_ *alloc(size_t count) {
        P_ *p = dalloc<P_>(count);
        owned.push_back(p);
        return p;
    }
    // free an allocation of this sampler before the sampler ends
    void release(void *p) {
        auto it = std::find(owned.begin(), owned.end(), p);
        if (it != owned.end()) {
            cudaFree(p);
            owned.erase(it);
        }
    }
    template <typename P_>
    P_ *upload(const std::vector<P_> &v) {
        P_ *p = dupload(v, stream);
        owned.push_back(p);
        return p;
    }
    size_t tsize() const { return fp32 ? sizeof(float) : sizeof(double); }
    void *talloc(i64 count) {
        void *p = alloc<char>((size_t)count * tsize());
        CK(cudaMemsetAsync(p, 0, (size_t)count * tsize(), stream));
        return p;
    }
    ~Sampler() {
        if (gexec) cudaGraphExecDestroy(gexec);
        if (graph) cudaGraphDestroy(graph);
        if (rexec) cudaGraphExecDestroy(rexec);
        if (rgraph) cudaGraphDestroy(rgraph);
        if (pexec) cudaGraphExecDestroy(pexec);
        if (pgraph) cudaGraphDestroy(pgraph);
        if (pa_exec) cudaGraphExecDestroy(pa_exec);
        if (pa_graph) cudaGraphDestroy(pa_graph);
        for (void *p : owned) cudaFree(p);
        if (stream) cudaStreamDestroy(stream);
    }

    void build(const mgmc_operator_desc &op);
    void build_lowrank(int lev);
    void make_tile_maps(Level &lv);
    double *adj_m = nullptr;  // m-vector for the adjoint's transposed low-rank solve
    void ensure_adjoint();
    // parameter adjoint: a replay of one step records the input and output
    // state of every sweep, the state entering each residual and every
    // level's right hand side (the tape); the reverse pass then adds each
    // event's derivative with respect to the fine centre weight and log Sigma
    enum { EV_SWEEP = 0, EV_RESID = 1, EV_COARSE = 2 };
    struct TapeEvent {
        int kind, lev;
        bool forward;
        void *xin, *xout, *f;
        NoiseArgs nzp, nzl;  // point (coarse) and low-rank noise of the event
    };
    bool taping = false, param_adj = false;
    std::vector<TapeEvent> tape;
    std::vector<std::vector<void *>> tape_pool;  // snapshot buffers per level
    std::vector<int> tape_next;
    std::vector<void *> tape_last;  // latest snapshot of the level's state (null once it changed)
    std::vector<void *> tape_f;     // snapshot of the level's current right hand side
    std::vector<std::array<double, 27>> pa_E;  // dA_0/ds on every level
    double *pa_gs = nullptr, *pa_gsig = nullptr;  // gradient accumulators
    double *pa_part = nullptr;
    int pa_part_cap = 0;
    double *pa_Bu = nullptr, *pa_Bv = nullptr, *pa_xi = nullptr, *pa_xic = nullptr, *pa_U = nullptr;
    void *pa_phi = nullptr, *pa_cv = nullptr, *pa_mu = nullptr;
    // with Philox noise every launch of the replay and the reverse pass has
    // the same arguments at every call (the tape's buffers are reused, the
    // step enters through the device step counter): after one direct call
    // the sequence runs as one CUDA graph
    cudaGraph_t pa_graph = nullptr;
    cudaGraphExec_t pa_exec = nullptr;
    int pa_calls = 0;
    void ensure_param_adjoint();
    void param_adjoint_pass();
    void upload_field(Level &lv);
    void *tape_snap(int lev, const void *src);
    void *tape_state(int lev);
    TapeEvent tape_pop(int kind, int lev, bool forward);
    template <typename T>
    void pgrad_sweep(const TapeEvent &ev, const void *u);
    template <typename T>
    void pgrad_minus_udav(int lev, const void *u, const void *v);
    template <typename T>
    void pgrad_coarse(const TapeEvent &ev);
    void autotune_sweeps();
    template <typename T>
    void adjoint_sample(int lev);
    void build_coarse();
    std::vector<double> level_precision(const Level &lv) const;
    void launch_step();
    void sor(int lev, bool forward, bool noisy, void *x, void *f, int nsparse = 1);
    void smooth(int lev, bool forward, int nsmooth);
    void sample(int lev);
    void ensure_solver();
    void ensure_solver_buffers();
    // exact sampler: x = Q^{-1}(f + eta), eta ~ N(0, Q), by the loop solver
    EdgeWeights ew{};
    double ex_offsum = 0.0;  // sum of |off-diagonal weights| of the fine stencil
    bool ew_ready = false;
    double *ex_y = nullptr;
    void ensure_exact();
    void coarse_sample(int lev);
    void resid_restrict(int lev);
    void prolong(int lev, double alpha, void *xc, void *x);
    void step_end();
    void ensure_scratch(int lev);
    void check_launch();
    NoiseArgs noise_args(int lev, i64 count);
};

template <typename T>
static StencilArg<T> stencil_arg(const Level &lv, double omega) {
    StencilArg<T> s;
    for (int k = 0; k < 27; ++k) s.w[k] = (T)lv.st[k];
    s.diag = (T)lv.diag;
    s.omega = (T)omega;
    s.sd = (T)lv.sd;
    s.omega_diag = (T)(omega / lv.diag);
    s.tmo = (T)(2. - omega);
    return s;
}

void Sampler::check_launch() {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) fail(MGMC_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
}

NoiseArgs Sampler::noise_args(int lev, i64 count) {
    NoiseArgs nz;
    nz.buf = nullptr;
    nz.seed = P.seed;
    nz.d_step = d_step;
    nz.invocation = inv;
    nz.level = (unsigned)lev;
    if (noise_mode == NOISE_INJECTED) {
        nz.buf = d_noise + noise_off;
        noise_off += count;
    }
    return nz;
}

// Launch with programmatic stream serialization (pdl): the kernel's CTAs
// may be scheduled while its predecessor on the stream drains; every step
// kernel starts with griddepcontrol.wait (pdl_begin), so no kernel touches
// memory before its predecessor has completed and flushed.  This hides the launch latency between the short
// dependent kernels of a multigrid step.
constexpr i64 PDL_MAX_POINTS = i64(1) << 22;
// supports of C up to this many rows take the fused solve + correction
#ifndef MGMC_LR_FUSE_MAX_ROWS
#define MGMC_LR_FUSE_MAX_ROWS 200000ll
#endif
constexpr i64 LR_FUSE_MAX_ROWS = MGMC_LR_FUSE_MAX_ROWS;
// CTAs per SM of the fused solve + correction (each CTA repeats the solve)
#ifndef MGMC_LR_APPLY_CTAS_PER_SM
#define MGMC_LR_APPLY_CTAS_PER_SM 2
#endif

template <typename... KArgs, typename... Args>
static void plaunch(bool pdl, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                    Args &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    CK(cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...));
}

// Raise a kernel's dynamic shared memory limit to at least `bytes`.  The
// limit belongs to the kernel and is shared by every sampler and level of
// the process, so it is only ever raised.
template <typename... KArgs>
static void raise_smem_limit(void (*kernel)(KArgs...), size_t bytes) {
    cudaFuncAttributes fa;
    CK(cudaFuncGetAttributes(&fa, kernel));
    if ((int)bytes > fa.maxDynamicSharedSizeBytes)
        CK(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
}

// ----------------------------------------------------------- sweep launch
// CTA shape of a level's colour passes: the autotuned width, or the
// smallest power of two covering the `count` work items of a row.
static dim3 level_block(const Level &lv, int count) {
    if (lv.sweep_tx > 0) {
        const int nt = lv.sweep_threads > 0 ? lv.sweep_threads : RBP_THREADS;
        return dim3(lv.sweep_tx, nt / lv.sweep_tx, 1);
    }
    return sweep_block(count);
}

template <typename T, bool EXACT, int NOISE>
static void launch_colour_passes(Sampler &S, const Level &lv, bool forward, T *x, const T *f, const StencilArg<T> &s,
                                 const NoiseArgs &nz);

template <typename T, int NPT, bool EXACT, int NOISE>
static void launch_sweep_t(Sampler &S, const Level &lv, bool forward, T *x, const T *f, const NoiseArgs &nz) {
    StencilArg<T> s = stencil_arg<T>(lv, S.P.omega);
    if (S.P.ordering == MGMC_ORDER_LEXICOGRAPHIC) {
        int hb = lv.ncol == 2 ? 1 : 2, hc = lv.ncol == 2 ? 1 : 4;
        plaunch(S.pdl && lv.g.pdl, k_sweep_wavefront<T, NPT, EXACT, NOISE>, 1, 1024, 0, S.stream, x, f, lv.g, s, forward ? 1 : 0, hb, hc, nz);
        S.launches++;
        return;
    }
    if (NPT == 7) {
        // red-black: two passes, the second walking the planes downwards;
        // FP32 rows padded to a multiple of 4 floats use the vector pass
        const bool vec = sizeof(T) == 4 && !EXACT && (lv.g.sy % 4) == 0 && (lv.g.sz % 4) == 0 && lv.var != 2;
        for (int pass = 0; pass < 2; ++pass) {
            const int colour = forward ? pass : 1 - pass;
            if constexpr (std::is_same<T, float>::value) {
                if (vec) {
                    const int ngrp = (lv.g.N0 + 8) / 8;
                    const dim3 blk = level_block(lv, ngrp);
                    dim3 grid((ngrp + blk.x - 1) / blk.x, (lv.g.N1 + blk.y - 1) / blk.y, lv.g.N2);
                    const bool v8 = (lv.g.sy % 8) == 0 && (lv.g.sz % 8) == 0;
                    const float *vd = lv.var == 1 ? (const float *)lv.vw : nullptr;
                    const bool pd = S.pdl && lv.g.pdl;
                    // the colour-split f exists for level 0's own f only
                    const bool fs = v8 && S.fsplit && f == S.L[0].f && &lv == &S.L[0];
                    const float *fsc = fs ? S.fsplit + colour * S.fhalf : nullptr;
                    if (lv.var == 1 && fs)
                        plaunch(pd, k_sweep_rb_vec<NOISE, true, true, true>, grid, blk, 0, S.stream, x, f, lv.g, s, colour, pass, nz, vd, fsc);
                    else if (lv.var == 1 && v8)
                        plaunch(pd, k_sweep_rb_vec<NOISE, true, true, false>, grid, blk, 0, S.stream, x, f, lv.g, s, colour, pass, nz, vd, fsc);
                    else if (lv.var == 1)
                        plaunch(pd, k_sweep_rb_vec<NOISE, true, false, false>, grid, blk, 0, S.stream, x, f, lv.g, s, colour, pass, nz, vd, fsc);
                    else if (fs)
                        plaunch(pd, k_sweep_rb_vec<NOISE, false, true, true>, grid, blk, 0, S.stream, x, f, lv.g, s, colour, pass, nz, vd, fsc);
                    else if (v8)
                        plaunch(pd, k_sweep_rb_vec<NOISE, false, true, false>, grid, blk, 0, S.stream, x, f, lv.g, s, colour, pass, nz, vd, fsc);
                    else
                        plaunch(pd, k_sweep_rb_vec<NOISE, false, false, false>, grid, blk, 0, S.stream, x, f, lv.g, s, colour, pass, nz, vd, fsc);
                    S.launches++;
                    continue;
                }
            }
            {
                const int na = (lv.g.N0 + 1) / 2;
                const dim3 blk = level_block(lv, na);
                dim3 grid((na + blk.x - 1) / blk.x, (lv.g.N1 + blk.y - 1) / blk.y, lv.g.N2);
                const VarField<T> vf = var_field<T>(lv);
                if (lv.var == 1)
                    plaunch(S.pdl && lv.g.pdl, k_sweep_rb_pass<T, EXACT, NOISE, 1>, grid, blk, 0, S.stream, x, f, lv.g, s, colour,
                            pass, nz, vf);
                else if (lv.var == 2)
                    plaunch(S.pdl && lv.g.pdl, k_sweep_rb_pass<T, EXACT, NOISE, 2>, grid, blk, 0, S.stream, x, f, lv.g, s, colour,
                            pass, nz, vf);
                else
                    plaunch(S.pdl && lv.g.pdl, k_sweep_rb_pass<T, EXACT, NOISE, 0>, grid, blk, 0, S.stream, x, f, lv.g, s, colour,
                            pass, nz, vf);
            }
            S.launches++;
        }
    } else {
        launch_colour_passes<T, EXACT, NOISE>(S, lv, forward, x, f, s, nz);
    }
}

// 2^dim colours, one launch per colour
template <typename T, bool EXACT, int NOISE>
static void launch_colour_passes(Sampler &S, const Level &lv, bool forward, T *x, const T *f, const StencilArg<T> &s,
                                 const NoiseArgs &nz) {
    for (int cc = 0; cc < lv.ncol; ++cc) {
        const int colour = forward ? cc : lv.ncol - 1 - cc;
        const int pa = colour & 1, pb = (colour >> 1) & 1, pc = (colour >> 2) & 1;
        const int na = (lv.g.N0 - pa + 1) / 2, nb = (lv.g.N1 - pb + 1) / 2, nc = (lv.g.N2 - pc + 1) / 2;
        if (na <= 0 || nb <= 0 || nc <= 0) continue;
        const dim3 blk = level_block(lv, na);
        dim3 grid((na + blk.x - 1) / blk.x, (nb + blk.y - 1) / blk.y, nc);
        const VarField<T> vf = var_field<T>(lv);
        if (lv.var == 2)
            plaunch(S.pdl && lv.g.pdl, k_sweep_c27_pass<T, EXACT, NOISE, 2>, grid, blk, 0, S.stream, x, f, lv.g, s, colour, nz, vf);
        else if (lv.var == 1)
            plaunch(S.pdl && lv.g.pdl, k_sweep_c27_pass<T, EXACT, NOISE, 1>, grid, blk, 0, S.stream, x, f, lv.g, s, colour, nz, vf);
        else
            plaunch(S.pdl && lv.g.pdl, k_sweep_c27_pass<T, EXACT, NOISE, 0>, grid, blk, 0, S.stream, x, f, lv.g, s, colour, nz, vf);
        S.launches++;
    }
}

template <typename T, bool EXACT, int NOISE>
static void launch_sweep_npt(Sampler &S, const Level &lv, bool forward, T *x, const T *f, const NoiseArgs &nz) {
    if (lv.npt == 7)
        launch_sweep_t<T, 7, EXACT, NOISE>(S, lv, forward, x, f, nz);
    else
        launch_sweep_t<T, 27, EXACT, NOISE>(S, lv, forward, x, f, nz);
}

template <typename T, bool EXACT>
static void launch_sweep_noise(Sampler &S, const Level &lv, bool forward, int noise, T *x, const T *f,
                               const NoiseArgs &nz) {
    if (noise == NOISE_NONE)
        launch_sweep_npt<T, EXACT, NOISE_NONE>(S, lv, forward, x, f, nz);
    else if (noise == NOISE_PHILOX)
        launch_sweep_npt<T, EXACT, NOISE_PHILOX>(S, lv, forward, x, f, nz);
    else
        launch_sweep_npt<T, EXACT, NOISE_INJECTED>(S, lv, forward, x, f, nz);
}

// One sweep of x with right hand side f.
static void launch_sweep(Sampler &S, const Level &lv, bool forward, int noise, void *x, const void *f, const NoiseArgs &nz,
                         bool fp32, bool exact) {
    if (fp32)
        launch_sweep_noise<float, false>(S, lv, forward, noise, (float *)x, (const float *)f, nz);
    else if (exact)
        launch_sweep_noise<double, true>(S, lv, forward, noise, (double *)x, (const double *)f, nz);
    else
        launch_sweep_noise<double, false>(S, lv, forward, noise, (double *)x, (const double *)f, nz);
}

// threads of the one-CTA low-rank solve: one per row, up to 256
static unsigned solve_block(int) { return 256u; }
// its dynamic shared memory: u (m) and the partial products (256)
static size_t solve_smem(int m) { return sizeof(double) * ((size_t)m + 256); }

template <typename T>
static void launch_lowrank(Sampler &S, Level &lv, int dir, int noise, T *x, const NoiseArgs &nz) {
    LowRankArg lr;
    lr.m = S.m;
    lr.Bptr = lv.Bptr;
    lr.Bidx = lv.Bidx;
    lr.Bval = lv.Bval;
    lr.Bvalf = lv.Bvalf;
    lr.zf = lv.zf;
    lr.SinvT = lv.SinvT[dir];
    lr.sigma_sqrt = S.d_sigma_sqrt;
    lr.SinvT_ff = lv.SinvT_ff[dir];
    lr.sigma_sqrt_ff = S.d_sigma_sqrt_ff;
    lr.y = lv.y;
    lr.z = lv.z;
    lr.part = lv.part;
    lr.counter = lv.counter;
    const CorrRows &C = lv.C[dir];
    const i64 nrows = C.n1 + C.nm;
    const dim3 bgrid(S.m, lv.bt_split);
    if (nrows > LR_FUSE_MAX_ROWS) {
        // large support: partial sums with the solve in their last CTA, then
        // the correction on the whole GPU
        const size_t smem = solve_smem(S.m);
        if (noise == NOISE_NONE)
            plaunch(S.pdl, k_bt_solve<T, NOISE_NONE, true>, bgrid, 256, smem, S.stream, (const T *)x, lr, nz);
        else if (noise == NOISE_PHILOX)
            plaunch(S.pdl, k_bt_solve<T, NOISE_PHILOX, true>, bgrid, 256, smem, S.stream, (const T *)x, lr, nz);
        else
            plaunch(S.pdl, k_bt_solve<T, NOISE_INJECTED, true>, bgrid, 256, smem, S.stream, (const T *)x, lr, nz);
        const unsigned blocks = (unsigned)std::min<i64>(nblk(nrows, 4 * 256), 8 * S.nsm);
        if (sizeof(T) == 4)
            plaunch(S.pdl, k_lr_scatter<T, float>, blocks, 256, 0, S.stream, x, C, (const float *)lv.zf);
        else
            plaunch(S.pdl, k_lr_scatter<T, double>, blocks, 256, 0, S.stream, x, C, (const double *)lv.z);
        S.launches++;
    } else if (nrows > 0) {
        plaunch(S.pdl, k_bt_partial<T>, bgrid, 256, 0, S.stream, (const T *)x, lr);
        S.launches++;
        // solve and correction in one launch; every CTA repeats the m x m
        // solve, so the grid stays at a few CTAs per SM
        const unsigned blocks = (unsigned)std::min<i64>(nblk(nrows, 256), MGMC_LR_APPLY_CTAS_PER_SM * S.nsm);
        const size_t sm = sizeof(double) * (2 * (size_t)S.m + 256);
        if (noise == NOISE_NONE)
            plaunch(S.pdl, k_lr_apply<T, NOISE_NONE>, blocks, 256, sm, S.stream, x, lr, lv.bt_split, nz, C);
        else if (noise == NOISE_PHILOX)
            plaunch(S.pdl, k_lr_apply<T, NOISE_PHILOX>, blocks, 256, sm, S.stream, x, lr, lv.bt_split, nz, C);
        else
            plaunch(S.pdl, k_lr_apply<T, NOISE_INJECTED>, blocks, 256, sm, S.stream, x, lr, lv.bt_split, nz, C);
    } else {
        plaunch(S.pdl, k_bt_partial<T>, bgrid, 256, 0, S.stream, (const T *)x, lr);
        S.launches++;
        const size_t smem = solve_smem(S.m);
        if (noise == NOISE_NONE)
            plaunch(S.pdl, k_lr_solve<T, NOISE_NONE, true>, 1, solve_block(S.m), smem, S.stream, lr, lv.bt_split, nz);
        else if (noise == NOISE_PHILOX)
            plaunch(S.pdl, k_lr_solve<T, NOISE_PHILOX, true>, 1, solve_block(S.m), smem, S.stream, lr, lv.bt_split, nz);
        else
            plaunch(S.pdl, k_lr_solve<T, NOISE_INJECTED, true>, 1, solve_block(S.m), smem, S.stream, lr, lv.bt_split, nz);
    }
    S.launches += 1;
}

// SORSampler::apply (sor_sampler.cc:37-59) / SORSmoother::apply
// (sor_smoother.cc:40-54) on level `lev`: noise draw order n point normals,
// then m low-rank normals.
// nsparse > 1 (noise-free only): that many sweeps of the sparse part before
// the one low-rank correction, as SORSmoother::apply does with nsmooth > 1
// (sor_smoother.cc:43-53 around the nsmooth sweeps of :64-76).
void Sampler::sor(int lev, bool forward, bool noisy, void *x, void *f, int nsparse) {
    Level &lv = L[lev];
    int noise = noisy ? noise_mode : NOISE_NONE;
    NoiseArgs nz = noisy ? noise_args(lev, lv.geo.n) : noise_args(lev, 0);
    if (!noisy) nz.buf = nullptr;
    void *xin = taping ? tape_state(lev) : nullptr;
    for (int k = 0; k < (noisy ? 1 : nsparse); ++k) launch_sweep(*this, lv, forward, noise, x, f, nz, fp32, exact);
    NoiseArgs nzl{};
    if (m > 0) {
        nzl = noisy ? noise_args(lev, m) : noise_args(lev, 0);
        if (!noisy) nzl.buf = nullptr;
        if (fp32)
            launch_lowrank<float>(*this, lv, forward ? 0 : 1, noise, (float *)x, nzl);
        else
            launch_lowrank<double>(*this, lv, forward ? 0 : 1, noise, (double *)x, nzl);
    }
    if (taping) {
        void *xout = tape_snap(lev, x);
        tape_last[lev] = xout;
        tape.push_back(TapeEvent{EV_SWEEP, lev, forward, xin, xout, tape_f[lev], nz, nzl});
    }
    if (noisy) inv++;
}

template <typename T>
static void launch_resid_restrict(Sampler &S, int lev, const void *x, const void *f, void *fc, void *xc, bool zero_stencil) {
    Level &lv = S.L[lev], &lc = S.L[lev + 1];
    StencilArg<T> s = stencil_arg<T>(lv, S.P.omega);
    if (zero_stencil)
        for (int k = 0; k < 27; ++k) s.w[k] = T(0);
    const i64 nc = lc.geo.n;
    if (lv.var && !zero_stencil) {  // variable coefficients: the plain fused kernel
        const VarField<T> vf = var_field<T>(lv);
        const bool pdl = S.pdl && lv.g.pdl;
        if (lv.npt == 7 && lv.var == 1)
            plaunch(pdl, k_resid_restrict<T, 7, 1>, nblk(nc, 256), 256, 0, S.stream, (const T *)x, (const T *)f, (T *)fc, (T *)xc,
                    lv.g, lc.g, s, S.dim, vf);
        else if (lv.var == 1)
            plaunch(pdl, k_resid_restrict<T, 27, 1>, nblk(nc, 256), 256, 0, S.stream, (const T *)x, (const T *)f, (T *)fc, (T *)xc,
                    lv.g, lc.g, s, S.dim, vf);
        else
            plaunch(pdl, k_resid_restrict<T, 27, 2>, nblk(nc, 256), 256, 0, S.stream, (const T *)x, (const T *)f, (T *)fc, (T *)xc,
                    lv.g, lc.g, s, S.dim, vf);
        S.launches++;
        return;
    }
    if (S.dim == 3 && !zero_stencil && lv.tma && x == lv.x && f == lv.f) {
        dim3 grid((lc.g.N0 + RR_TX - 1) / RR_TX, (lc.g.N1 + RR_TY - 1) / RR_TY, (lc.g.N2 + RR_TZ - 1) / RR_TZ);
        const size_t sm = rr_tma_smem_bytes<T>();
        if (lv.npt == 7)
            plaunch(S.pdl && lv.g.pdl, k_resid_restrict_tma<T, 7>, grid, RR_THREADS, sm, S.stream, lv.xmap, lv.fmap, (T *)fc, (T *)xc, lv.g, lc.g, s,
                    S.d_err);
        else
            plaunch(S.pdl && lv.g.pdl, k_resid_restrict_tma<T, 27>, grid, RR_THREADS, sm, S.stream, lv.xmap, lv.fmap, (T *)fc, (T *)xc, lv.g, lc.g,
                    s, S.d_err);
        S.launches++;
        return;
    }
    if (S.dim == 3 && !zero_stencil) {
        dim3 grid((lc.g.N0 + RR_TX - 1) / RR_TX, (lc.g.N1 + RR_TY - 1) / RR_TY, (lc.g.N2 + RR_TZ - 1) / RR_TZ);
        const size_t sm = rr_smem_bytes<T>();
        if (lv.npt == 7)
            plaunch(S.pdl && lv.g.pdl, k_resid_restrict_tiled<T, 7>, grid, RR_THREADS, sm, S.stream, (const T *)x, (const T *)f, (T *)fc, (T *)xc, lv.g, lc.g, s);
        else
            plaunch(S.pdl && lv.g.pdl, k_resid_restrict_tiled<T, 27>, grid, RR_THREADS, sm, S.stream, (const T *)x, (const T *)f, (T *)fc, (T *)xc, lv.g, lc.g, s);
        S.launches++;
        return;
    }
    const VarField<T> vf0{nullptr, 0};
    if (lv.npt == 7 && !zero_stencil)
        plaunch(S.pdl && lv.g.pdl, k_resid_restrict<T, 7, 0>, nblk(nc, 256), 256, 0, S.stream, (const T *)x, (const T *)f, (T *)fc, (T *)xc, lv.g, lc.g, s, S.dim, vf0);
    else
        plaunch(S.pdl && lv.g.pdl, k_resid_restrict<T, 27, 0>, nblk(nc, 256), 256, 0, S.stream, (const T *)x, (const T *)f, (T *)fc, (T *)xc, lv.g, lc.g, s, S.dim, vf0);
    S.launches++;
}

// y = B^T x on the level (into the level's y unless `y` is given)
template <typename T>
static void launch_bt_plain(Sampler &S, Level &lv, const void *x, double *y = nullptr) {
    LowRankArg lr{};
    lr.m = S.m;
    lr.Bptr = lv.Bptr;
    lr.Bidx = lv.Bidx;
    lr.Bval = lv.Bval;
    lr.Bvalf = lv.Bvalf;
    lr.y = y ? y : lv.y;
    lr.part = lv.part;
    lr.counter = lv.counter;
    NoiseArgs nz{};
    plaunch(S.pdl, k_bt_solve<T, NOISE_NONE, false>, dim3(S.m, lv.bt_split), 256, solve_smem(S.m), S.stream,
            (const T *)x, lr, nz);
    S.launches += 1;
}

template <typename T>
static void launch_add_Bq(Sampler &S, Level &lv, void *dst, const double *y, double sign) {
    const RowCsr &B = lv.Br;
    if (B.nrows == 0) return;
    plaunch(S.pdl, k_add_Bq<T>, nblk(B.nrows, 256), 256, 0, S.stream, (T *)dst, B.nrows, B.rows, B.ptr, B.col, (const double *)B.val, y,
                                                          S.d_sigma_inv, sign);
    S.launches++;
}

// residual f - A x of multigridmc_sampler.cc:124-125 restricted to the
// next level (:126): R (f - A_0 x) - B_c Sigma^{-1} B^T x.
void Sampler::resid_restrict(int lev) {
    Level &lv = L[lev], &lc = L[lev + 1];
    if (taping) tape.push_back(TapeEvent{EV_RESID, lev, true, tape_state(lev), nullptr, nullptr, NoiseArgs{}, NoiseArgs{}});
    if (fp32) {
        launch_resid_restrict<float>(*this, lev, lv.x, lv.f, lc.f, lc.x, false);
        if (m > 0) {
            launch_bt_plain<float>(*this, lv, lv.x);
            launch_add_Bq<float>(*this, lc, lc.f, lv.y, -1.0);
        }
    } else {
        launch_resid_restrict<double>(*this, lev, lv.x, lv.f, lc.f, lc.x, false);
        if (m > 0) {
            launch_bt_plain<double>(*this, lv, lv.x);
            launch_add_Bq<double>(*this, lc, lc.f, lv.y, -1.0);
        }
    }
    if (taping) {
        tape_last[lev + 1] = nullptr;  // the coarse state starts from zero
        tape_f[lev + 1] = tape_snap(lev + 1, lc.f);
    }
}

void Sampler::prolong(int lev, double alpha, void *xc, void *x) {
    Level &lv = L[lev], &lc = L[lev + 1];
    if (taping) tape_last[lev] = nullptr;
    dim3 grid((lc.g.N0 + 1 + 127) / 128, dim > 1 ? lc.g.N1 + 1 : 1, dim > 2 ? lc.g.N2 + 1 : 1);
    if (fp32)
        plaunch(pdl && lv.g.pdl, k_prolong_add<float>, grid, 128, 0, stream, (float *)x, (const float *)xc, lv.g, lc.g, (float)alpha, dim);
    else
        plaunch(pdl && lv.g.pdl, k_prolong_add<double>, grid, 128, 0, stream, (double *)x, (const double *)xc, lv.g, lc.g, alpha, dim);
    launches++;
}

template <typename T, int NOISE>
static void launch_chol(Sampler &S, Level &lv, const NoiseArgs &nz) {
    if (S.exact) {
        plaunch(S.pdl && lv.g.pdl, k_chol_subst<T, NOISE>, 1, 1024, 0, S.stream, (const T *)lv.f, (T *)lv.x, lv.g, S.dL, S.dgv, nz);
        S.launches++;
    } else {
        // FP32 chain: FP32 factor products (the state itself is FP32);
        // FP64 chain: FP64
        typedef T MT;
        const i64 n = lv.geo.n;
        unsigned blocks = (unsigned)((n + 7) / 8);
        plaunch(S.pdl && lv.g.pdl, k_chol_gemv_lower<T, MT, NOISE>, blocks, 256, S.chol_smem, S.stream, (const T *)lv.f, lv.g,
                                                                                (const MT *)S.dLinv, S.chol_ld,
                                                                                (MT *)S.dgv, nz);
        plaunch(S.pdl && lv.g.pdl, k_chol_gemv_upper<T, MT>, blocks, 256, S.chol_smem, S.stream, (const MT *)S.dgv, lv.g, (const MT *)S.dLinvT,
                                                                         S.chol_ld, (T *)lv.x);
        S.launches += 2;
    }
}

// coarsest level: CholeskySampler::apply or SSORSampler with ncoarsesmooth
// (multigridmc_sampler.cc:54-79, 112-116)
void Sampler::coarse_sample(int lev) {
    Level &lv = L[lev];
    if (!noisy) {
        // the preconditioner's coarse solver is always Cholesky
        // (multigrid_preconditioner.cc:41-46): x = Q^{-1} f
        NoiseArgs nz = noise_args(lev, 0);
        nz.buf = nullptr;
        if (fp32)
            launch_chol<float, NOISE_NONE>(*this, lv, nz);
        else
            launch_chol<double, NOISE_NONE>(*this, lv, nz);
        return;
    }
    if (chol) {
        NoiseArgs nz = noise_args(lev, lv.geo.n);
        if (taping) {
            tape.push_back(TapeEvent{EV_COARSE, lev, true, nullptr, nullptr, tape_f[lev], nz, NoiseArgs{}});
            tape_last[lev] = nullptr;
        }
        if (fp32) {
            if (noise_mode == NOISE_PHILOX)
                launch_chol<float, NOISE_PHILOX>(*this, lv, nz);
            else
                launch_chol<float, NOISE_INJECTED>(*this, lv, nz);
        } else {
            if (noise_mode == NOISE_PHILOX)
                launch_chol<double, NOISE_PHILOX>(*this, lv, nz);
            else
                launch_chol<double, NOISE_INJECTED>(*this, lv, nz);
        }
        inv++;
    } else {
        for (int k = 0; k < P.ncoarsesmooth; ++k) {
            sor(lev, true, true, lv.x, lv.f);
            sor(lev, false, true, lv.x, lv.f);
        }
    }
}

// MultigridMCSampler::sample (multigridmc_sampler.cc:109-136)
void Sampler::sample(int lev) {
    const int nlev = (int)L.size();
    if (lev == nlev - 1) {
        coarse_sample(lev);
        return;
    }
    Level &lv = L[lev], &lc = L[lev + 1];
    const int cyc = lev > 0 ? P.cycle : 1;
    const bool ssor = P.smoother == MGMC_SMOOTHER_SSOR;
    for (int j = 0; j < cyc; ++j) {
        if (ssor) {
            for (int k = 0; k < P.npresmooth; ++k) {
                sor(lev, true, noisy, lv.x, lv.f);
                sor(lev, false, noisy, lv.x, lv.f);
            }
        } else {
            smooth(lev, true, P.npresmooth);
        }
        resid_restrict(lev);  // also zeroes the coarse state
        sample(lev + 1);
        prolong(lev, P.coarse_scaling, lc.x, lv.x);
        if (ssor) {
            for (int k = 0; k < P.npostsmooth; ++k) {
                sor(lev, true, noisy, lv.x, lv.f);
                sor(lev, false, noisy, lv.x, lv.f);
            }
        } else {
            smooth(lev, false, P.npostsmooth);
        }
    }
}

// SOR smoothing with nsmooth passes in one direction: the sampler's
// SORSampler draws fresh noise for each sweep (sor_sampler.cc:37-59); the
// preconditioner's SORSmoother repeats nsmooth times nsmooth sparse sweeps
// and one low-rank correction (sor_smoother.cc:40-78), which is the same
// for nsmooth = 1.
void Sampler::smooth(int lev, bool forward, int nsmooth) {
    Level &lv = L[lev];
    for (int k = 0; k < nsmooth; ++k) sor(lev, forward, noisy, lv.x, lv.f, nsmooth);
}

void Sampler::step_end() {
    if (fp32)
        plaunch(pdl, k_step_end<float>, std::max(nprobe, 1), 256, 0, stream, (const float *)L[0].x, nprobe, d_bptr, d_bidx, d_bval, d_obs,
                                                                  obs_cap, d_obs_count, d_step, d_err, d_done);
    else
        plaunch(pdl, k_step_end<double>, std::max(nprobe, 1), 256, 0, stream, (const double *)L[0].x, nprobe, d_bptr, d_bidx, d_bval,
                                                                   d_obs, obs_cap, d_obs_count, d_step, d_err, d_done);
    launches++;
}

void Sampler::launch_step() {
    inv = 0;
    noise_off = noise_pos;
    launches = 0;
    sample(0);
    step_end();
    step_launches = launches;
}

// ------------------------------------------------------------- set-up
static int stencil_npt(int ncol, const double st[27]) {
    if (ncol != 2) return 27;
    for (int k = 0; k < 27; ++k) {
        int dx = k % 3 - 1, dy = (k / 3) % 3 - 1, dz = k / 9 - 1;
        if ((dx != 0) + (dy != 0) + (dz != 0) > 1 && st[k] != 0.0) return 27;
    }
    return 7;
}

__global__ void k_scatter(const unsigned *__restrict__ idx, const double *__restrict__ val, i64 cnt, double *__restrict__ dst) {
    i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < cnt) dst[idx[t]] = val[t];
}

__global__ void k_nonzeros(const double *__restrict__ x, Grid3 g, i64 *__restrict__ idx, double *__restrict__ val,
                           unsigned long long *__restrict__ count) {
    i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
    i64 n = (i64)g.N0 * g.N1 * g.N2;
    if (t >= n) return;
    int a = (int)(t % g.N0), b = (int)((t / g.N0) % g.N1), c = (int)(t / ((i64)g.N0 * g.N1));
    double v = x[g.pad(a, b, c)];
    if (v != 0.0) {
        unsigned long long k = atomicAdd(count, 1ull);
        idx[k] = t;
        val[k] = v;
    }
}

// C = M^{-1} B for both sweep directions, M = D/omega + (strictly lower
// part of A_0 in the sweep order): column j is one noise-free sweep from
// x = 0 with right hand side B e_j (sor_smoother.cc:17-37 in solve form).
// S = Sigma + B^T C (with G = B^T C) gives the m x m system of k_lr_solve.
void Sampler::build_lowrank(int lev) {
    Level &lv = L[lev];
    const Geometry &geo = lv.geo;
    const i64 n = geo.n;
    // B on this level: CSC with padded indices, and row-compressed form
    {
        if (geo.nalloc > (i64)UINT32_MAX)
            fail(MGMC_ERR_UNSUPPORTED, "measurements on a level of 2^32 or more padded points (32-bit indices of B and C)");
        std::vector<unsigned> bidx(lv.Bh.row.size());
        for (size_t e = 0; e < bidx.size(); ++e) bidx[e] = (unsigned)geo.pad(lv.Bh.row[e]);
        std::vector<i64> bptr(lv.Bh.ptr.begin(), lv.Bh.ptr.end());
        lv.Bptr = upload(bptr);
        lv.Bidx = upload(bidx);
        lv.Bval = upload(lv.Bh.val);
        std::vector<float> bvf(lv.Bh.val.begin(), lv.Bh.val.end());
        lv.Bvalf = upload(bvf);
        std::vector<std::tuple<i64, int, double>> trip;
        for (int j = 0; j < m; ++j)
            for (i64 e = lv.Bh.ptr[j]; e < lv.Bh.ptr[j + 1]; ++e) trip.emplace_back(lv.Bh.row[e], j, lv.Bh.val[e]);
        std::sort(trip.begin(), trip.end());
        std::vector<i64> rows, ptr{0};
        std::vector<int> col;
        std::vector<double> val;
        for (size_t e = 0; e < trip.size(); ++e) {
            if (e == 0 || std::get<0>(trip[e]) != std::get<0>(trip[e - 1])) {
                if (e > 0) ptr.push_back((i64)col.size());
                rows.push_back(geo.pad(std::get<0>(trip[e])));
            }
            col.push_back(std::get<1>(trip[e]));
            val.push_back(std::get<2>(trip[e]));
        }
        if (!trip.empty()) ptr.push_back((i64)col.size());
        lv.Br.nrows = (i64)rows.size();
        lv.Br.rows = upload(rows);
        lv.Br.ptr = upload(ptr);
        lv.Br.col = upload(col);
        lv.Br.val = upload(val);
    }
    lv.y = alloc<double>(m);
    lv.z = alloc<double>(m);
    lv.zf = alloc<float>(m);
    {
        i64 maxcol = 1;
        for (int j = 0; j < m; ++j) maxcol = std::max<i64>(maxcol, lv.Bh.ptr[j + 1] - lv.Bh.ptr[j]);
        // about 2048 entries of the longest column per CTA (measured at
        // 256^3 with 64 balls: 256 to 4096 entries per CTA gave 32.2, 27.8,
        // 23.3, 21.7, 23.1 us per low-rank correction); the split fixes the
        // order of the partial sums, so it depends on the sizes only
        lv.bt_split = (int)std::min<i64>(32, std::max<i64>(1, (maxcol + 2047) / 2048));
    }
    lv.part = alloc<double>((size_t)m * lv.bt_split);
    lv.counter = alloc<unsigned>(1);
    CK(cudaMemsetAsync(lv.counter, 0, sizeof(unsigned), stream));
    // FP64 work arrays, released at the end of the set-up
    double *xs = alloc<double>(geo.nalloc), *fs = alloc<double>(geo.nalloc);
    i64 *nzi = alloc<i64>(n);
    double *nzv = alloc<double>(n);
    unsigned long long *cnt = alloc<unsigned long long>(1);
    struct Release {
        Sampler &S;
        std::vector<void *> ptrs;
        ~Release() {
            cudaStreamSynchronize(S.stream);
            for (void *p : ptrs) S.release(p);
        }
    } work{*this, {xs, fs, nzi, nzv, cnt}};
    std::vector<double> yh(m);
    for (int dir = 0; dir < 2; ++dir) {
        std::vector<std::tuple<i64, int, double>> trip;
        std::vector<double> Sh((size_t)m * m);
        for (int j = 0; j < m; ++j) {
            CK(cudaMemsetAsync(xs, 0, geo.nalloc * sizeof(double), stream));
            CK(cudaMemsetAsync(fs, 0, geo.nalloc * sizeof(double), stream));
            const i64 b0 = lv.Bh.ptr[j], cntj = lv.Bh.ptr[j + 1] - lv.Bh.ptr[j];
            if (cntj > 0) k_scatter<<<nblk(cntj, 256), 256, 0, stream>>>(lv.Bidx + b0, lv.Bval + b0, cntj, fs);
            NoiseArgs nz{};
            nz.d_step = d_step;
            launch_sweep(*this, lv, dir == 0, NOISE_NONE, xs, fs, nz, false, exact);
            // G[:, j] = B^T C e_j
            LowRankArg lr{};
            lr.m = m;
            lr.Bptr = lv.Bptr;
            lr.Bidx = lv.Bidx;
            lr.Bval = lv.Bval;
            lr.Bvalf = lv.Bvalf;
            lr.y = lv.y;
            lr.part = lv.part;
            k_bt_partial<double><<<dim3(m, lv.bt_split), 256, 0, stream>>>(xs, lr);
            k_lr_solve<double, NOISE_NONE, false><<<1, solve_block(m), 0, stream>>>(lr, lv.bt_split, nz);
            CK(cudaMemcpyAsync(yh.data(), lv.y, m * sizeof(double), cudaMemcpyDeviceToHost, stream));
            CK(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), stream));
            k_nonzeros<<<nblk(n, 256), 256, 0, stream>>>(xs, lv.g, nzi, nzv, cnt);
            unsigned long long hc = 0;
            CK(cudaMemcpyAsync(&hc, cnt, sizeof(hc), cudaMemcpyDeviceToHost, stream));
            CK(cudaStreamSynchronize(stream));
            check_launch();
            std::vector<i64> ii(hc);
            std::vector<double> vv(hc);
            if (hc) {
                CK(cudaMemcpy(ii.data(), nzi, hc * sizeof(i64), cudaMemcpyDeviceToHost));
                CK(cudaMemcpy(vv.data(), nzv, hc * sizeof(double), cudaMemcpyDeviceToHost));
            }
            for (unsigned long long e = 0; e < hc; ++e) trip.emplace_back(ii[e], j, vv[e]);
            for (int a = 0; a < m; ++a) Sh[(size_t)a * m + j] = yh[a] + (a == j ? Sigma[a] : 0.0);
        }
        // rows with one entry as triples, the others in CSR form (entries
        // of a row in column order)
        std::sort(trip.begin(), trip.end());
        std::vector<unsigned> r1, rm;
        std::vector<int> c1, pm{0}, cm;
        std::vector<double> v1, vm;
        for (size_t e = 0; e < trip.size();) {
            size_t e1 = e + 1;
            while (e1 < trip.size() && std::get<0>(trip[e1]) == std::get<0>(trip[e])) ++e1;
            const unsigned row = (unsigned)geo.pad(std::get<0>(trip[e]));
            if (e1 == e + 1) {
                r1.push_back(row);
                c1.push_back(std::get<1>(trip[e]));
                v1.push_back(std::get<2>(trip[e]));
            } else {
                rm.push_back(row);
                for (size_t k = e; k < e1; ++k) {
                    cm.push_back(std::get<1>(trip[k]));
                    vm.push_back(std::get<2>(trip[k]));
                }
                pm.push_back((int)cm.size());
            }
            e = e1;
        }
        CorrRows &C = lv.C[dir];
        C.n1 = (i64)r1.size();
        C.nm = (i64)rm.size();
        C.r1 = upload(r1);
        C.c1 = upload(c1);
        C.rm = upload(rm);
        C.pm = upload(pm);
        C.cm = upload(cm);
        if (fp32) {
            C.v1 = upload(std::vector<float>(v1.begin(), v1.end()));
            C.vm = upload(std::vector<float>(vm.begin(), vm.end()));
        } else {
            C.v1 = upload(v1);
            C.vm = upload(vm);
        }
        {
            const std::vector<double> Si = small_inverse(Sh, m);
            std::vector<double> SiT((size_t)m * m);
            for (int a = 0; a < m; ++a)
                for (int q = 0; q < m; ++q) SiT[(size_t)q * m + a] = Si[(size_t)a * m + q];
            lv.SinvT[dir] = upload(SiT);
            lv.SinvT_ff[dir] = upload(float_float(SiT));
        }
    }
    CK(cudaStreamSynchronize(stream));
}

// dense A_0 + B Sigma^{-1} B^T of a level (constant stencil or field)
std::vector<double> Sampler::level_precision(const Level &lv) const {
    if (!lv.var) return dense_precision(lv.geo, lv.st, lv.Bh, Sigma);
    if (lv.var == 2) return dense_precision_field(lv.geo, lv.vh, lv.Bh, Sigma);
    std::vector<double> full((size_t)27 * lv.geo.n);
    for (int k = 0; k < 27; ++k)
        for (i64 i = 0; i < lv.geo.n; ++i) full[(size_t)k * lv.geo.n + i] = k == 13 ? lv.vh[i] : lv.st[k];
    return dense_precision_field(lv.geo, full, lv.Bh, Sigma);
}

void Sampler::build_coarse() {
    Level &lv = L.back();
    const i64 n = lv.geo.n;
    if (n > 12000) fail(MGMC_ERR_UNSUPPORTED, "coarse level has " + std::to_string(n) + " unknowns; the dense Cholesky sampler takes at most 12000");
    std::vector<double> Q = level_precision(lv);
    if (!dense_cholesky(Q, n)) fail(MGMC_ERR_NOT_SPD, "coarse precision matrix is not positive definite");
    dgv = alloc<double>(n);
    chol_smem = (size_t)n * sizeof(double);
    if (exact) dL = upload(Q);  // parity path: substitution in the oracle's order
    {
        // throughput path and adjoint: explicit inverse factors
        std::vector<double> T = inverse_factor_transposed(Q, n);  // (L^{-1})^T
        const size_t esz = fp32 ? sizeof(float) : sizeof(double);
        const i64 ld = (i64)((n * esz + 15) / 16 * 16 / esz);
        chol_ld = (int)ld;
        chol_smem = (size_t)ld * esz;
        auto put = [&](bool transpose) -> void * {
            if (fp32) {
                std::vector<float> M((size_t)n * ld, 0.0f);
                for (i64 i = 0; i < n; ++i)
                    for (i64 j = 0; j < n; ++j) M[(size_t)i * ld + j] = (float)(transpose ? T[(size_t)i * n + j] : T[(size_t)j * n + i]);
                return upload(M);
            }
            std::vector<double> M((size_t)n * ld, 0.0);
            for (i64 i = 0; i < n; ++i)
                for (i64 j = 0; j < n; ++j) M[(size_t)i * ld + j] = transpose ? T[(size_t)i * n + j] : T[(size_t)j * n + i];
            return upload(M);
        };
        dLinvT = put(true);
        dLinv = put(false);
        if (chol_smem > 48 * 1024) {
            raise_smem_limit(k_chol_gemv_lower<float, float, NOISE_PHILOX>, chol_smem);
            raise_smem_limit(k_chol_gemv_lower<double, double, NOISE_PHILOX>, chol_smem);
            raise_smem_limit(k_chol_gemv_lower<float, float, NOISE_INJECTED>, chol_smem);
            raise_smem_limit(k_chol_gemv_lower<double, double, NOISE_INJECTED>, chol_smem);
            raise_smem_limit(k_chol_gemv_lower<float, float, NOISE_NONE>, chol_smem);
            raise_smem_limit(k_chol_gemv_lower<double, double, NOISE_NONE>, chol_smem);
            raise_smem_limit(k_chol_gemv_upper<float, float>, chol_smem);
            raise_smem_limit(k_chol_gemv_upper<double, double>, chol_smem);
        }
    }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library).
static EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
        else
            cudaGetLastError();
    }
    return fn;
}

// Tile maps of a level's padded x and f as 3D tensors (row of sy elements
// including the shared ghost, sz / sy rows per plane, N2 + 2 planes) for
// k_resid_restrict_tma; levels whose row or plane pitch is not a multiple of
// 16 bytes keep the plain-load kernel.
void Sampler::make_tile_maps(Level &lv) {
    if (dim != 3) return;
    const size_t esz = fp32 ? sizeof(float) : sizeof(double);
    if ((lv.g.sy * esz) % 16 != 0 || (lv.g.sz * esz) % 16 != 0) return;
    EncodeTiledFn enc = encode_tiled();
    if (!enc) return;
    const cuuint64_t dims[3] = {(cuuint64_t)lv.g.sy, (cuuint64_t)(lv.g.sz / lv.g.sy), (cuuint64_t)lv.g.N2 + 2};
    const cuuint64_t strides[2] = {(cuuint64_t)(lv.g.sy * esz), (cuuint64_t)(lv.g.sz * esz)};
    const cuuint32_t xbox[3] = {RR_BW, RR_XH, RR_XD}, fbox[3] = {RR_BW, RR_FH, RR_FD}, es[3] = {1, 1, 1};
    const CUtensorMapDataType dt = fp32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
    if (enc(&lv.xmap, dt, 3, lv.x, dims, strides, xbox, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return;
    if (enc(&lv.fmap, dt, 3, lv.f, dims, strides, fbox, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return;
    lv.tma = true;
}

void Sampler::build(const mgmc_operator_desc &op) {
    if (op.dim < 1 || op.dim > 3) fail(MGMC_ERR_INVALID_ARGUMENT, "dim must be 1, 2 or 3");
    dim = op.dim;
    int cells[3] = {op.nx, op.dim > 1 ? op.ny : 2, op.dim > 2 ? op.nz : 2};
    for (int d = 0; d < dim; ++d)
        if (cells[d] < 2) fail(MGMC_ERR_LATTICE, "every active direction needs at least 2 cells");
    if (P.nlevel < 1) fail(MGMC_ERR_INVALID_ARGUMENT, "nlevel must be >= 1");
    if (P.smoother != MGMC_SMOOTHER_SOR && P.smoother != MGMC_SMOOTHER_SSOR) fail(MGMC_ERR_INVALID_ARGUMENT, "invalid smoother");
    if (P.coarse_solver != MGMC_COARSE_CHOLESKY && P.coarse_solver != MGMC_COARSE_SSOR) fail(MGMC_ERR_INVALID_ARGUMENT, "invalid coarse solver");
    if (P.ordering != MGMC_ORDER_LEXICOGRAPHIC && P.ordering != MGMC_ORDER_MULTICOLOUR) fail(MGMC_ERR_INVALID_ARGUMENT, "invalid ordering");
    if (P.precision != MGMC_FP64 && P.precision != MGMC_FP32_MIXED) fail(MGMC_ERR_INVALID_ARGUMENT, "invalid precision");
    if (P.noise != MGMC_NOISE_PHILOX && P.noise != MGMC_NOISE_INJECTED) fail(MGMC_ERR_INVALID_ARGUMENT, "invalid noise source");
    if (!(P.omega > 0.0 && P.omega < 2.0)) fail(MGMC_ERR_INVALID_ARGUMENT, "omega must lie in (0, 2)");
    if (P.cycle < 1 || P.npresmooth < 0 || P.npostsmooth < 0 || P.ncoarsesmooth < 0)
        fail(MGMC_ERR_INVALID_ARGUMENT, "cycle >= 1 and non-negative smoothing counts required");
    if (op.m < 0 || (op.m > 0 && (!op.B_colptr || !op.B_rowidx || !op.B_val || !op.Sigma)))
        fail(MGMC_ERR_INVALID_ARGUMENT, "low-rank term needs B and Sigma");
    if (op.m > 3072) fail(MGMC_ERR_UNSUPPORTED, "at most 3072 measurement columns");
    if ((op.centre || op.field) && op.dim < 2) fail(MGMC_ERR_UNSUPPORTED, "a per-vertex stencil needs dim >= 2");
    if ((op.centre || op.field) && P.ordering != MGMC_ORDER_MULTICOLOUR)
        fail(MGMC_ERR_UNSUPPORTED, "a per-vertex stencil needs the multicolour ordering");
    fp32 = P.precision == MGMC_FP32_MIXED;
    noise_mode = P.noise == MGMC_NOISE_INJECTED ? NOISE_INJECTED : NOISE_PHILOX;
    exact = !fp32 && noise_mode == NOISE_INJECTED;
    chol = P.coarse_solver == MGMC_COARSE_CHOLESKY;
    m = op.m;
    CK(cudaSetDevice(P.device));
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, P.device));
    {
        const char *e = std::getenv("MGMC_NO_PDL");
        pdl = !(e && e[0] == '1');
    }
    CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    raise_smem_limit(k_resid_restrict_tiled<double, 7>, rr_smem_bytes<double>());
    raise_smem_limit(k_resid_restrict_tiled<double, 27>, rr_smem_bytes<double>());
    raise_smem_limit(k_resid_restrict_tma<double, 7>, rr_tma_smem_bytes<double>());
    raise_smem_limit(k_resid_restrict_tma<double, 27>, rr_tma_smem_bytes<double>());
    d_step = alloc<u64>(1);
    d_obs_count = alloc<u64>(1);
    d_err = alloc<unsigned>(1);
    d_done = alloc<unsigned>(1);
    CK(cudaMemsetAsync(d_done, 0, sizeof(unsigned), stream));
    CK(cudaMemsetAsync(d_step, 0, sizeof(u64), stream));
    CK(cudaMemsetAsync(d_obs_count, 0, sizeof(u64), stream));
    CK(cudaMemsetAsync(d_err, 0, sizeof(unsigned), stream));
    // levels
    Geometry geo(dim, cells[0], cells[1], cells[2]);
    double st[27];
    std::memcpy(st, op.stencil, sizeof(st));
    for (int lev = 0; lev < P.nlevel; ++lev) {
        if (lev > 0) {
            if (!geo.coarsenable())
                fail(MGMC_ERR_LATTICE, "cannot coarsen lattice level " + std::to_string(lev - 1) + " [odd extent or no interior vertices left]");
            geo = geo.coarse();
            double stc[27];
            galerkin_stencil(dim, st, stc);
            std::memcpy(st, stc, sizeof(st));
        }
        Level lv;
        lv.geo = geo;
        lv.g.N0 = geo.N[0];
        lv.g.N1 = geo.N[1];
        lv.g.N2 = geo.N[2];
        lv.g.sy = geo.sy;
        lv.g.sz = geo.sz;
        std::memcpy(lv.st, st, sizeof(st));
        lv.diag = st[13];
        if (op.centre || op.field) {
            // variable coefficients: level 0 keeps the centre weights (or
            // the whole per-vertex stencils), every coarser level the
            // Galerkin product of the level above
            if (lev == 0 && op.field) {
                lv.var = 2;
                lv.vh.assign(op.field, op.field + (size_t)27 * geo.n);
                // the colouring follows the couplings present anywhere in the field
                for (int k = 0; k < 27; ++k) {
                    double mx = 0.0;
                    for (i64 i = 0; i < geo.n; ++i) mx = std::max(mx, std::fabs(lv.vh[(size_t)k * geo.n + i]));
                    if (k != 13 && mx > 0.0 && st[k] == 0.0) st[k] = -mx;
                }
                std::memcpy(lv.st, st, sizeof(st));
            } else if (lev == 0) {
                lv.var = 1;
                lv.vh.assign(op.centre, op.centre + geo.n);
            } else {
                Level &lf = L[lev - 1];
                lv.var = 2;
                lv.vh = galerkin_field(lf.geo, lf.st, lf.var == 1 ? lf.vh.data() : nullptr,
                                       lf.var == 2 ? lf.vh.data() : nullptr);
                if (lev > 1) std::vector<double>().swap(lf.vh);  // only the fine centre and the coarsest field stay
            }
            double dmin = HUGE_VAL, dsum = 0.0;
            const double *dp = lv.var == 1 ? lv.vh.data() : lv.vh.data() + (size_t)13 * geo.n;
            for (i64 i = 0; i < geo.n; ++i) {
                dmin = std::min(dmin, dp[i]);
                dsum += dp[i];
            }
            if (!(dmin > 0.0)) fail(MGMC_ERR_NOT_SPD, "stencil diagonal must be positive");
            lv.diag = dsum / (double)geo.n;  // a representative value; the kernels read the field
            upload_field(lv);
        }
        if (!(lv.diag > 0.0)) fail(MGMC_ERR_NOT_SPD, "stencil diagonal must be positive");
        lv.sd = std::sqrt(lv.diag * (2. - P.omega) / P.omega);
        lv.ncol = colour_count(dim, st);
        lv.npt = stencil_npt(lv.ncol, st);
        // programmatic dependent launch pays off for the short kernels of
        // the coarser levels; the many-CTA kernels of large levels run
        // without its per-CTA wait
        lv.g.pdl = geo.n <= PDL_MAX_POINTS ? 1 : 0;
        L.push_back(std::move(lv));
    }
    for (auto &lv : L) {
        lv.x = talloc(lv.geo.nalloc);
        lv.f = talloc(lv.geo.nalloc);
    }
    for (size_t lev = 0; lev + 1 < L.size(); ++lev) make_tile_maps(L[lev]);
    d_cvec = alloc<double>(L[0].geo.n);
    if (fp32 && P.ordering == MGMC_ORDER_MULTICOLOUR && L[0].npt == 7 && L[0].g.sy % 8 == 0 && L[0].g.sz % 8 == 0) {
        fhalf = (L[0].geo.nalloc / 2 + 64) / 64 * 64;
        fsplit = alloc<float>((size_t)2 * fhalf);
        CK(cudaMemsetAsync(fsplit, 0, (size_t)2 * fhalf * sizeof(float), stream));
    }
    // low-rank term on every level: B_{l+1} = R B_l
    if (m > 0) {
        SparseCols B;
        B.m = m;
        B.ptr.assign(op.B_colptr, op.B_colptr + m + 1);
        for (int j = 0; j < m; ++j) {
            for (i64 e = op.B_colptr[j]; e < op.B_colptr[j + 1]; ++e) {
                if (op.B_rowidx[e] < 0 || op.B_rowidx[e] >= L[0].geo.n) fail(MGMC_ERR_INVALID_ARGUMENT, "B row index out of range");
                if (e > op.B_colptr[j] && op.B_rowidx[e] <= op.B_rowidx[e - 1]) fail(MGMC_ERR_INVALID_ARGUMENT, "B row indices must ascend within a column");
            }
        }
        B.row.assign(op.B_rowidx, op.B_rowidx + op.B_colptr[m]);
        B.val.assign(op.B_val, op.B_val + op.B_colptr[m]);
        Sigma.assign(op.Sigma, op.Sigma + m);
        for (double s : Sigma)
            if (!(s > 0.0)) fail(MGMC_ERR_INVALID_ARGUMENT, "Sigma entries must be positive");
        L[0].Bh = B;
        for (size_t lev = 1; lev < L.size(); ++lev) L[lev].Bh = restrict_columns(L[lev - 1].geo, L[lev - 1].Bh);
        std::vector<double> si(m), ss(m);
        for (int j = 0; j < m; ++j) {
            si[j] = 1.0 / Sigma[j];
            ss[j] = std::sqrt(Sigma[j]);  // Sigma^{1/2}: scale of the low-rank noise term Sigma w
        }
        d_sigma_inv = upload(si);
        d_sigma_sqrt = upload(ss);
        d_sigma_sqrt_ff = upload(float_float(ss));
        const size_t lr_smem = sizeof(double) * (2 * (size_t)m + 256);
        if (lr_smem > 48 * 1024) {
            raise_smem_limit(k_lr_apply<float, NOISE_NONE>, lr_smem);
            raise_smem_limit(k_lr_apply<float, NOISE_PHILOX>, lr_smem);
            raise_smem_limit(k_lr_apply<float, NOISE_INJECTED>, lr_smem);
            raise_smem_limit(k_lr_apply<double, NOISE_NONE>, lr_smem);
            raise_smem_limit(k_lr_apply<double, NOISE_PHILOX>, lr_smem);
            raise_smem_limit(k_lr_apply<double, NOISE_INJECTED>, lr_smem);
        }
        for (size_t lev = 0; lev < L.size(); ++lev) build_lowrank((int)lev);
    }
    if (chol) build_coarse();
    // noise per step (dry count)
    noise_per_step = 0;
    {
        counting = true;
        i64 off0 = noise_off;
        noise_off = 0;
        // count without launching: replicate the recursion on the host
        std::function<void(int)> cnt = [&](int lev) {
            const int nlev = (int)L.size();
            const i64 per_sor = L[lev].geo.n + m;
            if (lev == nlev - 1) {
                noise_per_step += chol ? L[lev].geo.n : 2 * P.ncoarsesmooth * per_sor;
                return;
            }
            const int cyc = lev > 0 ? P.cycle : 1;
            for (int j = 0; j < cyc; ++j) {
                noise_per_step += (P.smoother == MGMC_SMOOTHER_SSOR ? 2 : 1) * (i64)P.npresmooth * per_sor;
                cnt(lev + 1);
                noise_per_step += (P.smoother == MGMC_SMOOTHER_SSOR ? 2 : 1) * (i64)P.npostsmooth * per_sor;
            }
        };
        cnt(0);
        noise_off = off0;
        counting = false;
    }
    autotune_sweeps();
    CK(cudaStreamSynchronize(stream));
    check_launch();
}

// A level's host field to the device: padded, in FP64 and (FP32 chains) in
// FP32 as well; ghosts stay zero.
void Sampler::upload_field(Level &lv) {
    const i64 n = lv.geo.n, na = lv.geo.nalloc;
    const int planes = lv.var == 1 ? 1 : 27;
    std::vector<double> pad((size_t)planes * na, 0.0);
    for (int k = 0; k < planes; ++k)
        for (i64 i = 0; i < n; ++i) pad[(size_t)k * na + lv.geo.pad(i)] = lv.vh[(size_t)k * n + i];
    lv.vw64 = upload(pad);
    if (fp32) {
        std::vector<float> pf(pad.begin(), pad.end());
        lv.vw = upload(pf);
    } else {
        lv.vw = lv.vw64;
    }
}

// Autotuner of the colour passes' CTA shape: for every level that sweeps,
// time a few sweeps on scratch vectors for each CTA of 128 or 256 threads
// whose width fits the level's rows (the block shape does not change any
// result: every thread owns whole points or spans) and keep the fastest.
// MGMC_AUTOTUNE=0 keeps the heuristic shapes.
void Sampler::autotune_sweeps() {
    if (const char *e = std::getenv("MGMC_AUTOTUNE"))
        if (e[0] == '0') return;
    if (P.ordering != MGMC_ORDER_MULTICOLOUR) return;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    const int nlev = (int)L.size();
    for (int lev = 0; lev < nlev; ++lev) {
        if (lev == nlev - 1 && chol) break;
        Level &lv = L[lev];
        ensure_scratch(lev);
        const bool vec = fp32 && !exact && lv.npt == 7 && (lv.g.sy % 4) == 0 && (lv.g.sz % 4) == 0 && lv.var != 2;
        const int count = vec ? (lv.g.N0 + 8) / 8 : (lv.g.N0 + 1) / 2;
        int cap = 8;
        while (cap < count && cap < RBP_THREADS) cap *= 2;
        NoiseArgs nz{};
        nz.d_step = d_step;
        const int noise = noise_mode == NOISE_PHILOX ? NOISE_PHILOX : NOISE_NONE;
        float best = 1e30f;
        int best_tx = 0, best_nt = RBP_THREADS;
        // the level's own f (still zero, only read): level 0 then runs the
        // kernel variant the chain runs (the colour-split f); best of three
        for (int nt : {RBP_THREADS, RBP_THREADS / 2})
            for (int tx = 8; tx <= std::min(nt, 2 * cap); tx *= 2) {
                lv.sweep_tx = tx;
                lv.sweep_threads = nt;
                for (int r = 0; r < 2; ++r) launch_sweep(*this, lv, true, noise, lv.s1, lv.f, nz, fp32, exact);
                for (int trial = 0; trial < 3; ++trial) {
                    CK(cudaEventRecord(e0, stream));
                    for (int r = 0; r < 4; ++r)
                        launch_sweep(*this, lv, r % 2 == 0, noise, lv.s1, lv.f, nz, fp32, exact);
                    CK(cudaEventRecord(e1, stream));
                    CK(cudaEventSynchronize(e1));
                    float ms = 0.f;
                    CK(cudaEventElapsedTime(&ms, e0, e1));
                    if (ms < best) {
                        best = ms;
                        best_tx = tx;
                        best_nt = nt;
                    }
                }
            }
        lv.sweep_tx = best_tx;
        lv.sweep_threads = best_nt;
        CK(cudaMemsetAsync(lv.s1, 0, (size_t)lv.geo.nalloc * tsize(), stream));
    }
    CK(cudaEventDestroy(e0));
    CK(cudaEventDestroy(e1));
    check_launch();
}

void Sampler::ensure_scratch(int lev) {
    Level &lv = L[lev];
    if (!lv.s1) lv.s1 = talloc(lv.geo.nalloc);
    if (!lv.s2) lv.s2 = talloc(lv.geo.nalloc);
}

// host / device compact FP64 vector -> padded T array of level lev
// Device address through which kernels can read or write a host array
// directly: page-locked (cudaHostAlloc / cudaHostRegister) memory is mapped
// into the device's address space, so the conversion kernels move the data
// across the host link themselves (one pass, no staging copy); null for
// pageable memory.
static void *mapped_host(const void *p) {
    cudaPointerAttributes pa;
    if (cudaPointerGetAttributes(&pa, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return pa.type == cudaMemoryTypeHost ? pa.devicePointer : nullptr;
}

static dim3 pack_grid(const Level &lv) { return dim3((lv.g.N0 + 255) / 256, lv.g.N1, lv.g.N2); }

void Sampler::refresh_fsplit() {
    if (!fsplit) return;
    const Level &l0 = L[0];
    k_split_colours<<<pack_grid(l0), 256, 0, stream>>>((const float *)l0.f, fsplit, fhalf, l0.g);
    check_launch();
}

// as_f64: dst is an FP64 array whatever the chain's precision
static void put_vec(Sampler &S, int lev, const double *src, int on_device, void *dst, bool as_f64 = false) {
    Level &lv = S.L[lev];
    const i64 n = lv.geo.n;
    if (n > S.L[0].geo.n) fail(MGMC_ERR_INVALID_ARGUMENT, "level size");
    const double *d = src;
    if (!on_device) {
        d = (const double *)mapped_host(src);
        if (!d) {
            CK(cudaMemcpyAsync(S.d_cvec, src, n * sizeof(double), cudaMemcpyHostToDevice, S.stream));
            d = S.d_cvec;
        }
    }
    if (S.fp32 && !as_f64)
        k_unpack<float><<<pack_grid(lv), 256, 0, S.stream>>>(d, (float *)dst, lv.g);
    else
        k_unpack<double><<<pack_grid(lv), 256, 0, S.stream>>>(d, (double *)dst, lv.g);
    S.check_launch();
}

static void get_vec(Sampler &S, int lev, const void *src, double *dst, int on_device, bool as_f64 = false) {
    Level &lv = S.L[lev];
    const i64 n = lv.geo.n;
    double *d = dst;
    bool staged = false;
    if (!on_device) {
        d = (double *)mapped_host(dst);
        if (!d) {
            d = S.d_cvec;
            staged = true;
        }
    }
    if (S.fp32 && !as_f64)
        k_pack<float><<<pack_grid(lv), 256, 0, S.stream>>>((const float *)src, d, lv.g);
    else
        k_pack<double><<<pack_grid(lv), 256, 0, S.stream>>>((const double *)src, d, lv.g);
    S.check_launch();
    if (staged) CK(cudaMemcpyAsync(dst, S.d_cvec, n * sizeof(double), cudaMemcpyDeviceToHost, S.stream));
    if (!on_device) CK(cudaStreamSynchronize(S.stream));
}

// Capture one step into a CUDA graph (Philox noise: the step's launches and
// arguments never change; the noise streams advance through the device
// step counter).
// Error bits raised on the device: 1 = non-finite observable, 2 = a tile
// copy wait ran out.
static void check_device_errors(Sampler &S) {
    unsigned err = 0;
    CK(cudaMemcpy(&err, S.d_err, sizeof(err), cudaMemcpyDeviceToHost));
    if (err & ERR_TILE_TIMEOUT) fail(MGMC_ERR_CUDA, "a shared-memory tile copy did not complete in time");
    if (err) fail(MGMC_ERR_NONFINITE, "non-finite observable in the chain");
}

static void ensure_graph(Sampler &S) {
    if (S.gexec) return;
    CK(cudaStreamBeginCapture(S.stream, cudaStreamCaptureModeThreadLocal));
    try {
        S.launch_step();
    } catch (...) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(S.stream, &g);
        if (g) cudaGraphDestroy(g);
        throw;
    }
    CK(cudaStreamEndCapture(S.stream, &S.graph));
    CK(cudaGraphInstantiate(&S.gexec, S.graph, 0));
}

static void run_steps(Sampler &S, i64 nsteps) {
    if (S.noise_mode == NOISE_INJECTED) {
        for (i64 k = 0; k < nsteps; ++k) {
            if (S.noise_len - S.noise_pos < S.noise_per_step)
                fail(MGMC_ERR_NOISE_EXHAUSTED, "injected noise exhausted: " + std::to_string(S.noise_len - S.noise_pos) +
                                                   " queued, " + std::to_string(S.noise_per_step) + " needed per step");
            S.launch_step();
            S.check_launch();
            S.noise_pos += S.noise_per_step;
        }
        return;
    }
    ensure_graph(S);
    for (i64 k = 0; k < nsteps; ++k) CK(cudaGraphLaunch(S.gexec, S.stream));
}

// ------------------------------------------------- deterministic solver
// LoopSolver (loop_solver.cc:9-53) around MultigridPreconditioner
// (multigrid_preconditioner.cc:8-108) on this hierarchy.  The
// preconditioner is the sampler's cycle with the noise switched off: the
// same sweeps with their low-rank corrections, residual-restriction,
// prolongation and coarse scaling, from a zero state, with the Cholesky
// coarse solve.  Two graphs: the FP64 residual r = b - A x with |r|^2 (and
// the preconditioner's input f_0 = r, x_0 = 0), and the cycle followed by
// x += P r.
void Sampler::ensure_solver_buffers() {
    Level &l0 = L[0];
    const i64 na = l0.geo.nalloc;
    if (!sv_x) {
        sv_x = alloc<double>(na);
        sv_b = alloc<double>(na);
        sv_r = alloc<double>(na);
        for (double *p : {sv_x, sv_b, sv_r}) CK(cudaMemsetAsync(p, 0, (size_t)na * sizeof(double), stream));
        const i64 nrows = (i64)l0.g.N1 * l0.g.N2;
        sv_np = (int)((nrows + SOLVE_ROWS - 1) / SOLVE_ROWS);
        sv_part = alloc<double>(sv_np);
        sv_norm = alloc<double>(1);
        sv_keep_x = talloc(na);
        sv_keep_f = talloc(na);
    }
}

void Sampler::ensure_solver() {
    if (rexec && pexec) return;
    if (!dLinv) build_coarse();
    ensure_solver_buffers();
    Level &l0 = L[0];
    const i64 na = l0.geo.nalloc;
    auto capture = [&](cudaGraph_t &g, cudaGraphExec_t &ge, const std::function<void()> &body) {
        CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        try {
            body();
            check_launch();
        } catch (...) {
            noisy = true;
            cudaGraph_t gg = nullptr;
            cudaStreamEndCapture(stream, &gg);
            if (gg) cudaGraphDestroy(gg);
            throw;
        }
        CK(cudaStreamEndCapture(stream, &g));
        CK(cudaGraphInstantiate(&ge, g, 0));
    };
    if (!rexec)
        capture(rgraph, rexec, [&]() {
            const StencilArg<double> st = stencil_arg<double>(l0, P.omega);
            const VarField<double> vf{l0.vw64, l0.geo.nalloc};
            if (l0.var == 2) {
                k_solve_resid<27, 2><<<pack_grid(l0), 256, 0, stream>>>(sv_x, sv_b, sv_r, l0.g, st, vf);
            } else if (l0.var == 1) {
                if (l0.npt == 7)
                    k_solve_resid<7, 1><<<pack_grid(l0), 256, 0, stream>>>(sv_x, sv_b, sv_r, l0.g, st, vf);
                else
                    k_solve_resid<27, 1><<<pack_grid(l0), 256, 0, stream>>>(sv_x, sv_b, sv_r, l0.g, st, vf);
            } else if (l0.npt == 7) {
                k_solve_resid<7, 0><<<pack_grid(l0), 256, 0, stream>>>(sv_x, sv_b, sv_r, l0.g, st, vf);
            } else {
                k_solve_resid<27, 0><<<pack_grid(l0), 256, 0, stream>>>(sv_x, sv_b, sv_r, l0.g, st, vf);
            }
            if (m > 0) {
                launch_bt_plain<double>(*this, l0, sv_x);
                launch_add_Bq<double>(*this, l0, sv_r, l0.y, -1.0);
            }
            if (fp32)
                k_solve_rhs<float><<<sv_np, 256, 0, stream>>>(sv_r, (float *)l0.f, (float *)l0.x, l0.g, sv_part);
            else
                k_solve_rhs<double><<<sv_np, 256, 0, stream>>>(sv_r, (double *)l0.f, (double *)l0.x, l0.g, sv_part);
            k_solve_norm<<<1, 256, 0, stream>>>(sv_part, sv_np, sv_norm);
            refresh_fsplit();  // the cycle's fine sweeps read f = r through the colour split
        });
    if (!pexec)
        capture(pgraph, pexec, [&]() {
            noisy = false;
            sample(0);
            noisy = true;
            const unsigned blocks = (unsigned)std::min<i64>(nblk(na, 256), 8 * nsm);
            if (fp32)
                k_solve_update<float><<<blocks, 256, 0, stream>>>(sv_x, (const float *)l0.x, na);
            else
                k_solve_update<double><<<blocks, 256, 0, stream>>>(sv_x, (const double *)l0.x, na);
        });
}

// Edge weights of the fine stencil for the exact sampler's perturbation
// (k_prior_perturbation): symmetric, non-positive off-diagonal weights and
// a non-negative diagonal surplus.
void Sampler::ensure_exact() {
    if (ew_ready) return;
    const double *w = L[0].st;
    double off = 0.0;
    for (int k = 0; k < 27; ++k) {
        if (k == 13) continue;
        if (w[k] > 0.0 || w[k] != w[26 - k])
            fail(MGMC_ERR_UNSUPPORTED, "the exact sampler needs a symmetric stencil with non-positive off-diagonal weights");
        off -= w[k];
    }
    double cmin = w[13];
    if (L[0].var == 1)
        for (double d : L[0].vh) cmin = std::min(cmin, d);
    else if (L[0].var == 2)
        fail(MGMC_ERR_UNSUPPORTED, "the exact sampler needs constant off-diagonal weights");
    if (cmin - off < -1e-12 * cmin) fail(MGMC_ERR_UNSUPPORTED, "the exact sampler needs a weakly diagonally dominant stencil");
    ew.c0 = std::sqrt(std::max(w[13] - off, 0.0));
    ex_offsum = off;
    for (int k = 14; k < 27; ++k) {
        ew.ck[k - 14] = std::sqrt(-w[k]);
        ew.off[k - 14][0] = k % 3 - 1;
        ew.off[k - 14][1] = (k / 3) % 3 - 1;
        ew.off[k - 14][2] = k / 9 - 1;
    }
    ex_y = alloc<double>((size_t)std::max(m, 1));
    ew_ready = true;
}

// The chain's x_0 and f_0 are borrowed by a solve and put back afterwards.
struct BorrowLevel0 {
    Sampler &S;
    explicit BorrowLevel0(Sampler &s) : S(s) {
        const size_t bytes = (size_t)S.L[0].geo.nalloc * S.tsize();
        CK(cudaMemcpyAsync(S.sv_keep_x, S.L[0].x, bytes, cudaMemcpyDeviceToDevice, S.stream));
        CK(cudaMemcpyAsync(S.sv_keep_f, S.L[0].f, bytes, cudaMemcpyDeviceToDevice, S.stream));
    }
    ~BorrowLevel0() {
        const size_t bytes = (size_t)S.L[0].geo.nalloc * S.tsize();
        cudaMemcpyAsync(S.L[0].x, S.sv_keep_x, bytes, cudaMemcpyDeviceToDevice, S.stream);
        cudaMemcpyAsync(S.L[0].f, S.sv_keep_f, bytes, cudaMemcpyDeviceToDevice, S.stream);
        if (S.fsplit)
            k_split_colours<<<dim3((S.L[0].g.N0 + 255) / 256, S.L[0].g.N1, S.L[0].g.N2), 256, 0, S.stream>>>(
                (const float *)S.L[0].f, S.fsplit, S.fhalf, S.L[0].g);
        cudaStreamSynchronize(S.stream);
    }
};

// ------------------------------------------------------------- adjoint
// Transpose of the linear part of one MGMC step with its noise held fixed.
// With fixed noise a step is affine: x' = Phi x + K f + (noise terms); the
// adjoint maps x-bar' to Phi^T x-bar' and adds K^T x-bar' to f-bar.  It is
// assembled from the forward kernels: a sweep of direction d is
// x <- x + M_d^{-1}(c - A_0 x), M_d = D / omega + (A_0's part before the
// point in the sweep order), and for symmetric A_0, M_d^T is the splitting
// of the opposite direction, so M_d^{-T} v is a noise-free sweep of the
// opposite direction from x = 0 with right hand side v.  The low-rank
// correction x <- (I - C S^{-1} B^T) x (C = M_d^{-1} B) has transpose
// I - B S^{-T} B^T M_d^{-T}; R = P^T; the coarse Cholesky sample
// L^{-T}(xi + L^{-1} f) has the symmetric linear part Q_c^{-1}.  No
// counterpart in the reference.
void Sampler::ensure_adjoint() {
    for (auto &lv : L)
        for (int k = 0; k < 4; ++k)
            if (!lv.adj[k]) lv.adj[k] = talloc(lv.geo.nalloc);
    if (!adj_m) adj_m = alloc<double>((size_t)std::max(m, 1));
}

template <typename T>
static void adj_zero(Sampler &S, const Level &lv, void *v) {
    CK(cudaMemsetAsync(v, 0, (size_t)lv.geo.nalloc * sizeof(T), S.stream));
}

template <typename T>
static void adj_axpy(Sampler &S, const Level &lv, void *y, const void *x, double alpha) {
    const unsigned blocks = (unsigned)std::min<i64>(nblk(lv.geo.nalloc, 256), 8 * S.nsm);
    plaunch(false, k_axpy<T>, blocks, 256, 0, S.stream, (T *)y, (const T *)x, (T)alpha, (i64)lv.geo.nalloc);
}

// y = A_0 x on a level (constant or variable stencil)
template <typename T>
static void launch_apply_stencil(Sampler &S, const Level &lv, const void *x, void *y) {
    const StencilArg<T> s = stencil_arg<T>(lv, S.P.omega);
    const VarField<T> vf = var_field<T>(lv);
    const unsigned nb = nblk(lv.geo.n, 256);
    if (lv.var == 1)
        plaunch(false, k_apply_stencil<T, 1>, nb, 256, 0, S.stream, (const T *)x, (T *)y, lv.g, s, vf);
    else if (lv.var == 2)
        plaunch(false, k_apply_stencil<T, 2>, nb, 256, 0, S.stream, (const T *)x, (T *)y, lv.g, s, vf);
    else
        plaunch(false, k_apply_stencil<T, 0>, nb, 256, 0, S.stream, (const T *)x, (T *)y, lv.g, s, vf);
}

// out = M^{-T} v for the sweep of direction `forward` on level lev
template <typename T>
static void adj_msolve(Sampler &S, int lev, bool forward, const void *v, void *out) {
    Level &lv = S.L[lev];
    adj_zero<T>(S, lv, out);
    NoiseArgs nz{};
    nz.d_step = S.d_step;
    launch_sweep(S, lv, !forward, NOISE_NONE, out, v, nz, S.fp32, false);
}

template <typename T>
static void adj_apply_a0(Sampler &S, Level &lv, const void *x, void *y) {
    launch_apply_stencil<T>(S, lv, x, y);
}

// adjoint of one SOR sweep of direction `forward` with its low-rank
// correction: a = x-bar (in/out), b = f-bar (accumulated)
template <typename T>
static void adjoint_sor(Sampler &S, int lev, bool forward) {
    Level &lv = S.L[lev];
    void *a = lv.adj[0], *b = lv.adj[1], *w = lv.adj[2], *u = lv.adj[3];
    if (S.m > 0) {
        adj_msolve<T>(S, lev, forward, a, w);  // w = M^{-T} a
        launch_bt_plain<T>(S, lv, w);          // y = B^T w
        k_sinvt_q<<<(S.m + 255) / 256, 256, 0, S.stream>>>(lv.SinvT[forward ? 0 : 1], lv.y, S.d_sigma_sqrt, S.adj_m, S.m);
        launch_add_Bq<T>(S, lv, a, S.adj_m, -1.0);  // a -= B S^{-T} y
    }
    adj_msolve<T>(S, lev, forward, a, u);  // u = M^{-T} a
    if (S.param_adj) S.pgrad_sweep<T>(S.tape_pop(Sampler::EV_SWEEP, lev, forward), u);
    adj_axpy<T>(S, lv, b, u, 1.0);        // f-bar += u
    adj_apply_a0<T>(S, lv, u, w);
    adj_axpy<T>(S, lv, a, w, -1.0);       // a -= A_0 u
}

// MultigridMCSampler::sample in reverse: on entry L[lev].adj[0] is the
// adjoint of the level's output state, on return the adjoint of its input
// state, and L[lev].adj[1] has accumulated the adjoint of its right hand side.
template <typename T>
void Sampler::adjoint_sample(int lev) {
    const int nlev = (int)L.size();
    Level &lv = L[lev];
    if (lev == nlev - 1) {
        if (chol) {
            // f-bar += Q_c^{-1} x-bar; the coarse sample does not read its input state
            const i64 n = lv.geo.n;
            const unsigned blocks = (unsigned)((n + 7) / 8);
            NoiseArgs nz{};
            plaunch(false, k_chol_gemv_lower<T, T, NOISE_NONE>, blocks, 256, chol_smem, stream, (const T *)lv.adj[0], lv.g,
                    (const T *)dLinv, chol_ld, (T *)dgv, nz);
            adj_zero<T>(*this, lv, lv.adj[2]);
            plaunch(false, k_chol_gemv_upper<T, T>, blocks, 256, chol_smem, stream, (const T *)dgv, lv.g, (const T *)dLinvT,
                    chol_ld, (T *)lv.adj[2]);
            if (param_adj) pgrad_coarse<T>(tape_pop(EV_COARSE, lev, true));
            adj_axpy<T>(*this, lv, lv.adj[1], lv.adj[2], 1.0);
        } else {
            for (int k = P.ncoarsesmooth - 1; k >= 0; --k) {
                adjoint_sor<T>(*this, lev, false);
                adjoint_sor<T>(*this, lev, true);
            }
        }
        // a coarse level starts from zero, and the Cholesky sample does not
        // read its input; a one-level SSOR sampler's input is the chain's
        // state, whose adjoint the sweeps above have formed
        if (chol || lev > 0) adj_zero<T>(*this, lv, lv.adj[0]);
        return;
    }
    Level &lc = L[lev + 1];
    const int cyc = lev > 0 ? P.cycle : 1;
    const bool ssor = P.smoother == MGMC_SMOOTHER_SSOR;
    for (int j = cyc - 1; j >= 0; --j) {
        for (int k = P.npostsmooth - 1; k >= 0; --k) {
            if (ssor) {
                adjoint_sor<T>(*this, lev, false);
                adjoint_sor<T>(*this, lev, true);
            } else {
                adjoint_sor<T>(*this, lev, false);
            }
        }
        // x += alpha P x_c  ->  x_c-bar = alpha R x-bar
        launch_resid_restrict<T>(*this, lev, lv.adj[0], lv.adj[0], lc.adj[2], nullptr, true);
        adj_zero<T>(*this, lc, lc.adj[0]);
        adj_axpy<T>(*this, lc, lc.adj[0], lc.adj[2], P.coarse_scaling);
        adj_zero<T>(*this, lc, lc.adj[1]);
        adjoint_sample<T>(lev + 1);
        // f_c = R (f - A x)  ->  t = P f_c-bar; f-bar += t; x-bar -= A t
        void *t = lv.adj[2], *u = lv.adj[3];
        adj_zero<T>(*this, lv, t);
        prolong(lev, 1.0, lc.adj[1], t);
        if (param_adj) pgrad_minus_udav<T>(lev, t, tape_pop(EV_RESID, lev, true).xin);
        adj_axpy<T>(*this, lv, lv.adj[1], t, 1.0);
        adj_apply_a0<T>(*this, lv, t, u);
        if (m > 0) {
            launch_bt_plain<T>(*this, lv, t);
            launch_add_Bq<T>(*this, lv, u, lv.y, 1.0);
        }
        adj_axpy<T>(*this, lv, lv.adj[0], u, -1.0);
        for (int k = P.npresmooth - 1; k >= 0; --k) {
            if (ssor) {
                adjoint_sor<T>(*this, lev, false);
                adjoint_sor<T>(*this, lev, true);
            } else {
                adjoint_sor<T>(*this, lev, true);
            }
        }
    }
}


// ------------------------------------------------------ parameter adjoint
void *Sampler::tape_snap(int lev, const void *src) {
    auto &pool = tape_pool[lev];
    int &k = tape_next[lev];
    if (k == (int)pool.size()) pool.push_back(talloc(L[lev].geo.nalloc));
    void *dst = pool[k++];
    CK(cudaMemcpyAsync(dst, src, (size_t)L[lev].geo.nalloc * tsize(), cudaMemcpyDeviceToDevice, stream));
    return dst;
}

void *Sampler::tape_state(int lev) {
    if (!tape_last[lev]) tape_last[lev] = tape_snap(lev, L[lev].x);
    return tape_last[lev];
}

Sampler::TapeEvent Sampler::tape_pop(int kind, int lev, bool forward) {
    if (tape.empty()) fail(MGMC_ERR_INVALID_ARGUMENT, "parameter adjoint: tape exhausted");
    TapeEvent ev = tape.back();
    if (ev.kind != kind || ev.lev != lev || (kind == EV_SWEEP && ev.forward != forward))
        fail(MGMC_ERR_INVALID_ARGUMENT, "parameter adjoint: tape out of order");
    tape.pop_back();
    return ev;
}

// dA_0/ds per level (the Galerkin stencils of the unit centre weight), the
// gradient accumulators, and for the Cholesky coarse level
// Phi(L^{-1} E_c L^{-T}) and L^{-1} B_c.
void Sampler::ensure_param_adjoint() {
    ensure_adjoint();
    if (pa_gs) return;
    for (const auto &lv : L)
        if (lv.var) fail(MGMC_ERR_UNSUPPORTED, "parameter derivatives need a constant stencil");
    const int nl = (int)L.size();
    pa_E.assign(nl, std::array<double, 27>{});
    pa_E[0][13] = 1.0;
    for (int l = 1; l < nl; ++l) galerkin_stencil(dim, pa_E[l - 1].data(), pa_E[l].data());
    tape_pool.assign(nl, {});
    tape_next.assign(nl, 0);
    tape_last.assign(nl, nullptr);
    tape_f.assign(nl, nullptr);
    const i64 np0 = ((i64)L[0].g.N1 * L[0].g.N2 + SOLVE_ROWS - 1) / SOLVE_ROWS;
    i64 cap = 8 * np0;
    const int mm = std::max(m, 1);
    pa_Bu = alloc<double>(mm);
    pa_Bv = alloc<double>(mm);
    pa_xi = alloc<double>(mm);
    for (double *p : {pa_Bu, pa_Bv, pa_xi}) CK(cudaMemsetAsync(p, 0, mm * sizeof(double), stream));
    if (chol) {
        Level &lv = L.back();
        const i64 n = lv.geo.n, ld = chol_ld;
        cap = std::max<i64>(cap, (n + 7) / 8);
        std::vector<double> Q = dense_precision(lv.geo, lv.st, lv.Bh, Sigma);
        if (!dense_cholesky(Q, n)) fail(MGMC_ERR_NOT_SPD, "coarse precision matrix is not positive definite");
        const std::vector<double> Tt = inverse_factor_transposed(Q, n);
        const std::vector<double> phi = cholesky_phi_sandwich(Tt, lv.geo, pa_E.back().data());
        if (fp32) {
            std::vector<float> M((size_t)n * ld, 0.0f);
            for (i64 i = 0; i < n; ++i)
                for (i64 j = 0; j <= i; ++j) M[(size_t)i * ld + j] = (float)phi[(size_t)i * n + j];
            pa_phi = upload(M);
        } else {
            std::vector<double> M((size_t)n * ld, 0.0);
            for (i64 i = 0; i < n; ++i)
                for (i64 j = 0; j <= i; ++j) M[(size_t)i * ld + j] = phi[(size_t)i * n + j];
            pa_phi = upload(M);
        }
        if (m > 0) pa_U = upload(inverse_factor_times(Tt, n, lv.Bh));
        pa_xic = alloc<double>(n);
        pa_cv = alloc<char>((size_t)ld * tsize());
        pa_mu = talloc(lv.geo.nalloc);
        if (chol_smem > 48 * 1024) {
            raise_smem_limit(k_pgrad_coarse_phi<float>, chol_smem);
            raise_smem_limit(k_pgrad_coarse_phi<double>, chol_smem);
        }
    }
    pa_part = alloc<double>(cap);
    pa_part_cap = (int)cap;
    pa_gs = alloc<double>(1);
    pa_gsig = alloc<double>(mm);
    CK(cudaStreamSynchronize(stream));
}

static PgradStencils pgrad_stencils(const Level &lv, const std::array<double, 27> &E) {
    PgradStencils st;
    for (int k = 0; k < 27; ++k) {
        st.a[k] = lv.st[k];
        st.e[k] = E[k];
        st.af[k] = (float)lv.st[k];
        st.ef[k] = (float)E[k];
    }
    return st;
}

template <typename T>
static void launch_pgrad_stencil(Sampler &S, const Level &lv, const std::array<double, 27> &E, const void *u,
                                 const void *v, const void *w, const void *f, int ncol, bool forward, int np) {
    const PgradStencils st = pgrad_stencils(lv, E);
    bool has_e = false;
    for (int k = 0; k < 27; ++k) has_e |= (k != 13 && E[k] != 0.0);
    const T *U = (const T *)u, *V = (const T *)v, *W = (const T *)w, *F = (const T *)f;
    const int fw = forward ? 1 : 0;
    if (lv.npt == 7) {
        if (has_e)
            k_pgrad_stencil<T, 7, true><<<np, 256, 0, S.stream>>>(U, V, W, F, lv.g, st, ncol, fw, S.pa_part);
        else
            k_pgrad_stencil<T, 7, false><<<np, 256, 0, S.stream>>>(U, V, W, F, lv.g, st, ncol, fw, S.pa_part);
    } else {
        if (has_e)
            k_pgrad_stencil<T, 27, true><<<np, 256, 0, S.stream>>>(U, V, W, F, lv.g, st, ncol, fw, S.pa_part);
        else
            k_pgrad_stencil<T, 27, false><<<np, 256, 0, S.stream>>>(U, V, W, F, lv.g, st, ncol, fw, S.pa_part);
    }
}

// One sweep's contribution: u = M_f^{-T} x-bar'' of the sweep, its input
// and output states and right hand side from the tape.
template <typename T>
void Sampler::pgrad_sweep(const TapeEvent &ev, const void *u) {
    Level &lv = L[ev.lev];
    const int ncol = P.ordering == MGMC_ORDER_LEXICOGRAPHIC ? 0 : lv.ncol;
    const int np = (int)(((i64)lv.g.N1 * lv.g.N2 + SOLVE_ROWS - 1) / SOLVE_ROWS);
    launch_pgrad_stencil<T>(*this, lv, pa_E[ev.lev], u, ev.xout, ev.xin, ev.f, ncol, ev.forward, np);
    if (m > 0) {
        launch_bt_plain<T>(*this, lv, u, pa_Bu);
        launch_bt_plain<T>(*this, lv, ev.xout, pa_Bv);
        if (noise_mode == NOISE_PHILOX)
            k_lowrank_normals<NOISE_PHILOX><<<nblk(m, 256), 256, 0, stream>>>(ev.nzl, m, pa_xi);
        else
            k_lowrank_normals<NOISE_INJECTED><<<nblk(m, 256), 256, 0, stream>>>(ev.nzl, m, pa_xi);
    }
    const double ac = lv.diag, ec = pa_E[ev.lev][13];
    const PgradCoef cf{ec / (2.0 * ac), P.omega, ac, ec, 0};
    k_pgrad_combine<<<1, 256, 0, stream>>>(pa_part, np, pa_Bu, pa_Bv, pa_xi, d_sigma_inv, d_sigma_sqrt, m, cf, pa_gs,
                                           pa_gsig);
    check_launch();
}

// -u^T dA v on level lev: the residual f - A x (u = P f_c-bar, v = the
// state entering the residual) and the coarse mean Q^{-1} f (u = Q^{-1}
// x-bar, v = Q^{-1} f).
template <typename T>
void Sampler::pgrad_minus_udav(int lev, const void *u, const void *v) {
    Level &lv = L[lev];
    const int np = (int)(((i64)lv.g.N1 * lv.g.N2 + SOLVE_ROWS - 1) / SOLVE_ROWS);
    launch_pgrad_stencil<T>(*this, lv, pa_E[lev], u, v, v, v, 0, true, np);
    if (m > 0) {
        launch_bt_plain<T>(*this, lv, u, pa_Bu);
        launch_bt_plain<T>(*this, lv, v, pa_Bv);
    }
    const PgradCoef cf{0.0, P.omega, lv.diag, pa_E[lev][13], 1};
    k_pgrad_combine<<<1, 256, 0, stream>>>(pa_part, np, pa_Bu, pa_Bv, pa_xi, d_sigma_inv, d_sigma_sqrt, m, cf, pa_gs,
                                           pa_gsig);
    check_launch();
}

// The coarse Cholesky sample's contribution; on entry the level's adj[2]
// holds w1 = Q^{-1} x-bar and dgv holds w2 = L^{-1} x-bar.
template <typename T>
void Sampler::pgrad_coarse(const TapeEvent &ev) {
    typedef T MT;
    Level &lv = L[ev.lev];
    const i64 n = lv.geo.n;
    const unsigned blocks = (unsigned)((n + 7) / 8);
    if (noise_mode == NOISE_PHILOX)
        k_coarse_normals<NOISE_PHILOX><<<nblk(n, 256), 256, 0, stream>>>(ev.nzp, (int)n, pa_xic);
    else
        k_coarse_normals<NOISE_INJECTED><<<nblk(n, 256), 256, 0, stream>>>(ev.nzp, (int)n, pa_xic);
    k_pgrad_coarse_phi<MT><<<blocks, 256, chol_smem, stream>>>((const MT *)pa_phi, chol_ld, (const MT *)dgv, pa_xic, (int)n,
                                                               pa_part);
    k_accum_sum<<<1, 256, 0, stream>>>(pa_part, (int)blocks, -1.0, pa_gs);
    if (m > 0)
        k_pgrad_coarse_sigma<MT><<<m, 256, 0, stream>>>(pa_U, (const MT *)dgv, pa_xic, d_sigma_inv, pa_gsig, (int)n);
    NoiseArgs nz{};
    plaunch(false, k_chol_gemv_lower<T, MT, NOISE_NONE>, blocks, 256, chol_smem, stream, (const T *)ev.f, lv.g,
            (const MT *)dLinv, chol_ld, (MT *)pa_cv, nz);
    plaunch(false, k_chol_gemv_upper<T, MT>, blocks, 256, chol_smem, stream, (const MT *)pa_cv, lv.g, (const MT *)dLinvT,
            chol_ld, (T *)pa_mu);
    pgrad_minus_udav<T>(ev.lev, lv.adj[2], pa_mu);
}
// The replay of one step from level 0's state, recording the tape, and the
// reverse pass from level 0's adj[0], accumulating the parameter gradients
// (device work only, so that it can be captured).
void Sampler::param_adjoint_pass() {
    Level &l0 = L[0];
    const int mm = std::max(m, 1);
    tape.clear();
    std::fill(tape_next.begin(), tape_next.end(), 0);
    std::fill(tape_last.begin(), tape_last.end(), nullptr);
    std::fill(tape_f.begin(), tape_f.end(), nullptr);
    tape_f[0] = l0.f;
    inv = 0;
    noise_off = noise_pos;
    taping = true;
    sample(0);
    taping = false;
    check_launch();
    CK(cudaMemsetAsync(pa_gs, 0, sizeof(double), stream));
    CK(cudaMemsetAsync(pa_gsig, 0, mm * sizeof(double), stream));
    param_adj = true;
    if (fp32) {
        adj_zero<float>(*this, l0, l0.adj[1]);
        adjoint_sample<float>(0);
    } else {
        adj_zero<double>(*this, l0, l0.adj[1]);
        adjoint_sample<double>(0);
    }
    param_adj = false;
    check_launch();
    if (!tape.empty()) fail(MGMC_ERR_INVALID_ARGUMENT, "parameter adjoint: tape not consumed");
}

}  // namespace mgmc

// ===================================================================== ABI
using namespace mgmc;

struct mgmc_sampler {
    Sampler *impl;
};

#define API_BEGIN try {
#define API_END                                \
    }                                          \
    catch (const Error &e) {                   \
        g_err = e.msg;                         \
        return e.st;                           \
    }                                          \
    catch (const std::bad_alloc &) {           \
        g_err = "host allocation failed";      \
        return MGMC_ERR_OUT_OF_MEMORY;         \
    }                                          \
    catch (const std::exception &e) {          \
        g_err = e.what();                      \
        return MGMC_ERR_INVALID_ARGUMENT;      \
    }                                          \
    return MGMC_OK;

static Sampler &impl(mgmc_sampler *s) {
    if (!s || !s->impl) fail(MGMC_ERR_INVALID_ARGUMENT, "null sampler");
    CK(cudaSetDevice(s->impl->P.device));
    return *s->impl;
}

static void check_level(Sampler &S, int level, bool need_coarser) {
    if (level < 0 || level >= (int)S.L.size() || (need_coarser && level + 1 >= (int)S.L.size()))
        fail(MGMC_ERR_INVALID_ARGUMENT, "level out of range");
}

extern "C" {

int mgmc_abi_version(void) { return MGMC_ABI_VERSION; }

const char *mgmc_last_error(void) { return g_err.c_str(); }

mgmc_status mgmc_fd_stencil(int dim, int nx, int ny, int nz, double kappa_sq, double stencil[27]) {
    API_BEGIN
    if (dim < 1 || dim > 3 || !stencil) fail(MGMC_ERR_INVALID_ARGUMENT, "dim must be 1, 2 or 3");
    Geometry g(dim, nx, ny, nz);
    fd_stencil(g, kappa_sq, stencil);
    API_END
}

mgmc_status mgmc_measurement_vector(int dim, int nx, int ny, int nz, const double *x0, double radius, int64_t *idx,
                                    double *val, int64_t capacity, int64_t *nnz) {
    API_BEGIN
    if (dim < 1 || dim > 3 || !x0 || !nnz) fail(MGMC_ERR_INVALID_ARGUMENT, "bad arguments");
    Geometry g(dim, nx, ny, nz);
    auto r = measurement_vector(g, x0, radius);
    int64_t k = 0;
    for (auto &e : r) {
        if (k < capacity && idx && val) {
            idx[k] = e.first;
            val[k] = e.second;
        }
        ++k;
    }
    *nnz = k;
    API_END
}

mgmc_status mgmc_fem_field(int dim, int nx, int ny, int nz, int model, double p0, double p1, double *field) {
    API_BEGIN
    if (dim < 1 || dim > 3 || !field) fail(MGMC_ERR_INVALID_ARGUMENT, "dim must be 1, 2 or 3");
    if (model != 0 && model != 1) fail(MGMC_ERR_INVALID_ARGUMENT, "model must be 0 (constant) or 1 (periodic)");
    if (model == 1 && !(p0 > 0.0 && p1 >= p0)) fail(MGMC_ERR_INVALID_ARGUMENT, "periodic model needs 0 < Lambda_min <= Lambda_max");
    Geometry g(dim, nx, ny, nz);
    const std::vector<double> f = fem_field(g, model, p0, p1);
    std::copy(f.begin(), f.end(), field);
    API_END
}

mgmc_status mgmc_galerkin_stencil(int dim, const double fine[27], double coarse[27]) {
    API_BEGIN
    if (dim < 1 || dim > 3 || !fine || !coarse) fail(MGMC_ERR_INVALID_ARGUMENT, "bad arguments");
    galerkin_stencil(dim, fine, coarse);
    API_END
}

mgmc_status mgmc_operator_coarsen(const mgmc_operator_desc *op, double coarse_stencil[27], double *coarse_field,
                                  int64_t *Bc_colptr, int64_t *Bc_rowidx, double *Bc_val, int64_t cap, int64_t *nnz) {
    API_BEGIN
    if (!op || !coarse_stencil || !nnz) fail(MGMC_ERR_INVALID_ARGUMENT, "null argument");
    if (op->dim < 1 || op->dim > 3) fail(MGMC_ERR_INVALID_ARGUMENT, "dim must be 1, 2 or 3");
    const int cells[3] = {op->nx, op->dim > 1 ? op->ny : 2, op->dim > 2 ? op->nz : 2};
    for (int d = 0; d < op->dim; ++d)
        if (cells[d] < 2) fail(MGMC_ERR_LATTICE, "every active direction needs at least 2 cells");
    const Geometry g(op->dim, cells[0], cells[1], cells[2]);
    if (!g.coarsenable()) fail(MGMC_ERR_LATTICE, "cannot coarsen the lattice [odd extent or no interior vertices left]");
    if (op->m < 0 || (op->m > 0 && (!op->B_colptr || !op->B_rowidx || !op->B_val)))
        fail(MGMC_ERR_INVALID_ARGUMENT, "low-rank term needs B");
    if ((op->centre || op->field) && !coarse_field)
        fail(MGMC_ERR_INVALID_ARGUMENT, "a per-vertex operator needs coarse_field (27 x n_c doubles)");
    galerkin_stencil(op->dim, op->stencil, coarse_stencil);
    if (op->centre || op->field) {
        const std::vector<double> cf = galerkin_field(g, op->stencil, op->field ? nullptr : op->centre, op->field);
        std::copy(cf.begin(), cf.end(), coarse_field);
    }
    SparseCols B;
    B.m = op->m;
    if (op->m > 0) {
        B.ptr.assign(op->B_colptr, op->B_colptr + op->m + 1);
        for (int j = 0; j < op->m; ++j)
            for (i64 e = op->B_colptr[j]; e < op->B_colptr[j + 1]; ++e) {
                if (op->B_rowidx[e] < 0 || op->B_rowidx[e] >= g.n) fail(MGMC_ERR_INVALID_ARGUMENT, "B row index out of range");
                if (e > op->B_colptr[j] && op->B_rowidx[e] <= op->B_rowidx[e - 1])
                    fail(MGMC_ERR_INVALID_ARGUMENT, "B row indices must ascend within a column");
            }
        B.row.assign(op->B_rowidx, op->B_rowidx + op->B_colptr[op->m]);
        B.val.assign(op->B_val, op->B_val + op->B_colptr[op->m]);
    }
    const SparseCols Bc = op->m > 0 ? restrict_columns(g, B) : B;
    *nnz = Bc.ptr[op->m];
    if (Bc_colptr) std::copy(Bc.ptr.begin(), Bc.ptr.end(), Bc_colptr);
    if (Bc_rowidx || Bc_val) {
        if (!Bc_rowidx || !Bc_val || cap < *nnz) fail(MGMC_ERR_INVALID_ARGUMENT, "Bc arrays missing or shorter than nnz");
        std::copy(Bc.row.begin(), Bc.row.end(), Bc_rowidx);
        std::copy(Bc.val.begin(), Bc.val.end(), Bc_val);
    }
    API_END
}

mgmc_status mgmc_sampler_create(const mgmc_operator_desc *op, const mgmc_sampler_params *params, mgmc_sampler **out) {
    Sampler *S = nullptr;
    API_BEGIN
    if (!op || !params || !out) fail(MGMC_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    S = new Sampler();
    S->P = *params;
    S->build(*op);
    *out = new mgmc_sampler{S};
    S = nullptr;
    }
    catch (const Error &e) {
        delete S;
        g_err = e.msg;
        return e.st;
    }
    catch (const std::exception &e) {
        delete S;
        g_err = e.what();
        return MGMC_ERR_INVALID_ARGUMENT;
    }
    return MGMC_OK;
}

mgmc_status mgmc_sampler_destroy(mgmc_sampler *s) {
    API_BEGIN
    if (!s) return MGMC_OK;
    if (s->impl) {
        cudaSetDevice(s->impl->P.device);
        cudaStreamSynchronize(s->impl->stream);
    }
    delete s->impl;
    delete s;
    API_END
}

mgmc_status mgmc_sampler_fix_rhs(mgmc_sampler *s, const double *f, int on_device) {
    API_BEGIN
    Sampler &S = impl(s);
    if (!f) fail(MGMC_ERR_INVALID_ARGUMENT, "null f");
    put_vec(S, 0, f, on_device, S.L[0].f);
    S.refresh_fsplit();
    S.rhs_set = true;
    API_END
}

mgmc_status mgmc_sampler_set_state(mgmc_sampler *s, const double *x, int on_device) {
    API_BEGIN
    Sampler &S = impl(s);
    if (!x) fail(MGMC_ERR_INVALID_ARGUMENT, "null x");
    put_vec(S, 0, x, on_device, S.L[0].x);
    API_END
}

mgmc_status mgmc_sampler_get_state(mgmc_sampler *s, double *x, int on_device) {
    API_BEGIN
    Sampler &S = impl(s);
    if (!x) fail(MGMC_ERR_INVALID_ARGUMENT, "null x");
    get_vec(S, 0, S.L[0].x, x, on_device);
    API_END
}

mgmc_status mgmc_sampler_set_step_counter(mgmc_sampler *s, int64_t step) {
    API_BEGIN
    Sampler &S = impl(s);
    if (step < 0) fail(MGMC_ERR_INVALID_ARGUMENT, "step < 0");
    const u64 k = (u64)step;
    CK(cudaMemcpyAsync(S.d_step, &k, sizeof(u64), cudaMemcpyHostToDevice, S.stream));
    CK(cudaStreamSynchronize(S.stream));
    API_END
}

mgmc_status mgmc_sampler_get_step_counter(mgmc_sampler *s, int64_t *step) {
    API_BEGIN
    Sampler &S = impl(s);
    if (!step) fail(MGMC_ERR_INVALID_ARGUMENT, "null step");
    u64 k = 0;
    CK(cudaMemcpyAsync(&k, S.d_step, sizeof(u64), cudaMemcpyDeviceToHost, S.stream));
    CK(cudaStreamSynchronize(S.stream));
    *step = (int64_t)k;
    API_END
}

mgmc_status mgmc_sampler_step(mgmc_sampler *s, int64_t nsteps) {
    API_BEGIN
    Sampler &S = impl(s);
    if (nsteps < 0) fail(MGMC_ERR_INVALID_ARGUMENT, "nsteps < 0");
    run_steps(S, nsteps);
    API_END
}

mgmc_status mgmc_sampler_apply(mgmc_sampler *s, const double *f, double *x, int on_device) {
    API_BEGIN
    Sampler &S = impl(s);
    if (!x) fail(MGMC_ERR_INVALID_ARGUMENT, "null x");
    if (!f) {
        // the right hand side already on the device (Sampler::fix_rhs, then
        // apply(f, x) with the fixed f: sampling_time.cc:28-41): only x
        // travels
        if (!S.rhs_set) fail(MGMC_ERR_INVALID_ARGUMENT, "f is NULL but no right hand side has been set");
        put_vec(S, 0, x, on_device, S.L[0].x);
        run_steps(S, 1);
        get_vec(S, 0, S.L[0].x, x, on_device);
        CK(cudaStreamSynchronize(S.stream));
        check_device_errors(S);
        return MGMC_OK;
    }
    S.rhs_set = true;
    const double *fm = on_device ? f : (const double *)mapped_host(f);
    const double *xm = on_device ? x : (const double *)mapped_host(x);
    if (fm && xm) {
        Level &l0 = S.L[0];
        if (S.fp32)
            k_unpack2<float><<<pack_grid(l0), 256, 0, S.stream>>>(fm, xm, (float *)l0.f, (float *)l0.x, l0.g);
        else
            k_unpack2<double><<<pack_grid(l0), 256, 0, S.stream>>>(fm, xm, (double *)l0.f, (double *)l0.x, l0.g);
        S.check_launch();
    } else {
        put_vec(S, 0, f, on_device, S.L[0].f);
        put_vec(S, 0, x, on_device, S.L[0].x);
    }
    S.refresh_fsplit();
    run_steps(S, 1);
    get_vec(S, 0, S.L[0].x, x, on_device);
    CK(cudaStreamSynchronize(S.stream));
    check_device_errors(S);
    API_END
}

static void set_probes(Sampler &S, int nprobe, const int64_t *ptr, const int64_t *idx, const double *val,
                       int64_t capacity) {
    if (nprobe < 0 || capacity < 0 || (nprobe > 0 && (!ptr || !idx || !val))) fail(MGMC_ERR_INVALID_ARGUMENT, "bad observable");
    if (nprobe > 65535) fail(MGMC_ERR_UNSUPPORTED, "at most 65535 probes");
    CK(cudaStreamSynchronize(S.stream));
    const i64 nnz = nprobe > 0 ? ptr[nprobe] : 0;
    std::vector<i64> pptr(ptr, ptr + nprobe + 1), pidx(nnz);
    if (nprobe == 0) pptr.assign(1, 0);
    for (i64 e = 0; e < nnz; ++e) {
        if (idx[e] < 0 || idx[e] >= S.L[0].geo.n) fail(MGMC_ERR_INVALID_ARGUMENT, "observable index out of range");
        pidx[e] = S.L[0].geo.pad(idx[e]);
    }
    for (int q = 0; q < nprobe; ++q)
        if (pptr[q + 1] < pptr[q]) fail(MGMC_ERR_INVALID_ARGUMENT, "probe pointers must not decrease");
    std::vector<double> v(val, val + nnz);
    S.d_bptr = S.upload(pptr);
    S.d_bidx = S.upload(pidx);
    S.d_bval = S.upload(v);
    S.d_obs = S.alloc<double>((size_t)std::max<int64_t>(capacity, 1) * std::max(nprobe, 1));
    S.nprobe = nprobe;
    S.obs_cap = capacity;
    CK(cudaMemsetAsync(S.d_obs_count, 0, sizeof(u64), S.stream));
    // the captured step embeds the observable arguments: capture again
    if (S.gexec) {
        cudaGraphExecDestroy(S.gexec);
        cudaGraphDestroy(S.graph);
        S.gexec = nullptr;
        S.graph = nullptr;
    }
    CK(cudaStreamSynchronize(S.stream));
}

mgmc_status mgmc_sampler_set_observable(mgmc_sampler *s, int64_t nnz, const int64_t *idx, const double *val,
                                        int64_t capacity) {
    API_BEGIN
    Sampler &S = impl(s);
    if (nnz < 0) fail(MGMC_ERR_INVALID_ARGUMENT, "bad observable");
    const int64_t ptr[2] = {0, nnz};
    set_probes(S, nnz > 0 ? 1 : 0, ptr, idx, val, capacity);
    API_END
}

mgmc_status mgmc_sampler_set_probes(mgmc_sampler *s, int nprobe, const int64_t *ptr, const int64_t *idx,
                                    const double *val, int64_t capacity) {
    API_BEGIN
    Sampler &S = impl(s);
    set_probes(S, nprobe, ptr, idx, val, capacity);
    API_END
}

mgmc_status mgmc_sampler_read_observations(mgmc_sampler *s, double *out, int64_t capacity, int64_t *count) {
    API_BEGIN
    Sampler &S = impl(s);
    if (!count) fail(MGMC_ERR_INVALID_ARGUMENT, "null count");
    CK(cudaStreamSynchronize(S.stream));
    u64 c = 0;
    CK(cudaMemcpy(&c, S.d_obs_count, sizeof(c), cudaMemcpyDeviceToHost));
    i64 k = std::min<i64>((i64)c, S.obs_cap);
    const int np = std::max(S.nprobe, 1);
    k = std::min<i64>(k, capacity / np);
    if (k > 0 && out) CK(cudaMemcpy(out, S.d_obs, (size_t)k * np * sizeof(double), cudaMemcpyDeviceToHost));
    *count = (int64_t)c;
    CK(cudaMemset(S.d_obs_count, 0, sizeof(u64)));
    check_device_errors(S);
    API_END
}

mgmc_status mgmc_sampler_inject_noise(mgmc_sampler *s, const double *normals, int64_t count, int on_device) {
    API_BEGIN
    Sampler &S = impl(s);
    if (S.noise_mode != NOISE_INJECTED) fail(MGMC_ERR_INVALID_ARGUMENT, "sampler was not created with MGMC_NOISE_INJECTED");
    if (count < 0 || (count > 0 && !normals)) fail(MGMC_ERR_INVALID_ARGUMENT, "bad noise buffer");
    CK(cudaStreamSynchronize(S.stream));
    i64 keep = S.noise_len - S.noise_pos;
    if (keep + count > S.noise_cap) {
        i64 cap = std::max<i64>(keep + count, 2 * S.noise_cap);
        double *nb = dalloc<double>(cap);
        if (keep > 0) CK(cudaMemcpy(nb, S.d_noise + S.noise_pos, keep * sizeof(double), cudaMemcpyDeviceToDevice));
        if (S.d_noise) {
            auto it = std::find(S.owned.begin(), S.owned.end(), (void *)S.d_noise);
            if (it != S.owned.end()) S.owned.erase(it);
            cudaFree(S.d_noise);
        }
        S.owned.push_back(nb);
        S.d_noise = nb;
        S.noise_cap = cap;
    } else if (S.noise_pos > 0 && keep > 0) {
        CK(cudaMemcpy(S.d_noise, S.d_noise + S.noise_pos, keep * sizeof(double), cudaMemcpyDeviceToDevice));
    }
    S.noise_pos = 0;
    S.noise_len = keep;
    if (count > 0)
        CK(cudaMemcpy(S.d_noise + S.noise_len, normals, count * sizeof(double),
                      on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice));
    S.noise_len += count;
    API_END
}

mgmc_status mgmc_sampler_noise_per_step(mgmc_sampler *s, int64_t *count) {
    API_BEGIN
    Sampler &S = impl(s);
    if (!count) fail(MGMC_ERR_INVALID_ARGUMENT, "null count");
    *count = S.noise_per_step;
    API_END
}

mgmc_status mgmc_sampler_synchronize(mgmc_sampler *s) {
    API_BEGIN
    Sampler &S = impl(s);
    CK(cudaStreamSynchronize(S.stream));
    unsigned err = 0;
    CK(cudaMemcpy(&err, S.d_err, sizeof(err), cudaMemcpyDeviceToHost));
    if (err & ERR_TILE_TIMEOUT) fail(MGMC_ERR_CUDA, "a shared-memory tile copy did not complete in time");
    API_END
}

mgmc_status mgmc_sampler_stream(mgmc_sampler *s, void **cuda_stream) {
    API_BEGIN
    Sampler &S = impl(s);
    if (!cuda_stream) fail(MGMC_ERR_INVALID_ARGUMENT, "null argument");
    *cuda_stream = (void *)S.stream;
    API_END
}

mgmc_status mgmc_sampler_nlevel(mgmc_sampler *s, int *nlevel) {
    API_BEGIN
    Sampler &S = impl(s);
    if (!nlevel) fail(MGMC_ERR_INVALID_ARGUMENT, "null argument");
    *nlevel = (int)S.L.size();
    API_END
}

mgmc_status mgmc_sampler_level_size(mgmc_sampler *s, int level, int64_t *n) {
    API_BEGIN
    Sampler &S = impl(s);
    check_level(S, level, false);
    if (!n) fail(MGMC_ERR_INVALID_ARGUMENT, "null argument");
    *n = S.L[level].geo.n;
    API_END
}

mgmc_status mgmc_sampler_launches_per_step(mgmc_sampler *s, int64_t *count) {
    API_BEGIN
    Sampler &S = impl(s);
    if (!count) fail(MGMC_ERR_INVALID_ARGUMENT, "null argument");
    if (S.noise_mode == NOISE_PHILOX) ensure_graph(S);
    *count = S.step_launches;
    API_END
}

mgmc_status mgmc_level_stencil(mgmc_sampler *s, int level, double stencil[27]) {
    API_BEGIN
    Sampler &S = impl(s);
    check_level(S, level, false);
    if (!stencil) fail(MGMC_ERR_INVALID_ARGUMENT, "null argument");
    std::memcpy(stencil, S.L[level].st, 27 * sizeof(double));
    API_END
}

mgmc_status mgmc_level_apply(mgmc_sampler *s, int level, const double *x, double *y) {
    API_BEGIN
    Sampler &S = impl(s);
    check_level(S, level, false);
    if (!x || !y) fail(MGMC_ERR_INVALID_ARGUMENT, "null argument");
    S.ensure_scratch(level);
    Level &lv = S.L[level];
    put_vec(S, level, x, 0, lv.s1);
    if (S.fp32) {
        launch_apply_stencil<float>(S, lv, lv.s1, lv.s2);
        if (S.m > 0 && lv.Bptr) {
            launch_bt_plain<float>(S, lv, lv.s1);
            launch_add_Bq<float>(S, lv, lv.s2, lv.y, 1.0);
        }
    } else {
        launch_apply_stencil<double>(S, lv, lv.s1, lv.s2);
        if (S.m > 0 && lv.Bptr) {
            launch_bt_plain<double>(S, lv, lv.s1);
            launch_add_Bq<double>(S, lv, lv.s2, lv.y, 1.0);
        }
    }
    S.check_launch();
    get_vec(S, level, lv.s2, y, 0);
    API_END
}

mgmc_status mgmc_level_restrict(mgmc_sampler *s, int level, const double *x, double *xc) {
    API_BEGIN
    Sampler &S = impl(s);
    check_level(S, level, true);
    if (!x || !xc) fail(MGMC_ERR_INVALID_ARGUMENT, "null argument");
    S.ensure_scratch(level);
    S.ensure_scratch(level + 1);
    Level &lv = S.L[level], &lc = S.L[level + 1];
    put_vec(S, level, x, 0, lv.s1);
    if (S.fp32)
        launch_resid_restrict<float>(S, level, lv.s1, lv.s1, lc.s1, nullptr, true);
    else
        launch_resid_restrict<double>(S, level, lv.s1, lv.s1, lc.s1, nullptr, true);
    S.check_launch();
    get_vec(S, level + 1, lc.s1, xc, 0);
    API_END
}

mgmc_status mgmc_level_prolongate_add(mgmc_sampler *s, int level, double alpha, const double *xc, double *x) {
    API_BEGIN
    Sampler &S = impl(s);
    check_level(S, level, true);
    if (!x || !xc) fail(MGMC_ERR_INVALID_ARGUMENT, "null argument");
    S.ensure_scratch(level);
    S.ensure_scratch(level + 1);
    Level &lv = S.L[level], &lc = S.L[level + 1];
    put_vec(S, level + 1, xc, 0, lc.s1);
    put_vec(S, level, x, 0, lv.s1);
    S.prolong(level, alpha, lc.s1, lv.s1);
    S.check_launch();
    get_vec(S, level, lv.s1, x, 0);
    API_END
}

mgmc_status mgmc_level_sor(mgmc_sampler *s, int level, int direction, int with_noise, const double *f, double *x) {
    API_BEGIN
    Sampler &S = impl(s);
    check_level(S, level, false);
    if (!x || !f) fail(MGMC_ERR_INVALID_ARGUMENT, "null argument");
    if (direction != MGMC_FORWARD && direction != MGMC_BACKWARD) fail(MGMC_ERR_INVALID_ARGUMENT, "direction must be MGMC_FORWARD or MGMC_BACKWARD");
    Level &lv = S.L[level];
    S.ensure_scratch(level);
    put_vec(S, level, f, 0, lv.s1);
    put_vec(S, level, x, 0, lv.s2);
    i64 need = with_noise ? lv.geo.n + S.m : 0;
    if (with_noise && S.noise_mode == NOISE_INJECTED && S.noise_len - S.noise_pos < need)
        fail(MGMC_ERR_NOISE_EXHAUSTED, "injected noise exhausted");
    S.inv = 4095;
    S.noise_off = S.noise_pos;
    S.sor(level, direction == MGMC_FORWARD, with_noise != 0, lv.s2, lv.s1);
    S.check_launch();
    if (with_noise && S.noise_mode == NOISE_INJECTED) S.noise_pos += need;
    get_vec(S, level, lv.s2, x, 0);
    API_END
}

mgmc_status mgmc_level_sweep_device(mgmc_sampler *s, int level, int direction, int with_noise, int with_lowrank,
                                    int64_t nrepeat) {
    API_BEGIN
    Sampler &S = impl(s);
    check_level(S, level, false);
    if (direction != MGMC_FORWARD && direction != MGMC_BACKWARD) fail(MGMC_ERR_INVALID_ARGUMENT, "direction must be MGMC_FORWARD or MGMC_BACKWARD");
    if (with_noise && S.noise_mode != NOISE_PHILOX) fail(MGMC_ERR_UNSUPPORTED, "device sweeps draw Philox noise only");
    if (nrepeat < 0) fail(MGMC_ERR_INVALID_ARGUMENT, "nrepeat < 0");
    Level &lv = S.L[level];
    const int saved_m = S.m;
    for (int64_t r = 0; r < nrepeat; ++r) {
        S.inv = 4094;
        if (!with_lowrank) S.m = 0;
        S.sor(level, direction == MGMC_FORWARD, with_noise != 0, lv.x, lv.f);
        S.m = saved_m;
    }
    S.check_launch();
    API_END
}

mgmc_status mgmc_level_transfer_device(mgmc_sampler *s, int level, int which, int64_t nrepeat) {
    API_BEGIN
    Sampler &S = impl(s);
    check_level(S, level, true);
    if (which != 0 && which != 1) fail(MGMC_ERR_INVALID_ARGUMENT, "which must be 0 (residual-restriction) or 1 (prolongation)");
    if (nrepeat < 0) fail(MGMC_ERR_INVALID_ARGUMENT, "nrepeat < 0");
    Level &lv = S.L[level], &lc = S.L[level + 1];
    for (int64_t r = 0; r < nrepeat; ++r) {
        if (which == 0)
            S.resid_restrict(level);
        else
            S.prolong(level, S.P.coarse_scaling, lc.x, lv.x);
    }
    S.check_launch();
    API_END
}

}  // extern "C"

// ------------------------------------------------------------------- batch
// Chains that share a lattice geometry and a step structure advance
// through the batched kernels (k_*_batch in kernels.cuh): one launch per
// kernel of the step covers every chain of the group, instead of one launch
// per chain.  Eligible: FP32-mixed, Philox noise, multicolour order, SSOR
// smoother, coarse Cholesky sampler, constant stencils, 3D.  A chain stepped
// this way runs the same arithmetic on the same normals as when it is
// stepped alone (the kernels share their bodies with the one-chain ones).
// MGMC_BATCH_KERNELS=0 turns the grouping off (every chain then runs its own
// step graph inside the batch graph).
static bool batchable(const Sampler &S) {
    if (!S.fp32 || S.exact || S.noise_mode != NOISE_PHILOX || S.dim != 3) return false;
    if (S.P.ordering != MGMC_ORDER_MULTICOLOUR || S.P.smoother != MGMC_SMOOTHER_SSOR || !S.chol) return false;
    if (S.L.size() < 2 || !S.dLinv) return false;
    for (const Level &lv : S.L) {
        if (lv.var != 0) return false;
        if (lv.npt == 7 && !((lv.g.sy % 4) == 0 && (lv.g.sz % 4) == 0)) return false;
    }
    return true;
}

// chains with equal keys step through the same launches
static std::vector<long long> batch_key(const Sampler &S) {
    std::vector<long long> k = {S.dim, (long long)S.L.size(), S.P.npresmooth, S.P.npostsmooth, S.P.cycle, S.chol_ld,
                                (long long)S.chol_smem};
    long long cs;
    std::memcpy(&cs, &S.P.coarse_scaling, sizeof(cs));
    k.push_back(cs);
    for (const Level &lv : S.L) {
        for (long long v : {(long long)lv.g.N0, (long long)lv.g.N1, (long long)lv.g.N2, lv.g.sy, lv.g.sz,
                            (long long)lv.npt, (long long)lv.ncol})
            k.push_back(v);
    }
    return k;
}

struct BatchGroup {
    std::vector<Sampler *> ch;
    int G = 0, nlev = 0, max_m = 0, max_probe = 1;
    std::vector<BatchLevelArg *> la;          // per level: G entries
    BatchChainArg *ca = nullptr;
    std::vector<std::array<BatchLowRank *, 2>> lr;  // per level and sweep direction
    std::vector<BatchLowRank *> lr_res;       // per level: the residual's y = B^T x
    std::vector<BtJob *> bt_jobs;             // per level
    std::vector<int> n_bt;
    std::vector<std::array<RowJob *, 2>> sc_jobs;
    std::vector<std::array<int, 2>> n_sc;
    std::vector<BatchAddBq *> bq;             // per level: rows of the next level's B
    std::vector<RowJob *> bq_jobs;
    std::vector<int> n_bq;
    unsigned inv = 0;
    std::vector<void *> owned;
    ~BatchGroup() {
        for (void *p : owned) cudaFree(p);
    }
    template <typename P_>
    P_ *put(const std::vector<P_> &v, cudaStream_t st) {
        if (v.empty()) return nullptr;
        P_ *p = dupload(v, st);
        owned.push_back(p);
        return p;
    }
    void build(cudaStream_t st);
    void record(cudaStream_t st);
    void sor(int lev, bool forward, cudaStream_t st);
    void sample(int lev, cudaStream_t st);
};

// row ranges of `rows` rows per chain in jobs of at most 1024 rows
static void row_jobs(std::vector<RowJob> &jobs, int chain, i64 rows) {
    for (i64 r = 0; r < rows; r += 1024) jobs.push_back(RowJob{chain, r, std::min(rows, r + 1024)});
}

void BatchGroup::build(cudaStream_t st) {
    G = (int)ch.size();
    const Sampler &S0 = *ch[0];
    nlev = (int)S0.L.size();
    la.resize(nlev);
    lr.resize(nlev);
    lr_res.resize(nlev);
    bt_jobs.resize(nlev);
    n_bt.assign(nlev, 0);
    sc_jobs.resize(nlev);
    n_sc.resize(nlev);
    bq.resize(nlev);
    bq_jobs.resize(nlev);
    n_bq.assign(nlev, 0);
    for (Sampler *S : ch) {
        max_m = std::max(max_m, S->m);
        max_probe = std::max(max_probe, S->nprobe);
    }
    for (int lev = 0; lev < nlev; ++lev) {
        std::vector<BatchLevelArg> a(G);
        std::vector<BatchLowRank> l0(G), l1(G), lres(G);
        std::vector<BtJob> jobs;
        std::vector<RowJob> sj0, sj1, qj;
        std::vector<BatchAddBq> q(G);
        for (int c = 0; c < G; ++c) {
            Sampler &S = *ch[c];
            Level &lv = S.L[lev];
            BatchLevelArg &A = a[c];
            A.x = (float *)lv.x;
            A.f = (float *)lv.f;
            A.fsplit = lev == 0 ? S.fsplit : nullptr;
            A.fhalf = S.fhalf;
            A.xc = lev + 1 < nlev ? (float *)S.L[lev + 1].x : nullptr;
            A.fc = lev + 1 < nlev ? (float *)S.L[lev + 1].f : nullptr;
            A.s = stencil_arg<float>(lv, S.P.omega);
            if (S.m == 0) continue;
            for (int dir = 0; dir < 2; ++dir) {
                BatchLowRank &b = dir == 0 ? l0[c] : l1[c];
                LowRankArg &r = b.lr;
                r.m = S.m;
                r.Bptr = lv.Bptr;
                r.Bidx = lv.Bidx;
                r.Bval = lv.Bval;
                r.Bvalf = lv.Bvalf;
                r.zf = lv.zf;
                r.SinvT = lv.SinvT[dir];
                r.sigma_sqrt = S.d_sigma_sqrt;
                r.SinvT_ff = lv.SinvT_ff[dir];
                r.sigma_sqrt_ff = S.d_sigma_sqrt_ff;
                r.y = lv.y;
                r.z = lv.z;
                r.part = lv.part;
                r.counter = lv.counter;
                const CorrRows &C = lv.C[dir];
                b.C = C;
                row_jobs(dir == 0 ? sj0 : sj1, c, C.n1 + C.nm);
            }
            LowRankArg &r = lres[c].lr;  // launch_bt_plain's arguments
            r.m = S.m;
            r.Bptr = lv.Bptr;
            r.Bidx = lv.Bidx;
            r.Bval = lv.Bval;
            r.Bvalf = lv.Bvalf;
            r.y = lv.y;
            r.part = lv.part;
            r.counter = lv.counter;
            for (int j = 0; j < S.m; ++j)
                for (int p = 0; p < lv.bt_split; ++p) jobs.push_back(BtJob{c, j, p, lv.bt_split});
            if (lev + 1 < nlev) {
                const Level &lc = S.L[lev + 1];
                const RowCsr &B = lc.Br;
                q[c] = BatchAddBq{B.nrows, B.rows, B.ptr, B.col, (const double *)B.val, lv.y, S.d_sigma_inv,
                                  (float *)lc.f};
                row_jobs(qj, c, B.nrows);
            }
        }
        la[lev] = put(a, st);
        lr[lev] = {put(l0, st), put(l1, st)};
        lr_res[lev] = put(lres, st);
        bt_jobs[lev] = put(jobs, st);
        n_bt[lev] = (int)jobs.size();
        sc_jobs[lev] = {put(sj0, st), put(sj1, st)};
        n_sc[lev] = {(int)sj0.size(), (int)sj1.size()};
        bq[lev] = put(q, st);
        bq_jobs[lev] = put(qj, st);
        n_bq[lev] = (int)qj.size();
    }
    std::vector<BatchChainArg> c(G);
    for (int k = 0; k < G; ++k) {
        Sampler &S = *ch[k];
        BatchChainArg &A = c[k];
        A.seed = S.P.seed;
        A.d_step = S.d_step;
        A.Linv = (const float *)S.dLinv;
        A.LinvT = (const float *)S.dLinvT;
        A.gv = (float *)S.dgv;
        A.nprobe = S.nprobe;
        A.bptr = S.d_bptr;
        A.bidx = S.d_bidx;
        A.bval = S.d_bval;
        A.obs = S.d_obs;
        A.capacity = S.obs_cap;
        A.obs_count = S.d_obs_count;
        A.err = S.d_err;
        A.done = S.d_done;
    }
    ca = put(c, st);
    CK(cudaStreamSynchronize(st));
}

template <typename Kern>
static void batch_launch_check(Kern) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) fail(MGMC_ERR_CUDA, std::string("batched kernel launch: ") + cudaGetErrorString(e));
}

// Sampler::sor for the whole group: one sweep, its low-rank correction
void BatchGroup::sor(int lev, bool forward, cudaStream_t st) {
    const Sampler &S0 = *ch[0];
    const Level &lv = S0.L[lev];
    Grid3 g = lv.g;
    g.pdl = 0;
    if (lv.npt == 7) {
        const int ngrp = (g.N0 + 8) / 8;
        const dim3 blk = level_block(lv, ngrp);
        const dim3 grid((ngrp + blk.x - 1) / blk.x, (g.N1 + blk.y - 1) / blk.y, g.N2 * G);
        const bool v8 = (g.sy % 8) == 0 && (g.sz % 8) == 0;
        bool fs = v8 && lev == 0;
        for (Sampler *S : ch) fs = fs && S->fsplit;
        for (int pass = 0; pass < 2; ++pass) {
            const int colour = forward ? pass : 1 - pass;
            if (fs)
                k_sweep_rb_vec_batch<NOISE_PHILOX, true, true><<<grid, blk, 0, st>>>(la[lev], ca, g, colour, pass, inv,
                                                                                    (unsigned)lev);
            else if (v8)
                k_sweep_rb_vec_batch<NOISE_PHILOX, true, false><<<grid, blk, 0, st>>>(la[lev], ca, g, colour, pass,
                                                                                     inv, (unsigned)lev);
            else
                k_sweep_rb_vec_batch<NOISE_PHILOX, false, false><<<grid, blk, 0, st>>>(la[lev], ca, g, colour, pass,
                                                                                      inv, (unsigned)lev);
            batch_launch_check(0);
        }
    } else {
        for (int cc = 0; cc < lv.ncol; ++cc) {
            const int colour = forward ? cc : lv.ncol - 1 - cc;
            const int pa = colour & 1, pb = (colour >> 1) & 1, pc = (colour >> 2) & 1;
            const int na = (g.N0 - pa + 1) / 2, nb = (g.N1 - pb + 1) / 2, nc = (g.N2 - pc + 1) / 2;
            if (na <= 0 || nb <= 0 || nc <= 0) continue;
            const dim3 blk = level_block(lv, na);
            const dim3 grid((na + blk.x - 1) / blk.x, (nb + blk.y - 1) / blk.y, nc * G);
            k_sweep_c27_batch<NOISE_PHILOX><<<grid, blk, 0, st>>>(la[lev], ca, g, colour, nc, inv, (unsigned)lev);
            batch_launch_check(0);
        }
    }
    if (n_bt[lev] > 0) {
        const int dir = forward ? 0 : 1;
        k_bt_solve_batch<NOISE_PHILOX, true><<<n_bt[lev], 256, solve_smem(max_m), st>>>(la[lev], lr[lev][dir], ca,
                                                                                       bt_jobs[lev], inv, (unsigned)lev);
        batch_launch_check(0);
        if (n_sc[lev][dir] > 0) {
            k_lr_scatter_batch<<<n_sc[lev][dir], 256, 0, st>>>(la[lev], lr[lev][dir], sc_jobs[lev][dir]);
            batch_launch_check(0);
        }
    }
    inv++;
}

// Sampler::sample for the whole group (multigridmc_sampler.cc:109-136)
void BatchGroup::sample(int lev, cudaStream_t st) {
    const Sampler &S0 = *ch[0];
    if (lev == nlev - 1) {
        const Level &lv = S0.L[lev];
        Grid3 g = lv.g;
        g.pdl = 0;
        const unsigned blocks = (unsigned)((lv.geo.n + 7) / 8);
        k_chol_lower_batch<NOISE_PHILOX><<<dim3(blocks, G), 256, S0.chol_smem, st>>>(la[lev], ca, g, S0.chol_ld, inv,
                                                                                     (unsigned)lev);
        batch_launch_check(0);
        k_chol_upper_batch<<<dim3(blocks, G), 256, S0.chol_smem, st>>>(la[lev], ca, g, S0.chol_ld);
        batch_launch_check(0);
        inv++;
        return;
    }
    const Level &lv = S0.L[lev], &lc = S0.L[lev + 1];
    Grid3 gf = lv.g, gc = lc.g;
    gf.pdl = gc.pdl = 0;
    const int cyc = lev > 0 ? S0.P.cycle : 1;
    for (int j = 0; j < cyc; ++j) {
        for (int k = 0; k < S0.P.npresmooth; ++k) {
            sor(lev, true, st);
            sor(lev, false, st);
        }
        // residual-restriction (also zeroes the coarse state), then the
        // low-rank term of the residual
        const int tz = (gc.N2 + RR_TZ - 1) / RR_TZ;
        const dim3 rgrid((gc.N0 + RR_TX - 1) / RR_TX, (gc.N1 + RR_TY - 1) / RR_TY, tz * G);
        if (lv.npt == 7)
            k_resid_restrict_batch<7><<<rgrid, RR_THREADS, rr_smem_bytes<float>(), st>>>(la[lev], gf, gc, tz);
        else
            k_resid_restrict_batch<27><<<rgrid, RR_THREADS, rr_smem_bytes<float>(), st>>>(la[lev], gf, gc, tz);
        batch_launch_check(0);
        if (n_bt[lev] > 0) {
            k_bt_solve_batch<NOISE_NONE, false><<<n_bt[lev], 256, solve_smem(max_m), st>>>(la[lev], lr_res[lev], ca,
                                                                                          bt_jobs[lev], 0u, 0u);
            batch_launch_check(0);
            if (n_bq[lev] > 0) {
                k_add_Bq_batch<<<n_bq[lev], 256, 0, st>>>(bq[lev], bq_jobs[lev]);
                batch_launch_check(0);
            }
        }
        sample(lev + 1, st);
        const dim3 pgrid((gc.N0 + 1 + 127) / 128, gc.N1 + 1, (gc.N2 + 1) * G);
        k_prolong_batch<<<pgrid, 128, 0, st>>>(la[lev], gf, gc, (float)S0.P.coarse_scaling, 3, gc.N2 + 1);
        batch_launch_check(0);
        for (int k = 0; k < S0.P.npostsmooth; ++k) {
            sor(lev, true, st);
            sor(lev, false, st);
        }
    }
}

void BatchGroup::record(cudaStream_t st) {
    inv = 0;
    sample(0, st);
    k_step_end_batch<<<dim3(max_probe, G), 256, 0, st>>>(la[0], ca);
    batch_launch_check(0);
}

extern "C" {

struct mgmc_batch {
    std::vector<Sampler *> chains;
    std::vector<std::unique_ptr<BatchGroup>> groups;
    std::vector<cudaGraph_t> group_graphs;
    cudaStream_t stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    int device = 0;
};

mgmc_status mgmc_batch_create(int nchain, mgmc_sampler *const *samplers, mgmc_batch **out) {
    mgmc_batch *B = nullptr;
    API_BEGIN
    if (nchain < 1 || !samplers || !out) fail(MGMC_ERR_INVALID_ARGUMENT, "need at least one sampler");
    *out = nullptr;
    B = new mgmc_batch();
    for (int i = 0; i < nchain; ++i) {
        Sampler &S = impl(samplers[i]);
        if (S.noise_mode != NOISE_PHILOX) fail(MGMC_ERR_UNSUPPORTED, "batched chains draw Philox noise");
        if (i == 0) B->device = S.P.device;
        if (S.P.device != B->device) fail(MGMC_ERR_INVALID_ARGUMENT, "batched chains must share one device");
        if (std::find(B->chains.begin(), B->chains.end(), &S) != B->chains.end())
            fail(MGMC_ERR_INVALID_ARGUMENT, "a sampler appears twice in the batch");
        B->chains.push_back(&S);
    }
    CK(cudaSetDevice(B->device));
    CK(cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking));
    CK(cudaGraphCreate(&B->graph, 0));
    // groups of chains that step through the batched kernels
    std::vector<Sampler *> solo;
    {
        bool group = true;
        if (const char *e = std::getenv("MGMC_BATCH_KERNELS"))
            if (e[0] == '0') group = false;
        std::map<std::vector<long long>, std::vector<Sampler *>> keyed;
        for (Sampler *S : B->chains) {
            if (group && batchable(*S))
                keyed[batch_key(*S)].push_back(S);
            else
                solo.push_back(S);
        }
        for (auto &kv : keyed) {
            std::vector<Sampler *> &v = kv.second;
            if (v.size() < 2) {
                solo.insert(solo.end(), v.begin(), v.end());
                continue;
            }
            // grid.z carries chains x planes: at most 65535
            const int zmax = std::max(1, 65535 / std::max(1, v[0]->L[0].g.N2 + 1));
            for (size_t a = 0; a < v.size(); a += (size_t)zmax) {
                auto grp = std::make_unique<BatchGroup>();
                grp->ch.assign(v.begin() + a, v.begin() + std::min(v.size(), a + (size_t)zmax));
                for (Sampler *S : grp->ch) CK(cudaStreamSynchronize(S->stream));
                grp->build(B->stream);
                cudaGraph_t gg = nullptr;
                CK(cudaStreamBeginCapture(B->stream, cudaStreamCaptureModeThreadLocal));
                try {
                    grp->record(B->stream);
                } catch (...) {
                    cudaStreamEndCapture(B->stream, &gg);
                    if (gg) cudaGraphDestroy(gg);
                    throw;
                }
                CK(cudaStreamEndCapture(B->stream, &gg));
                B->group_graphs.push_back(gg);
                cudaGraphNode_t node;
                CK(cudaGraphAddChildGraphNode(&node, B->graph, nullptr, 0, gg));
                B->groups.push_back(std::move(grp));
            }
        }
    }
    for (Sampler *S : solo) {
        CK(cudaStreamSynchronize(S->stream));
        // a chain's step graph becomes a child graph: captured with plain
        // (non-programmatic) dependencies
        if (S->pdl) {
            S->pdl = false;
            if (S->gexec) cudaGraphExecDestroy(S->gexec);
            if (S->graph) cudaGraphDestroy(S->graph);
            S->gexec = nullptr;
            S->graph = nullptr;
        }
        ensure_graph(*S);
        cudaGraphNode_t node;
        CK(cudaGraphAddChildGraphNode(&node, B->graph, nullptr, 0, S->graph));
    }
    CK(cudaGraphInstantiate(&B->gexec, B->graph, 0));
    *out = B;
    B = nullptr;
    }
    catch (const Error &e) {
        if (B) {
            if (B->gexec) cudaGraphExecDestroy(B->gexec);
            if (B->graph) cudaGraphDestroy(B->graph);
            for (cudaGraph_t gg : B->group_graphs) cudaGraphDestroy(gg);
            if (B->stream) cudaStreamDestroy(B->stream);
            delete B;
        }
        g_err = e.msg;
        return e.st;
    }
    return MGMC_OK;
}

mgmc_status mgmc_batch_step(mgmc_batch *b, int64_t nsteps) {
    API_BEGIN
    if (!b || nsteps < 0) fail(MGMC_ERR_INVALID_ARGUMENT, "bad arguments");
    CK(cudaSetDevice(b->device));
    for (int64_t k = 0; k < nsteps; ++k) CK(cudaGraphLaunch(b->gexec, b->stream));
    API_END
}

mgmc_status mgmc_batch_info(mgmc_batch *b, int *ngroups, int *ngrouped) {
    API_BEGIN
    if (!b || !ngroups || !ngrouped) fail(MGMC_ERR_INVALID_ARGUMENT, "null argument");
    *ngroups = (int)b->groups.size();
    int n = 0;
    for (const auto &g : b->groups) n += g->G;
    *ngrouped = n;
    API_END
}

mgmc_status mgmc_batch_synchronize(mgmc_batch *b) {
    API_BEGIN
    if (!b) fail(MGMC_ERR_INVALID_ARGUMENT, "null batch");
    CK(cudaSetDevice(b->device));
    CK(cudaStreamSynchronize(b->stream));
    API_END
}

mgmc_status mgmc_batch_stream(mgmc_batch *b, void **cuda_stream) {
    API_BEGIN
    if (!b || !cuda_stream) fail(MGMC_ERR_INVALID_ARGUMENT, "null argument");
    *cuda_stream = (void *)b->stream;
    API_END
}

mgmc_status mgmc_batch_destroy(mgmc_batch *b) {
    API_BEGIN
    if (!b) return MGMC_OK;
    cudaSetDevice(b->device);
    cudaStreamSynchronize(b->stream);
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (cudaGraph_t gg : b->group_graphs) cudaGraphDestroy(gg);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    API_END
}

}  // extern "C"

// --------------------------------------------- low-rank Cholesky sampler
// LowRankCholeskySampler (cholesky_sampler.cc:41-129) on the GPU.  The
// factors come from lowrank_cholesky_factors (setup.cc): D_k = L_kk^{-1}
// and O_k = L_{k,k-1} of the block factor of A_0, and Q, QW, QWT.  A sample
// is xi ~ N(0, 1) (n normals: Philox or injected), g = L^{-1} f block by
// block (g_k = D_k (f_k - O_k g_{k-1})), g += QW (Q^T g), xi += g,
// xi += QWT (Q^T xi), and x = L^{-T} xi block by block from the last
// (x_k = D_k^T (xi_k - O_{k+1}^T x_{k+1})) -- dense FP64 matrix-vector
// products (k_dgemv_rows, k_dgemv_cols_partial / _finish) captured into
// one CUDA graph.
struct LrChol {
    int device = 0, nb = 0, m = 0, noise = NOISE_PHILOX;
    i64 n = 0, p = 0;
    u64 seed = 0;
    cudaStream_t stream = nullptr;
    double *D = nullptr, *O = nullptr, *Q = nullptr, *QW = nullptr, *QWT = nullptr;
    double *f = nullptr, *x = nullptr, *xi = nullptr, *g = nullptr, *t = nullptr, *mt = nullptr, *part = nullptr;
    double *noise_buf = nullptr;
    i64 noise_cap = 0, noise_len = 0, noise_pos = 0;
    u64 *d_step = nullptr;
    bool rhs_set = false;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    std::vector<void *> owned;
    static constexpr int RCH = 64;  // rows per partial sum of a transposed product
    ~LrChol() {
        if (gexec) cudaGraphExecDestroy(gexec);
        if (graph) cudaGraphDestroy(graph);
        for (void *q : owned) cudaFree(q);
        if (stream) cudaStreamDestroy(stream);
    }
    template <typename P_>
    P_ *alloc(size_t count) {
        P_ *q = dalloc<P_>(count);
        owned.push_back(q);
        return q;
    }
    template <typename P_>
    P_ *upload(const std::vector<P_> &v) {
        P_ *q = dupload(v, stream);
        owned.push_back(q);
        return q;
    }
    // y = yadd + alpha A v, A rows x cols row-major
    void rows(const double *A, i64 r, i64 c, i64 lda, const double *v, const double *yadd, double alpha, double *y,
              bool lower) {
        const unsigned blocks = (unsigned)((r * 32 + 255) / 256);
        if (lower)
            k_dgemv_rows<true><<<blocks, 256, 0, stream>>>(A, r, c, lda, v, yadd, alpha, y);
        else
            k_dgemv_rows<false><<<blocks, 256, 0, stream>>>(A, r, c, lda, v, yadd, alpha, y);
    }
    // y = yadd + alpha A^T v
    void cols(const double *A, i64 r, i64 c, i64 lda, const double *v, const double *yadd, double alpha, double *y,
              bool lower) {
        const int nch = (int)((r + RCH - 1) / RCH);
        const int bs = c >= 256 ? 256 : (int)((c + 31) / 32 * 32);
        const dim3 grid((unsigned)((c + bs - 1) / bs), (unsigned)nch);
        if (lower)
            k_dgemv_cols_partial<true><<<grid, bs, 0, stream>>>(A, r, c, lda, v, RCH, part);
        else
            k_dgemv_cols_partial<false><<<grid, bs, 0, stream>>>(A, r, c, lda, v, RCH, part);
        k_dgemv_cols_finish<<<(unsigned)((c + 255) / 256), 256, 0, stream>>>(part, nch, c, yadd, alpha, y);
    }
    void sample() {
        NoiseArgs nz{};
        nz.seed = seed;
        nz.d_step = d_step;
        nz.invocation = 0;
        nz.level = 0;
        if (noise == NOISE_INJECTED) {
            nz.buf = noise_buf + noise_pos;
            k_cholesky_normals<NOISE_INJECTED><<<nblk(n, 256), 256, 0, stream>>>(nz, n, xi);
        } else {
            k_cholesky_normals<NOISE_PHILOX><<<nblk(n, 256), 256, 0, stream>>>(nz, n, xi);
        }
        // g = L^{-1} f
        for (int k = 0; k < nb; ++k) {
            const double *Dk = D + (size_t)k * p * p;
            const double *v = f + k * p;
            if (k > 0) {
                rows(O + (size_t)k * p * p, p, p, p, g + (k - 1) * p, f + k * p, -1.0, t, false);
                v = t;
            }
            rows(Dk, p, p, p, v, nullptr, 1.0, g + k * p, true);
        }
        if (m > 0) {  // g += QW (Q^T g)
            cols(Q, n, m, m, g, nullptr, 1.0, mt, false);
            rows(QW, n, m, m, mt, g, 1.0, g, false);
        }
        k_axpy<double><<<nblk(n, 256), 256, 0, stream>>>(xi, g, 1.0, n);
        if (m > 0) {  // xi += QWT (Q^T xi)
            cols(Q, n, m, m, xi, nullptr, 1.0, mt, false);
            rows(QWT, n, m, m, mt, xi, 1.0, xi, false);
        }
        // x = L^{-T} xi
        for (int k = nb - 1; k >= 0; --k) {
            const double *v = xi + k * p;
            if (k + 1 < nb) {
                cols(O + (size_t)(k + 1) * p * p, p, p, p, x + (k + 1) * p, xi + k * p, -1.0, t, false);
                v = t;
            }
            cols(D + (size_t)k * p * p, p, p, p, v, nullptr, 1.0, x + k * p, true);
        }
        k_counter_advance<<<1, 1, 0, stream>>>(d_step);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) fail(MGMC_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    }
    void run() {
        if (noise == NOISE_INJECTED) {
            if (noise_len - noise_pos < n)
                fail(MGMC_ERR_NOISE_EXHAUSTED, "injected noise exhausted: " + std::to_string(noise_len - noise_pos) +
                                                   " queued, " + std::to_string(n) + " needed per sample");
            sample();
            noise_pos += n;
            return;
        }
        if (!gexec) {
            CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
            try {
                sample();
            } catch (...) {
                cudaGraph_t gg = nullptr;
                cudaStreamEndCapture(stream, &gg);
                if (gg) cudaGraphDestroy(gg);
                throw;
            }
            CK(cudaStreamEndCapture(stream, &graph));
            CK(cudaGraphInstantiate(&gexec, graph, 0));
        }
        CK(cudaGraphLaunch(gexec, stream));
    }
};

struct mgmc_lrchol {
    std::unique_ptr<LrChol> impl;
};

static LrChol &lrimpl(mgmc_lrchol *s) {
    if (!s || !s->impl) fail(MGMC_ERR_INVALID_ARGUMENT, "null sampler");
    CK(cudaSetDevice(s->impl->device));
    return *s->impl;
}

// n doubles host or device -> device buffer dst of the sampler
static void lr_put(LrChol &S, const double *src, int on_device, double *dst) {
    CK(cudaMemcpyAsync(dst, src, (size_t)S.n * sizeof(double), on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                       S.stream));
}

extern "C" {

mgmc_status mgmc_lrchol_create(const mgmc_operator_desc *op, int noise, uint64_t seed, int device, mgmc_lrchol **out) {
    mgmc_lrchol *h = nullptr;
    API_BEGIN
    if (!op || !out) fail(MGMC_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    if (op->dim < 1 || op->dim > 3) fail(MGMC_ERR_INVALID_ARGUMENT, "dim must be 1, 2 or 3");
    if (op->centre || op->field) fail(MGMC_ERR_UNSUPPORTED, "the low-rank Cholesky sampler takes a constant stencil");
    if (noise != MGMC_NOISE_PHILOX && noise != MGMC_NOISE_INJECTED) fail(MGMC_ERR_INVALID_ARGUMENT, "invalid noise source");
    if (op->m < 0 || (op->m > 0 && (!op->B_colptr || !op->B_rowidx || !op->B_val || !op->Sigma)))
        fail(MGMC_ERR_INVALID_ARGUMENT, "low-rank term needs B and Sigma");
    const int cells[3] = {op->nx, op->dim > 1 ? op->ny : 2, op->dim > 2 ? op->nz : 2};
    for (int d = 0; d < op->dim; ++d)
        if (cells[d] < 2) fail(MGMC_ERR_LATTICE, "every active direction needs at least 2 cells");
    Geometry geo(op->dim, cells[0], cells[1], cells[2]);
    SparseCols B;
    B.m = op->m;
    std::vector<double> Sigma;
    if (op->m > 0) {
        B.ptr.assign(op->B_colptr, op->B_colptr + op->m + 1);
        for (int j = 0; j < op->m; ++j)
            for (i64 e = op->B_colptr[j]; e < op->B_colptr[j + 1]; ++e)
                if (op->B_rowidx[e] < 0 || op->B_rowidx[e] >= geo.n) fail(MGMC_ERR_INVALID_ARGUMENT, "B row index out of range");
        B.row.assign(op->B_rowidx, op->B_rowidx + op->B_colptr[op->m]);
        B.val.assign(op->B_val, op->B_val + op->B_colptr[op->m]);
        Sigma.assign(op->Sigma, op->Sigma + op->m);
    }
    LowRankCholeskyFactors F;
    if (!lowrank_cholesky_factors(geo, op->stencil, B, Sigma, F))
        fail(MGMC_ERR_NOT_SPD, "the prior or the low-rank system is not positive definite");
    h = new mgmc_lrchol();
    h->impl.reset(new LrChol());
    LrChol &S = *h->impl;
    S.device = device;
    CK(cudaSetDevice(device));
    CK(cudaStreamCreateWithFlags(&S.stream, cudaStreamNonBlocking));
    S.n = geo.n;
    S.nb = F.nb;
    S.p = F.p;
    S.m = F.m;
    S.noise = noise == MGMC_NOISE_INJECTED ? NOISE_INJECTED : NOISE_PHILOX;
    S.seed = seed;
    S.D = S.upload(F.D);
    S.O = S.upload(F.O);
    if (S.m > 0) {
        S.Q = S.upload(F.Q);
        S.QW = S.upload(F.QW);
        S.QWT = S.upload(F.QWT);
    }
    S.f = S.alloc<double>(S.n);
    S.x = S.alloc<double>(S.n);
    S.xi = S.alloc<double>(S.n);
    S.g = S.alloc<double>(S.n);
    S.t = S.alloc<double>(S.p);
    S.mt = S.alloc<double>(std::max(S.m, 1));
    const i64 maxr = std::max<i64>(S.n, S.p), maxc = std::max<i64>(S.p, S.m);
    S.part = S.alloc<double>((size_t)((maxr + LrChol::RCH - 1) / LrChol::RCH) * maxc);
    S.d_step = S.alloc<u64>(1);
    CK(cudaMemsetAsync(S.d_step, 0, sizeof(u64), S.stream));
    for (double *q : {S.f, S.x, S.xi, S.g}) CK(cudaMemsetAsync(q, 0, (size_t)S.n * sizeof(double), S.stream));
    CK(cudaStreamSynchronize(S.stream));
    *out = h;
    h = nullptr;
    }
    catch (const Error &e) {
        delete h;
        g_err = e.msg;
        return e.st;
    }
    catch (const std::bad_alloc &) {
        delete h;
        g_err = "host allocation failed";
        return MGMC_ERR_OUT_OF_MEMORY;
    }
    return MGMC_OK;
}

mgmc_status mgmc_lrchol_destroy(mgmc_lrchol *s) {
    API_BEGIN
    if (!s) return MGMC_OK;
    if (s->impl) {
        cudaSetDevice(s->impl->device);
        cudaStreamSynchronize(s->impl->stream);
    }
    delete s;
    API_END
}

mgmc_status mgmc_lrchol_fix_rhs(mgmc_lrchol *s, const double *f, int on_device) {
    API_BEGIN
    LrChol &S = lrimpl(s);
    if (!f) fail(MGMC_ERR_INVALID_ARGUMENT, "null f");
    lr_put(S, f, on_device, S.f);
    CK(cudaStreamSynchronize(S.stream));
    S.rhs_set = true;
    API_END
}

mgmc_status mgmc_lrchol_apply(mgmc_lrchol *s, const double *f, double *x, int on_device) {
    API_BEGIN
    LrChol &S = lrimpl(s);
    if (!x) fail(MGMC_ERR_INVALID_ARGUMENT, "null x");
    if (f) {
        lr_put(S, f, on_device, S.f);
        S.rhs_set = true;
    } else if (!S.rhs_set) {
        fail(MGMC_ERR_INVALID_ARGUMENT, "f is NULL but no right hand side has been set");
    }
    S.run();
    CK(cudaMemcpyAsync(x, S.x, (size_t)S.n * sizeof(double), on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                       S.stream));
    CK(cudaStreamSynchronize(S.stream));
    API_END
}

mgmc_status mgmc_lrchol_inject_noise(mgmc_lrchol *s, const double *normals, int64_t count) {
    API_BEGIN
    LrChol &S = lrimpl(s);
    if (S.noise != NOISE_INJECTED) fail(MGMC_ERR_INVALID_ARGUMENT, "the sampler draws Philox noise");
    if (count < 0 || (count > 0 && !normals)) fail(MGMC_ERR_INVALID_ARGUMENT, "bad noise buffer");
    // keep the unread tail, append the new normals
    const i64 tail = S.noise_len - S.noise_pos;
    std::vector<double> keep((size_t)tail);
    if (tail > 0) CK(cudaMemcpy(keep.data(), S.noise_buf + S.noise_pos, (size_t)tail * sizeof(double), cudaMemcpyDeviceToHost));
    const i64 need = tail + count;
    if (need > S.noise_cap) {
        if (S.noise_buf) {
            cudaFree(S.noise_buf);
            S.owned.erase(std::find(S.owned.begin(), S.owned.end(), (void *)S.noise_buf));
        }
        S.noise_buf = S.alloc<double>((size_t)need);
        S.noise_cap = need;
    }
    if (tail > 0) CK(cudaMemcpy(S.noise_buf, keep.data(), (size_t)tail * sizeof(double), cudaMemcpyHostToDevice));
    if (count > 0) CK(cudaMemcpy(S.noise_buf + tail, normals, (size_t)count * sizeof(double), cudaMemcpyHostToDevice));
    S.noise_pos = 0;
    S.noise_len = need;
    API_END
}

mgmc_status mgmc_lrchol_stream(mgmc_lrchol *s, void **cuda_stream) {
    API_BEGIN
    LrChol &S = lrimpl(s);
    if (!cuda_stream) fail(MGMC_ERR_INVALID_ARGUMENT, "null argument");
    *cuda_stream = (void *)S.stream;
    API_END
}

}  // extern "C"

mgmc_status mgmc_sampler_precondition(mgmc_sampler *s, const double *b, double *x, int on_device) {
    API_BEGIN
    Sampler &S = impl(s);
    if (!b || !x) fail(MGMC_ERR_INVALID_ARGUMENT, "null argument");
    CK(cudaStreamSynchronize(S.stream));
    S.ensure_solver();
    Level &l0 = S.L[0];
    BorrowLevel0 borrow(S);
    put_vec(S, 0, b, on_device, l0.f);
    S.refresh_fsplit();
    CK(cudaMemsetAsync(l0.x, 0, (size_t)l0.geo.nalloc * S.tsize(), S.stream));
    CK(cudaGraphLaunch(S.pexec, S.stream));
    get_vec(S, 0, l0.x, x, on_device);
    CK(cudaStreamSynchronize(S.stream));
    check_device_errors(S);
    API_END
}

// LoopSolver::apply on the solver's FP64 vectors: b in sv_b, x from zero
// (loop_solver.cc:17) into sv_x; returns the iteration at which the test
// passed (maxiter when it never did), the last residual norm (-1 when
// maxiter = 0) and whether it passed.
static int loop_solve(Sampler &S, double rtol, double atol, int maxiter, double *rnorm, bool *converged) {
    Level &l0 = S.L[0];
    CK(cudaMemsetAsync(S.sv_x, 0, (size_t)l0.geo.nalloc * sizeof(double), S.stream));
    int k = 0;
    double r0 = 0.0, rn = -1.0;
    bool conv = false;
    for (k = 0; k < maxiter; ++k) {
        CK(cudaGraphLaunch(S.rexec, S.stream));
        double r2 = 0.0;
        CK(cudaMemcpyAsync(&r2, S.sv_norm, sizeof(double), cudaMemcpyDeviceToHost, S.stream));
        CK(cudaStreamSynchronize(S.stream));
        rn = std::sqrt(r2);
        if (!std::isfinite(rn)) fail(MGMC_ERR_NONFINITE, "non-finite residual in the solver");
        if (k == 0) r0 = rn;  // |A 0 - b| = |b| (loop_solver.cc:11)
        if (rn / r0 < rtol && rn < atol) {
            conv = true;
            break;
        }
        CK(cudaGraphLaunch(S.pexec, S.stream));
    }
    *rnorm = rn;
    *converged = conv;
    return k;
}

mgmc_status mgmc_sampler_solve(mgmc_sampler *s, const double *b, double *x, double rtol, double atol, int maxiter,
                               int on_device, int *niter, double *rnorm, int *converged) {
    API_BEGIN
    Sampler &S = impl(s);
    if (!b || !x || !niter || !rnorm || !converged) fail(MGMC_ERR_INVALID_ARGUMENT, "null argument");
    if (maxiter < 0) fail(MGMC_ERR_INVALID_ARGUMENT, "maxiter < 0");
    CK(cudaStreamSynchronize(S.stream));
    S.ensure_solver();
    int k = 0;
    double rn = -1.0;
    bool conv = false;
    {
        BorrowLevel0 borrow(S);
        put_vec(S, 0, b, on_device, S.sv_b, true);
        k = loop_solve(S, rtol, atol, maxiter, &rn, &conv);
        get_vec(S, 0, S.sv_x, x, on_device, true);
    }
    check_device_errors(S);
    *niter = k;
    *rnorm = rn;
    *converged = conv ? 1 : 0;
    API_END
}

mgmc_status mgmc_sampler_exact_sample(mgmc_sampler *s, const double *f, double *x, double rtol, int maxiter,
                                      int on_device, int *niter) {
    API_BEGIN
    Sampler &S = impl(s);
    if (!f || !x) fail(MGMC_ERR_INVALID_ARGUMENT, "null argument");
    if (maxiter < 1 || !(rtol > 0.0)) fail(MGMC_ERR_INVALID_ARGUMENT, "maxiter >= 1 and rtol > 0 required");
    CK(cudaStreamSynchronize(S.stream));
    S.ensure_solver();
    S.ensure_exact();
    Level &l0 = S.L[0];
    int k = 0;
    double rn = -1.0;
    bool conv = false;
    {
        BorrowLevel0 borrow(S);
        put_vec(S, 0, f, on_device, S.sv_b, true);
        NoiseArgs nz{};
        nz.seed = S.P.seed;
        nz.d_step = S.d_step;
        const double *cdiag = l0.var == 1 ? l0.vw64 : nullptr;
        if (l0.npt == 7)
            k_prior_perturbation<7><<<pack_grid(l0), 256, 0, S.stream>>>(S.sv_b, l0.g, S.ew, nz, cdiag, S.ex_offsum);
        else
            k_prior_perturbation<27><<<pack_grid(l0), 256, 0, S.stream>>>(S.sv_b, l0.g, S.ew, nz, cdiag, S.ex_offsum);
        if (S.m > 0) {
            k_lowrank_perturbation<<<nblk(S.m, 256), 256, 0, S.stream>>>(nz, S.d_sigma_sqrt, S.m, S.ex_y);
            launch_add_Bq<double>(S, l0, S.sv_b, S.ex_y, 1.0);
        }
        S.check_launch();
        k = loop_solve(S, rtol, HUGE_VAL, maxiter, &rn, &conv);
        if (!conv) fail(MGMC_ERR_NONFINITE, "exact sample: the solve did not reach the tolerance");
        get_vec(S, 0, S.sv_x, x, on_device, true);
        u64 step = 0;
        CK(cudaMemcpyAsync(&step, S.d_step, sizeof(u64), cudaMemcpyDeviceToHost, S.stream));
        CK(cudaStreamSynchronize(S.stream));
        step += 1;  // the next sample draws new noise
        CK(cudaMemcpyAsync(S.d_step, &step, sizeof(u64), cudaMemcpyHostToDevice, S.stream));
        CK(cudaStreamSynchronize(S.stream));
    }
    check_device_errors(S);
    if (niter) *niter = k;
    API_END
}

// x-bar out of level 0's adj[0], and f-bar += level 0's adj[1]
static void adjoint_outputs(Sampler &S, double *xbar, double *fbar, int on_device) {
    Level &l0 = S.L[0];
    get_vec(S, 0, l0.adj[0], xbar, on_device);
    const i64 n = l0.geo.n;
    double *d = S.d_cvec;
    if (S.fp32)
        k_pack<float><<<pack_grid(l0), 256, 0, S.stream>>>((const float *)l0.adj[1], d, l0.g);
    else
        k_pack<double><<<pack_grid(l0), 256, 0, S.stream>>>((const double *)l0.adj[1], d, l0.g);
    S.check_launch();
    if (on_device) {
        const unsigned blocks = (unsigned)std::min<i64>(nblk(n, 256), 8 * S.nsm);
        k_axpy<double><<<blocks, 256, 0, S.stream>>>(fbar, d, 1.0, n);
        S.check_launch();
    } else {
        std::vector<double> h(n);
        CK(cudaMemcpyAsync(h.data(), d, n * sizeof(double), cudaMemcpyDeviceToHost, S.stream));
        CK(cudaStreamSynchronize(S.stream));
        for (i64 i = 0; i < n; ++i) fbar[i] += h[i];
    }
    CK(cudaStreamSynchronize(S.stream));
}

mgmc_status mgmc_sampler_adjoint_step(mgmc_sampler *s, double *xbar, double *fbar, int on_device) {
    API_BEGIN
    Sampler &S = impl(s);
    if (!xbar || !fbar) fail(MGMC_ERR_INVALID_ARGUMENT, "null argument");
    CK(cudaStreamSynchronize(S.stream));
    S.ensure_adjoint();
    Level &l0 = S.L[0];
    put_vec(S, 0, xbar, on_device, l0.adj[0]);
    if (S.fp32) {
        adj_zero<float>(S, l0, l0.adj[1]);
        S.adjoint_sample<float>(0);
    } else {
        adj_zero<double>(S, l0, l0.adj[1]);
        S.adjoint_sample<double>(0);
    }
    S.check_launch();
    adjoint_outputs(S, xbar, fbar, on_device);
    API_END
}

mgmc_status mgmc_sampler_adjoint_params(mgmc_sampler *s, const double *x_in, int64_t step_index, double *xbar,
                                        double *fbar, double *g_centre, double *g_logsigma, int on_device) {
    API_BEGIN
    Sampler &S = impl(s);
    if (!x_in || !xbar || !fbar || !g_centre || (S.m > 0 && !g_logsigma)) fail(MGMC_ERR_INVALID_ARGUMENT, "null argument");
    if (step_index < 0) fail(MGMC_ERR_INVALID_ARGUMENT, "step_index < 0");
    CK(cudaStreamSynchronize(S.stream));
    if (S.noise_mode == NOISE_INJECTED && S.noise_len - S.noise_pos < S.noise_per_step)
        fail(MGMC_ERR_NOISE_EXHAUSTED, "injected noise exhausted: " + std::to_string(S.noise_len - S.noise_pos) + " queued, " +
                                           std::to_string(S.noise_per_step) + " needed per step");
    S.ensure_solver_buffers();
    S.ensure_param_adjoint();
    Level &l0 = S.L[0];
    const int mm = std::max(S.m, 1);
    double gs = 0.0;
    std::vector<double> gsig(mm, 0.0);
    u64 saved_step = 0;
    CK(cudaMemcpy(&saved_step, S.d_step, sizeof(u64), cudaMemcpyDeviceToHost));
    struct Restore {
        Sampler &S;
        u64 step;
        ~Restore() {
            S.taping = false;
            S.param_adj = false;
            S.noisy = true;
            S.tape.clear();
            cudaMemcpyAsync(S.d_step, &step, sizeof(u64), cudaMemcpyHostToDevice, S.stream);
            cudaStreamSynchronize(S.stream);
        }
    };
    {
        BorrowLevel0 borrow(S);
        Restore restore{S, saved_step};
        put_vec(S, 0, x_in, on_device, l0.x);
        const u64 k = (u64)step_index;
        CK(cudaMemcpyAsync(S.d_step, &k, sizeof(u64), cudaMemcpyHostToDevice, S.stream));
        put_vec(S, 0, xbar, on_device, l0.adj[0]);
        if (S.noise_mode == NOISE_PHILOX && S.pa_calls > 0) {
            if (!S.pa_exec) {
                CK(cudaStreamBeginCapture(S.stream, cudaStreamCaptureModeThreadLocal));
                try {
                    S.param_adjoint_pass();
                } catch (...) {
                    cudaGraph_t g = nullptr;
                    cudaStreamEndCapture(S.stream, &g);
                    if (g) cudaGraphDestroy(g);
                    throw;
                }
                CK(cudaStreamEndCapture(S.stream, &S.pa_graph));
                CK(cudaGraphInstantiate(&S.pa_exec, S.pa_graph, 0));
            }
            CK(cudaGraphLaunch(S.pa_exec, S.stream));
        } else {
            S.param_adjoint_pass();
        }
        S.pa_calls++;
        adjoint_outputs(S, xbar, fbar, on_device);
        CK(cudaMemcpy(&gs, S.pa_gs, sizeof(double), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(gsig.data(), S.pa_gsig, mm * sizeof(double), cudaMemcpyDeviceToHost));
    }
    if (S.noise_mode == NOISE_INJECTED) S.noise_pos += S.noise_per_step;
    check_device_errors(S);
    *g_centre += gs;
    for (int k = 0; k < S.m; ++k) g_logsigma[k] += gsig[k];
    API_END
}
