// kernels.cuh -- sm_103a kernels of the Multigrid Monte Carlo step.
//
// Data layout (every level): padded lexicographic arrays with shared ghost
// rows/planes, see Geometry in setup.h.  A point with 0-based interior
// coordinates (a, b, c) lives at P = (c+1) sz + (b+1) sy + (a+1); ghosts are
// zero, so stencil loads need no boundary tests.
//
// Kernels (one V-cycle at level l uses them in this order):
//   k_sweep_rb_vec      one colour of the red-black SOR sweep of the 7-point
//                       level, FP32, 8-point spans with float4 loads/stores
//   k_sweep_rb_pass     the same, one point per thread (FP64, parity)
//   k_sweep_c27_pass    one colour of the 8-colour SOR sweep of a 27-point level
//   k_sweep_wavefront   lexicographic SOR sweep as a hyperplane wavefront
//                       (one CTA; parity mode)
//   k_bt_partial        partial sums of y = B^T x
//   k_bt_solve          the partial sums and, in the last CTA, the solve
//   k_lr_solve          y and the m x m low-rank solve
//   k_lr_apply          the solve and x += C z over the rows of C = M^{-1} B
//   k_lr_scatter        x += C z (large supports, after k_bt_solve)
//   k_resid_restrict_tma    f_c = R (f - A_0 x), TMA tiles (fused residual
//                           + restriction; _tiled / plain variants otherwise)
//   k_add_Bq            f_c -= B_c Sigma^{-1} y
//   k_prolong_add       x += alpha P x_c
//   k_chol_gemv_*       coarse-level Cholesky sample (k_chol_subst: parity)
//   k_step_end          observables z = b^T x, step counter
// Host conversions: k_unpack / k_unpack2 / k_pack; adjoint helpers: k_axpy,
// k_sinvt_q; deterministic solver (FP64 loop around the noise-free cycle):
// k_solve_resid, k_solve_rhs, k_solve_norm, k_solve_update; parameter
// adjoint: k_pgrad_stencil, k_pgrad_combine, k_lowrank_normals,
// k_coarse_normals, k_pgrad_coarse_phi, k_pgrad_coarse_sigma, k_accum_sum;
// building blocks: k_apply_stencil.
#pragma once

#include <cstdint>
#include <cuda.h>  // CUtensorMap (type only; the driver entry point is resolved at run time)
#include <cuda_runtime.h>
#include <type_traits>

namespace mgmc {

typedef long long i64;
typedef unsigned long long u64;

// Programmatic dependent launch: wait until the previous kernel on the
// stream has completed and its writes are visible (a kernel launched with
// the programmatic-serialization attribute may start while its predecessor
// drains; the predecessor triggers it implicitly as its CTAs exit).  Without
// the attribute this is a no-op.  (An explicit griddepcontrol.launch_dependents
// right after the wait, which schedules the next kernel's CTAs while this
// grid runs, made the 256^3 step 1.8 % slower: the waiting CTAs hold SM
// slots the running grid needs.)
__device__ __forceinline__ void pdl_begin() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
// Let the next kernel on the stream start its CTAs now (they still wait in
// pdl_begin until this grid has completed).  Used where one CTA is left
// working alone, so that the next kernel's independent loads overlap it.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// ------------------------------------------------------------- geometry
struct Grid3 {
    int N0, N1, N2;  // interior vertices per direction
    i64 sy, sz;      // padded strides
    int pdl = 0;     // kernels on this level take part in programmatic dependent launch
    __host__ __device__ i64 pad(int a, int b, int c) const { return (i64)(c + 1) * sz + (i64)(b + 1) * sy + (a + 1); }
    __host__ __device__ i64 compact(int a, int b, int c) const { return ((i64)c * N1 + b) * N0 + a; }
};

template <typename T>
struct StencilArg {
    T w[27];  // (dz+1)*9 + (dy+1)*3 + (dx+1)
    T diag;   // w[13]
    T omega;
    T sd;         // sqrt(diag (2 - omega) / omega): noise scale (sor_sampler.cc:20-27)
    T omega_diag; // omega / diag
    T tmo;        // 2 - omega (per-point noise scales of variable stencils)
};

// Per-point stencil of a level with variable coefficients.  VAR == 1: w[P]
// (padded index) is the centre weight, the other weights are the constant
// ones of StencilArg; VAR == 2: w[k * stride + P] is weight k.  VAR == 0:
// the constant StencilArg alone.
template <typename T>
struct VarField {
    const T *w;
    i64 stride;
};

template <typename T, int VAR>
__device__ __forceinline__ T vweight(const StencilArg<T> &s, const VarField<T> &vf, i64 P, int k) {
    if (VAR == 2) return vf.w[(i64)k * vf.stride + P];
    if (VAR == 1 && k == 13) return vf.w[P];
    return s.w[k];
}

// ---------------------------------------------------------------- noise
enum { NOISE_NONE = 0, NOISE_PHILOX = 1, NOISE_INJECTED = 2 };
enum { PURPOSE_POINT = 0, PURPOSE_LOWRANK = 1, PURPOSE_COARSE = 2, PURPOSE_EXACT = 3, PURPOSE_CHOLESKY = 4 };

struct NoiseArgs {
    const double *buf;   // injected: normals for this consumer, index = vertex / column
    u64 seed;            // Philox key
    const u64 *d_step;   // device step counter
    unsigned invocation; // position of this noise consumer inside one step
    unsigned level;
};

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11): 10 rounds of the 4x32 bijection with the
// published multipliers and Weyl key increments.
__device__ __forceinline__ uint4 philox4x32_10(uint4 ctr, uint2 key) {
    const unsigned M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const unsigned W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        unsigned lo0 = M0 * ctr.x, hi0 = __umulhi(M0, ctr.x);
        unsigned lo1 = M1 * ctr.z, hi1 = __umulhi(M1, ctr.z);
        ctr = make_uint4(hi1 ^ ctr.y ^ key.x, lo1, hi0 ^ ctr.w ^ key.y, lo0);
        key.x += W0;
        key.y += W1;
    }
    return ctr;
}

// Two Box-Muller pairs in FP32 (Box & Muller 1958) with the SFU
// approximations of log2, reciprocal square root and sine/cosine (absolute
// error of order 1e-6 per normal).  u1 is in (0, 1]: the product of a
// value <= 2^32 with 2^-32 plus 2^-33 rounds to at most 1.0f, so -log2(u1)
// is never negative; the angle lies in [-pi, pi), the accurate range of the
// fast sine and cosine.
__device__ __forceinline__ float4 normals4(uint4 r) {
    const float two_m32 = 2.3283064365386963e-10f;  // 2^-32
    const float two_m33 = 1.1641532182693481e-10f;  // 2^-33
    const float m2ln2 = -1.3862943611198906f;       // -2 ln 2
    const float twopi = 6.283185307179586f;
    float u1a = __fmaf_rn(__uint2float_rn(r.x), two_m32, two_m33);
    float u1b = __fmaf_rn(__uint2float_rn(r.z), two_m32, two_m33);
    float qa = fmaxf(m2ln2 * __log2f(u1a), 1e-30f);
    float qb = fmaxf(m2ln2 * __log2f(u1b), 1e-30f);
    float ra = qa * rsqrtf(qa), rb = qb * rsqrtf(qb);
    float sa, ca, sb, cb;
    __sincosf(__fmaf_rn(__uint2float_rz(r.y), two_m32, -0.5f) * twopi, &sa, &ca);
    __sincosf(__fmaf_rn(__uint2float_rz(r.w), two_m32, -0.5f) * twopi, &sb, &cb);
    return make_float4(ra * ca, ra * sa, rb * cb, rb * sb);
}

__device__ __forceinline__ float pick(float4 v, int lane) {
    return lane == 0 ? v.x : (lane == 1 ? v.y : (lane == 2 ? v.z : v.w));
}

__device__ __forceinline__ uint4 noise_ctr(const NoiseArgs &nz, unsigned x, unsigned purpose, unsigned low) {
    u64 sc = (*nz.d_step) * 4096ull + nz.invocation;
    return make_uint4(x, (purpose << 24) | (nz.level << 8) | low, (unsigned)sc, (unsigned)(sc >> 32));
}

__device__ __forceinline__ uint2 noise_key(const NoiseArgs &nz) {
    return make_uint2((unsigned)nz.seed, (unsigned)(nz.seed >> 32));
}

// Normals of the 4 points of x-parity (a & 1) inside the 8-point x-group
// a >> 3 of row (b, c): lane (a & 7) >> 1.
__device__ __forceinline__ float4 point_normals(const NoiseArgs &nz, const Grid3 &g, int a, int b, int c) {
    unsigned G0 = (unsigned)((g.N0 + 7) >> 3);
    unsigned grp = (unsigned)(((u64)c * g.N1 + b) * G0 + (a >> 3));
    return normals4(philox4x32_10(noise_ctr(nz, grp, PURPOSE_POINT, a & 1), noise_key(nz)));
}

// ------------------------------------------------------- exact arithmetic
// Parity kernels evaluate the reference's expressions with one rounding per
// operation (no FMA contraction), as the reference's compiled CPU code does.
template <bool EXACT>
struct Ar;
template <>
struct Ar<true> {
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
};
template <>
struct Ar<false> {
    template <typename T>
    static __device__ __forceinline__ T mul(T a, T b) { return a * b; }
    template <typename T>
    static __device__ __forceinline__ T add(T a, T b) { return a + b; }
    template <typename T>
    static __device__ __forceinline__ T sub(T a, T b) { return a - b; }
};

// One SOR point update (sor_smoother.cc:66-76 with the noisy right hand
// side of sor_sampler.cc:42-46):
//   c = sd * xi + f;  res = sum_k w_k x_k (ascending index, diagonal
//   included);  x += omega * (c - res) / diag.
// Row P of A_0 x: sum_k w_k x_k in ascending index order, diagonal
// included, with the neighbour (dz, dy, dx) of P read through xa(dz, dy, dx)
// (global memory or values loaded beforehand: the same arithmetic either way).
template <typename T, int NPT, bool EXACT, int VAR, typename XA>
__device__ __forceinline__ T stencil_row_acc(const XA &xa, const StencilArg<T> &s, i64 P, const VarField<T> &vf) {
    typedef Ar<EXACT> A;
    T res = T(0);
    if (NPT == 7) {
        const int ks[7] = {4, 10, 12, 13, 14, 16, 22};
        const int dzs[7] = {-1, 0, 0, 0, 0, 0, 1}, dys[7] = {0, -1, 0, 0, 0, 1, 0}, dxs[7] = {0, 0, -1, 0, 1, 0, 0};
#pragma unroll
        for (int q = 0; q < 7; ++q) res = A::add(res, A::mul(vweight<T, VAR>(s, vf, P, ks[q]), xa(dzs[q], dys[q], dxs[q])));
    } else {
#pragma unroll
        for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
            for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
                for (int dx = -1; dx <= 1; ++dx)
                    res = A::add(res, A::mul(vweight<T, VAR>(s, vf, P, (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1)),
                                             xa(dz, dy, dx)));
    }
    return res;
}

template <typename T, int NPT, bool EXACT, int VAR = 0>
__device__ __forceinline__ T stencil_row(const T *__restrict__ x, const Grid3 &g, const StencilArg<T> &s, i64 P,
                                         const VarField<T> &vf = VarField<T>{nullptr, 0}) {
    return stencil_row_acc<T, NPT, EXACT, VAR>(
        [&](int dz, int dy, int dx) { return x[P + dz * g.sz + dy * g.sy + dx]; }, s, P, vf);
}

// The updated value of point P from its neighbours (xa), old value xo and
// right hand side fv.  With a variable stencil (VAR != 0) the diagonal, the
// noise scale sqrt(d (2 - omega) / omega) and omega / d are formed per
// point, in the oracle's operation order on the parity path.
template <typename T, int NPT, bool EXACT, int VAR, typename XA>
__device__ __forceinline__ T sor_value(const XA &xa, T xo, T fv, const StencilArg<T> &s, i64 P, bool noisy, T xi,
                                       const VarField<T> &vf) {
    typedef Ar<EXACT> A;
    const T res = stencil_row_acc<T, NPT, EXACT, VAR>(xa, s, P, vf);
    T cval = fv;
    if (VAR == 0) {
        if (noisy) cval = A::add(A::mul(s.sd, xi), cval);
        if (EXACT) return A::add(xo, A::mul(s.omega, A::sub(cval, res)) / s.diag);
        return xo + s.omega_diag * (cval - res);
    }
    const T d = vweight<T, VAR>(s, vf, P, 13);
    if (noisy) {
        const T sd = sqrt(A::mul(d, s.tmo) / s.omega);
        cval = A::add(A::mul(sd, xi), cval);
    }
    if (EXACT) return A::add(xo, A::mul(s.omega, A::sub(cval, res)) / d);
    return xo + (s.omega / d) * (cval - res);
}

template <typename T, int NPT, bool EXACT, int VAR = 0>
__device__ __forceinline__ void sor_point(T *__restrict__ x, const T *__restrict__ f, const Grid3 &g,
                                          const StencilArg<T> &s, i64 P, bool noisy, T xi,
                                          const VarField<T> &vf = VarField<T>{nullptr, 0}) {
    x[P] = sor_value<T, NPT, EXACT, VAR>([&](int dz, int dy, int dx) { return x[P + dz * g.sz + dy * g.sy + dx]; },
                                         x[P], f[P], s, P, noisy, xi, vf);
}

// ------------------------------------------------- red-black SOR sweep
// Noise of a 7-point level: the normals of the 4 points of one x-parity in
// the 8-aligned group of padded positions P = a + 1 in [8q, 8q + 8) of row
// (b, c) come from one Philox block, lane (P & 7) >> 1.
__device__ __forceinline__ float4 fine_normals(const NoiseArgs &nz, const Grid3 &g, int P, int b, int c) {
    const unsigned G0 = (unsigned)((g.N0 + 1) >> 3) + 1u;
    const unsigned grp = (unsigned)(((u64)c * g.N1 + b) * G0 + (P >> 3));
    return normals4(philox4x32_10(noise_ctr(nz, grp, PURPOSE_POINT, P & 1), noise_key(nz)));
}

// One colour of a red-black sweep of an axis-only (7-point) level, one
// thread per point of the colour.  A CTA is blockDim.x points along x times
// blockDim.y rows (b) of one plane c (sweep_block() picks the shape so that
// no thread idles on short rows); each warp load reads a contiguous span.
// `reverse` walks the planes from the top so that the second colour finds
// the data the first colour touched last in L2.
constexpr int RBP_THREADS = 256;

// CTA shape for `count` work items along x: the smallest power of two
// >= count (at least 8, at most RBP_THREADS) along x, the rest along y.
__host__ __forceinline__ dim3 sweep_block(int count) {
    int tx = 8;
    while (tx < count && tx < RBP_THREADS) tx *= 2;
    return dim3(tx, RBP_THREADS / tx, 1);
}

template <typename T, bool EXACT, int NOISE, int VAR = 0>
__global__ void __launch_bounds__(RBP_THREADS) k_sweep_rb_pass(T *__restrict__ x, const T *__restrict__ f, Grid3 g,
                                                               StencilArg<T> s, int colour, int reverse, NoiseArgs nz,
                                                               VarField<T> vf) {
    if (g.pdl) pdl_begin();
    const int b = blockIdx.y * blockDim.y + threadIdx.y;
    const int c = reverse ? g.N2 - 1 - (int)blockIdx.z : (int)blockIdx.z;
    if (b >= g.N1) return;
    const int p = (colour + b + c) & 1;
    const int a = 2 * (blockIdx.x * blockDim.x + threadIdx.x) + p;
    T xi = T(0);
    if (NOISE == NOISE_PHILOX) xi = (T)pick(fine_normals(nz, g, a + 1, b, c), ((a + 1) & 7) >> 1);
    if (a >= g.N0) return;
    if (NOISE == NOISE_INJECTED) xi = (T)nz.buf[g.compact(a, b, c)];
    sor_point<T, 7, EXACT, VAR>(x, f, g, s, g.pad(a, b, c), NOISE != NOISE_NONE, xi, vf);
}

// 256-bit vector access (sm_100 and later): 8 floats at a 32-byte aligned
// address in one instruction.  ld8 reads through L1 (x is written in the
// same pass); read-once streams use ld8_stream below.
__device__ __forceinline__ void ld8(const float *p, float *v) {
    asm volatile("ld.global.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
                 : "l"(p)
                 : "memory");
}
// Read-once streams (f and the centre field of the fine sweep): no L1
// allocation, and first in line for L2 eviction, so that the L2 keeps x --
// which the next colour pass reads again -- rather than f, which it does
// not.  (Measured at 256^3: 53.3 -> 49.7 us per two-pass sweep.)
__device__ __forceinline__ unsigned long long l2_evict_first_policy() {
    unsigned long long p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ float4 ld4_stream(const float *p, unsigned long long pol) {
    float4 r;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.f32 {%0,%1,%2,%3}, [%4], %5;"
        : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w)
        : "l"(p), "l"(pol));
    return r;
}
__device__ __forceinline__ void ld8_stream(const float *p, float *v, unsigned long long pol) {
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8], %9;"
        : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
        : "l"(p), "l"(pol));
}
__device__ __forceinline__ void st8(float *p, const float *v) {
    asm volatile("st.global.v8.f32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"l"(p), "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]),
                 "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7])
                 : "memory");
}

// FP32 variant with vector loads (rows padded to a multiple of 4 floats): a
// thread owns the 8 padded positions [8q, 8q + 8) of a row, loads them and
// the matching spans of the four neighbouring rows and f as float4, draws
// one Philox block for its 4 points of the colour and stores those 4 points.
// VD: a per-point centre weight field vd (same padded layout), loaded as a
// fifth pair of float4 spans.  V8 (rows a multiple of 8 floats): every span
// is one 256-bit access instead of two float4 ones, which halves the L1
// wavefronts of the loads (a warp's 32-byte spans are contiguous).  FS (with
// V8): f comes from fsc, the colour's half of f split by colour
// (k_split_colours), so the pass reads one float4 of f per span -- only the
// values it uses -- instead of the whole span.
// The body, with the CTA coordinates (bx, by, bz) passed in: the solo
// kernel below and the batched kernel (k_sweep_rb_vec_batch) run the same
// arithmetic.
template <int NOISE, bool VD, bool V8, bool FS>
__device__ __forceinline__ void sweep_rb_vec_body(float *__restrict__ x, const float *__restrict__ f, const Grid3 &g,
                                                  const StencilArg<float> &s, int colour, int reverse,
                                                  const NoiseArgs &nz, const float *__restrict__ vd,
                                                  const float *__restrict__ fsc, int bx, int by, int bz) {
    const int b = by * blockDim.y + threadIdx.y;
    const int c = reverse ? g.N2 - 1 - bz : bz;
    const int q = bx * blockDim.x + threadIdx.x;
    const int ngrp = (g.N0 + 8) >> 3;
    if (q >= ngrp || b >= g.N1) return;
    const int P0 = 8 * q;
    const i64 rb = (i64)(c + 1) * g.sz + (i64)(b + 1) * g.sy;
    const float4 *xr = reinterpret_cast<const float4 *>(x + rb + P0);
    const float4 *xn = reinterpret_cast<const float4 *>(x + rb - g.sy + P0);
    const float4 *xs_ = reinterpret_cast<const float4 *>(x + rb + g.sy + P0);
    const float4 *xd = reinterpret_cast<const float4 *>(x + rb - g.sz + P0);
    const float4 *xu = reinterpret_cast<const float4 *>(x + rb + g.sz + P0);
    const float4 *fr = reinterpret_cast<const float4 *>(f + rb + P0);
    float v[10], ym[8], yp[8], zm[8], zp[8], fv[8], dv[8];
    const unsigned long long pol_stream = V8 ? l2_evict_first_policy() : 0ull;
    if (VD) {
        if (V8) {
            ld8_stream(vd + rb + P0, dv, pol_stream);
        } else {
            const float4 *dr = reinterpret_cast<const float4 *>(vd + rb + P0);
            const float4 d0 = dr[0], d1 = dr[1];
            dv[0] = d0.x; dv[1] = d0.y; dv[2] = d0.z; dv[3] = d0.w; dv[4] = d1.x; dv[5] = d1.y; dv[6] = d1.z; dv[7] = d1.w;
        }
    }
    // points of the colour: padded P with (P - 1 + b + c) & 1 == colour; the
    // two parities get separate code so that every register index is static
    const int j0 = (colour + b + c + 1) & 1;  // first local index j (P = P0 + j) of the colour
    if (V8) {
        v[0] = P0 > 0 ? x[rb + P0 - 1] : 0.f;
        ld8(x + rb + P0, v + 1);
        v[9] = x[rb + P0 + 8];
        ld8(x + rb - g.sy + P0, ym);
        ld8(x + rb + g.sy + P0, yp);
        ld8(x + rb - g.sz + P0, zm);
        ld8(x + rb + g.sz + P0, zp);
        if (FS) {
            const float4 fq = ld4_stream(fsc + ((rb + P0) >> 1), pol_stream);
            if (j0 == 0) {
                fv[0] = fq.x; fv[2] = fq.y; fv[4] = fq.z; fv[6] = fq.w;
            } else {
                fv[1] = fq.x; fv[3] = fq.y; fv[5] = fq.z; fv[7] = fq.w;
            }
        } else {
            ld8_stream(f + rb + P0, fv, pol_stream);
        }
    } else {
        const float4 a0 = xr[0], a1 = xr[1];
        v[0] = P0 > 0 ? x[rb + P0 - 1] : 0.f;  // P0 - 1 is a ghost column for q = 0 (read 0 directly)
        v[1] = a0.x; v[2] = a0.y; v[3] = a0.z; v[4] = a0.w;
        v[5] = a1.x; v[6] = a1.y; v[7] = a1.z; v[8] = a1.w;
        v[9] = x[rb + P0 + 8];
        const float4 n0 = xn[0], n1 = xn[1], s0 = xs_[0], s1 = xs_[1], d0 = xd[0], d1 = xd[1], u0 = xu[0], u1 = xu[1];
        const float4 f0 = fr[0], f1 = fr[1];
        ym[0] = n0.x; ym[1] = n0.y; ym[2] = n0.z; ym[3] = n0.w; ym[4] = n1.x; ym[5] = n1.y; ym[6] = n1.z; ym[7] = n1.w;
        yp[0] = s0.x; yp[1] = s0.y; yp[2] = s0.z; yp[3] = s0.w; yp[4] = s1.x; yp[5] = s1.y; yp[6] = s1.z; yp[7] = s1.w;
        zm[0] = d0.x; zm[1] = d0.y; zm[2] = d0.z; zm[3] = d0.w; zm[4] = d1.x; zm[5] = d1.y; zm[6] = d1.z; zm[7] = d1.w;
        zp[0] = u0.x; zp[1] = u0.y; zp[2] = u0.z; zp[3] = u0.w; zp[4] = u1.x; zp[5] = u1.y; zp[6] = u1.z; zp[7] = u1.w;
        fv[0] = f0.x; fv[1] = f0.y; fv[2] = f0.z; fv[3] = f0.w; fv[4] = f1.x; fv[5] = f1.y; fv[6] = f1.z; fv[7] = f1.w;
    }
    float4 nrm = make_float4(0.f, 0.f, 0.f, 0.f);
    if (NOISE == NOISE_PHILOX) nrm = fine_normals(nz, g, P0 + j0, b, c);
    auto upd = [&](int j, int k) {
        const int a = P0 + j - 1;
        if (a < 0 || a >= g.N0) return;
        float xi = 0.f;
        if (NOISE == NOISE_PHILOX) xi = pick(nrm, k);
        if (NOISE == NOISE_INJECTED) xi = (float)nz.buf[g.compact(a, b, c)];
        const float dg = VD ? dv[j] : s.w[13];
        float res = s.w[4] * zm[j];
        res = fmaf(s.w[10], ym[j], res);
        res = fmaf(s.w[12], v[j], res);
        res = fmaf(dg, v[j + 1], res);
        res = fmaf(s.w[14], v[j + 2], res);
        res = fmaf(s.w[16], yp[j], res);
        res = fmaf(s.w[22], zp[j], res);
        float cval = fv[j];
        const float sd = VD ? sqrtf(dg * s.tmo / s.omega) : s.sd;
        if (NOISE != NOISE_NONE) cval = fmaf(sd, xi, cval);
        const float od = VD ? s.omega / dg : s.omega_diag;
        v[j + 1] = v[j + 1] + od * (cval - res);  // neighbours are of the other colour
    };
    if (j0 == 0) {
        upd(0, 0);
        upd(2, 1);
        upd(4, 2);
        upd(6, 3);
    } else {
        upd(1, 0);
        upd(3, 1);
        upd(5, 2);
        upd(7, 3);
    }
    // Whole 8-position spans go back as two float4 stores (full sectors
    // instead of one partial sector per point); the other colour's values
    // are rewritten unchanged -- no thread writes them in this pass.  A span
    // that reaches past its row (short rows only) stores its second half
    // point by point.
    if (V8 && P0 + 8 <= g.sy) {
        st8(x + rb + P0, v + 1);
        return;
    }
    float4 *xo = reinterpret_cast<float4 *>(x + rb + P0);
    xo[0] = make_float4(v[1], v[2], v[3], v[4]);
    if (P0 + 8 <= g.sy) {
        xo[1] = make_float4(v[5], v[6], v[7], v[8]);
    } else {
#pragma unroll
        for (int j = 4; j < 8; ++j) {
            const int a = P0 + j - 1;
            if (((j - j0) & 1) == 0 && a >= 0 && a < g.N0) x[rb + P0 + j] = v[j + 1];
        }
    }
}

template <int NOISE, bool VD = false, bool V8 = false, bool FS = false>
__global__ void __launch_bounds__(RBP_THREADS) k_sweep_rb_vec(float *__restrict__ x, const float *__restrict__ f,
                                                              Grid3 g, StencilArg<float> s, int colour, int reverse,
                                                              NoiseArgs nz, const float *__restrict__ vd,
                                                              const float *__restrict__ fsc) {
    if (g.pdl) pdl_begin();
    sweep_rb_vec_body<NOISE, VD, V8, FS>(x, f, g, s, colour, reverse, nz, vd, fsc, blockIdx.x, blockIdx.y, blockIdx.z);
}

// Level 0's f split by colour for the FP32 fine sweep: the value of point
// (a, b, c) of colour k = (a + b + c) & 1 at fs[k * half + (P >> 1)], P its
// padded index.  With even row and plane pitches, the two points P = 2i,
// 2i + 1 of a row have different colours, so each colour's half holds one
// value per pair, and a span [8q, 8q + 8) of a row maps to one float4.
__global__ void __launch_bounds__(256) k_split_colours(const float *__restrict__ f, float *__restrict__ fs, i64 half,
                                                       Grid3 g) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y, c = blockIdx.z;
    if (a >= g.N0) return;
    const i64 P = g.pad(a, b, c);
    fs[(i64)((a + b + c) & 1) * half + (P >> 1)] = f[P];
}

// One colour of an 8-colour (27-point) sweep, one thread per point (colour
// index (a & 1) | (b & 1) << 1 | (c & 1) << 2).
template <typename T, bool EXACT, int NOISE, int VAR>
__device__ __forceinline__ void sweep_c27_body(T *__restrict__ x, const T *__restrict__ f, const Grid3 &g,
                                               const StencilArg<T> &s, int colour, const NoiseArgs &nz,
                                               const VarField<T> &vf, int bx, int by, int bz) {
    const int pa = colour & 1, pb = (colour >> 1) & 1, pc = (colour >> 2) & 1;
    const int a = 2 * (bx * blockDim.x + threadIdx.x) + pa;
    const int b = 2 * (by * blockDim.y + threadIdx.y) + pb, c = 2 * bz + pc;
    if (b >= g.N1 || c >= g.N2) return;
    T xi = T(0);
    if (NOISE == NOISE_PHILOX) xi = (T)pick(point_normals(nz, g, a, b, c), (a & 7) >> 1);
    if (a >= g.N0) return;
    if (NOISE == NOISE_INJECTED) xi = (T)nz.buf[g.compact(a, b, c)];
    const i64 P = g.pad(a, b, c);
    if (sizeof(T) == 4 && (g.sy & 1) == 0 && (g.sz & 1) == 0) {
        // FP32, even pitches: the points of a colour share the parity of P,
        // and each of the nine rows of the stencil is one aligned pair load
        // plus one single load (the threads of a warp, two points apart, then
        // read whole sectors); the same values in the same order as
        // sor_point.  (Measured at 256^3: FP32 step 0.766 -> 0.759 ms; the
        // FP64 chain was 0.4 % slower with 16-byte pairs and keeps sor_point.)
        typedef typename std::conditional<sizeof(T) == 4, float2, double2>::type T2;
        const bool odd = (P & 1) != 0;
        T v[27];
#pragma unroll
        for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
            for (int dy = -1; dy <= 1; ++dy) {
                const T *r = x + P + dz * g.sz + dy * g.sy;
                const int k = (dz + 1) * 9 + (dy + 1) * 3;
                if (odd) {
                    const T2 q = *reinterpret_cast<const T2 *>(r - 1);
                    v[k] = q.x;
                    v[k + 1] = q.y;
                    v[k + 2] = r[1];
                } else {
                    const T2 q = *reinterpret_cast<const T2 *>(r);
                    v[k] = r[-1];
                    v[k + 1] = q.x;
                    v[k + 2] = q.y;
                }
            }
        x[P] = sor_value<T, 27, EXACT, VAR>([&](int dz, int dy, int dx) { return v[(dz + 1) * 9 + (dy + 1) * 3 + dx + 1]; },
                                            v[13], f[P], s, P, NOISE != NOISE_NONE, xi, vf);
        return;
    }
    sor_point<T, 27, EXACT, VAR>(x, f, g, s, P, NOISE != NOISE_NONE, xi, vf);
}

template <typename T, bool EXACT, int NOISE, int VAR = 0>
__global__ void __launch_bounds__(RBP_THREADS) k_sweep_c27_pass(T *__restrict__ x, const T *__restrict__ f, Grid3 g,
                                                                StencilArg<T> s, int colour, NoiseArgs nz,
                                                                VarField<T> vf) {
    if (g.pdl) pdl_begin();
    sweep_c27_body<T, EXACT, NOISE, VAR>(x, f, g, s, colour, nz, vf, blockIdx.x, blockIdx.y, blockIdx.z);
}

// ------------------------------------------------ lexicographic wavefront
// Lexicographic order as hyperplanes t = a + hb b + hc c: every neighbour
// that precedes a point lexicographically lies on an earlier hyperplane
// ((1,1,1) for axis stencils, (1,2,4) for 27-point stencils), points on one
// hyperplane are independent.  One CTA, one __syncthreads per hyperplane.
template <typename T, int NPT, bool EXACT, int NOISE>
__global__ void __launch_bounds__(1024) k_sweep_wavefront(T *__restrict__ x, const T *__restrict__ f, Grid3 g,
                                                           StencilArg<T> s, int forward, int hb, int hc, NoiseArgs nz) {
    if (g.pdl) pdl_begin();
    const int tmax = (g.N0 - 1) + hb * (g.N1 - 1) + hc * (g.N2 - 1);
    const int npair = g.N1 * g.N2;
    for (int step = 0; step <= tmax; ++step) {
        const int t = forward ? step : tmax - step;
        for (int pr = threadIdx.x; pr < npair; pr += blockDim.x) {
            int b = pr % g.N1, c = pr / g.N1;
            int a = t - hb * b - hc * c;
            if (a < 0 || a >= g.N0) continue;
            T xi = T(0);
            if (NOISE == NOISE_PHILOX) xi = (T)pick(point_normals(nz, g, a, b, c), (a & 7) >> 1);
            if (NOISE == NOISE_INJECTED) xi = (T)nz.buf[g.compact(a, b, c)];
            sor_point<T, NPT, EXACT>(x, f, g, s, g.pad(a, b, c), NOISE != NOISE_NONE, xi);
        }
        __syncthreads();
    }
}

// ----------------------------------------------------------- reductions
template <int NT>
__device__ __forceinline__ double block_sum(double v, double *sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sh[w] = v;
    __syncthreads();
    v = (threadIdx.x < NT / 32) ? sh[threadIdx.x] : 0.0;
    if (w == 0) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    }
    __syncthreads();
    return v;  // valid in warp 0
}

// ------------------------------------------------ float-float arithmetic
// An unevaluated sum hi + lo of two FP32 numbers carries about 48
// significant bits.  GB300 issues about two FP64 FMAs per clock per SM
// against 128 FP32 ones, so the FP32 chain forms the cross-thread sums of
// B^T x and the low-rank m x m product in this arithmetic instead of FP64.
// Error-free transformations: TwoSum (Knuth, TAOCP vol. 2, 4.2.2), Fast
// TwoSum (Dekker 1971) and TwoProd with an FMA (Ogita, Rump, Oishi,
// "Accurate sum and dot product", SIAM J. Sci. Comput. 26, 2005).  The _rn
// intrinsics keep the compiler from contracting a product and a sum into one
// FMA, which would break the transformations.
struct ff32 {
    float hi, lo;
};

__device__ __forceinline__ ff32 two_sum(float a, float b) {  // s + e == a + b exactly
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ ff32 fast_two_sum(float a, float b) {  // exact when |a| >= |b| or a == 0
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
// (a.hi + a.lo) + (b.hi + b.lo): both parts summed with TwoSum, then
// renormalised twice (accurate under cancellation).  Symmetric in a and b
// bit for bit, since TwoSum's error term is the exact error.
__device__ __forceinline__ ff32 ff_add(ff32 a, ff32 b) {
    ff32 s = two_sum(a.hi, b.hi);
    const ff32 t = two_sum(a.lo, b.lo);
    s = fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
    return fast_two_sum(s.hi, __fadd_rn(s.lo, t.lo));
}
// (a.hi + a.lo) (b.hi + b.lo) without the a.lo b.lo term
__device__ __forceinline__ ff32 ff_mul(ff32 a, ff32 b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return fast_two_sum(p, e);
}
__device__ __forceinline__ ff32 ff_neg(ff32 a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ ff32 ff_of(float2 v) { return {v.x, v.y}; }
__device__ __forceinline__ double ff_to_double(ff32 a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ float ff_to_float(ff32 a) { return __fadd_rn(a.hi, a.lo); }

// block_sum's shuffle tree in float-float; the result is valid in warp 0
template <int NT>
__device__ __forceinline__ ff32 block_sum_ff(ff32 v, float2 *sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v = ff_add(v, ff32{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)});
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sh[w] = make_float2(v.hi, v.lo);
    __syncthreads();
    v = (threadIdx.x < NT / 32) ? ff_of(sh[threadIdx.x]) : ff32{0.f, 0.f};
    if (w == 0) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            v = ff_add(v, ff32{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)});
    }
    __syncthreads();
    return v;
}

// Low-rank arguments of one level and sweep direction.
struct LowRankArg {
    int m;
    const i64 *Bptr;    // m+1, CSC of B
    const unsigned *Bidx;  // padded indices (levels below 2^32 padded points)
    const double *Bval;
    const double *SinvT; // m x m, S^{-1} = (Sigma + B^T M^{-1} B)^{-1}, transposed (column q contiguous)
    const double *sigma_sqrt; // Sigma^{1/2}
    double *y;          // m scratch: B^T x
    double *z;          // m scratch: coefficients of C
    float *zf;          // the same coefficients rounded to FP32 (FP32 chain)
    const float *Bvalf; // B values rounded to FP32 (FP32 chain)
    double *part;       // m x P scratch: partial sums of B^T x (the FP32 chain
                        // stores float-float pairs, float2, in the same slots)
    unsigned *counter;  // CTA counter of k_bt_solve (reset by its last CTA)
    const float2 *SinvT_ff;      // SinvT as float-float pairs (FP32 chain)
    const float2 *sigma_sqrt_ff; // Sigma^{1/2} as float-float pairs (FP32 chain)
};

// Partial sums of y_j = sum_i B_ij x_i: gridDim.y CTAs per column j, CTA p
// writing part[j * P + p].  Each thread issues eight index/value loads, then
// the eight gathers of x, before it accumulates them in entry order; the
// per-thread sums are in the state's precision (FP32 products for the FP32
// chain) and are combined across the CTA in FP64, or in float-float for the
// FP32 chain (stored as a float2 in the slot).  B does not change, so a
// thread's first index/value loads are issued before the wait for the
// kernel that wrote x (`wait`: the caller has not waited yet).
template <typename T>
__device__ __forceinline__ void bt_partial_cta(const T *__restrict__ x, const LowRankArg &lr, double *sh, int j, int p,
                                               int P, bool wait = false) {
    const i64 e0 = lr.Bptr[j], e1 = lr.Bptr[j + 1];
    const i64 len = (e1 - e0 + P - 1) / P;
    const i64 lo = e0 + p * len, hi = min(e1, lo + len);
    T tacc = T(0);
    i64 idx[8];
    T val[8];
    auto load = [&](i64 e) {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const i64 ee = e + 256 * k;
            idx[k] = ee < hi ? (i64)lr.Bidx[ee] : -1;
            val[k] = ee < hi ? (sizeof(T) == 4 ? (T)lr.Bvalf[ee] : (T)lr.Bval[ee]) : T(0);
        }
    };
    i64 e = lo + threadIdx.x;
    load(e);
    if (wait) pdl_begin();
    // eight index/value loads, then the eight gathers, in flight at once;
    // the products are added in entry order
    for (; e < hi; e += 8 * 256) {
        T xv[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) xv[k] = idx[k] >= 0 ? x[idx[k]] : T(0);
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (idx[k] >= 0) tacc += val[k] * xv[k];
        if (e + 8 * 256 < hi) load(e + 8 * 256);
    }
    if (sizeof(T) == 4) {
        const ff32 acc = block_sum_ff<256>(ff32{(float)tacc, 0.f}, reinterpret_cast<float2 *>(sh));
        if (threadIdx.x == 0) reinterpret_cast<float2 *>(lr.part)[j * P + p] = make_float2(acc.hi, acc.lo);
    } else {
        const double acc = block_sum<256>((double)tacc, sh);
        if (threadIdx.x == 0) lr.part[j * P + p] = acc;
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_bt_partial(const T *__restrict__ x, LowRankArg lr) {
    __shared__ double sh[32];
    bt_partial_cta<T>(x, lr, sh, blockIdx.x, blockIdx.y, gridDim.y, true);
}

// One CTA: y_k = sum_p part[k * P + p] (fixed order, so the result does not
// depend on block timing).  With SOLVE it then forms the coefficients z of
// the correction x += C z,
//   z = w - S^{-1} (y + G w) = S^{-1} (Sigma w - y) = S^{-1} (Sigma^{1/2} xi' - y)
// with w = Sigma^{-1/2} xi' the low-rank noise of sor_sampler.cc:29-33,
// G = B^T C and S = Sigma + G (so S - G = Sigma and a single m x m product
// remains); with_noise == 0 gives z = -S^{-1} y, the smoother's correction
// x -= Bbar B^T x of sor_smoother.cc:47-51, Bbar = C S^{-1}.
// One thread per row k: FP64 arithmetic is scarce on this GPU, so every
// FP64 instruction works on 32 different rows (no shuffle trees); S^{-1} is
// stored transposed (SinvT[q * m + k]) so that a warp's loads of one column
// q are contiguous.
// The low-rank solve of one CTA of 256 threads (see k_lr_solve); with
// SOLVE the coefficients z end up in zs (shared, m doubles) and, if
// `publish`, in lr.z / lr.zf.  u and acc are shared scratch of m and 256
// doubles.
template <int NOISE, bool SOLVE>
__device__ __forceinline__ void lr_solve_cta(const LowRankArg &lr, int P, const NoiseArgs &nz, double *u, double *acc,
                                             double *zs, bool publish) {
    const int m = lr.m;
    // rows handled at once and threads per row (blockDim.x = 256)
    const int rows = m < 256 ? m : 256;
    const int tpr = 256 / rows;
    const int g = threadIdx.x / rows, kk = threadIdx.x % rows;
    // m <= 64: each thread's slice of S^{-1} (at most 16 values) is loaded
    // here, while the partial sums below are read, instead of after them
    const int cnt = g < tpr ? (m - g + tpr - 1) / tpr : 0;
    const bool pre = SOLVE && m <= 64;
    double pv[16];
    if (pre) {
#pragma unroll
        for (int i = 0; i < 16; ++i) pv[i] = i < cnt ? __ldg(lr.SinvT + (i64)(g + i * tpr) * m + kk) : 0.0;
    }
    for (int k = threadIdx.x; k < m; k += blockDim.x) {
        double pv[8];
        double t = 0.0;
        for (int q0 = 0; q0 < P; q0 += 8) {
#pragma unroll
            for (int r = 0; r < 8; ++r) pv[r] = q0 + r < P ? __ldcg(lr.part + (i64)k * P + q0 + r) : 0.0;
#pragma unroll
            for (int r = 0; r < 8; ++r)
                if (q0 + r < P) t += pv[r];
        }
        if (publish) lr.y[k] = t;
        if (SOLVE) {
            double xi = 0.0;
            if (NOISE == NOISE_PHILOX) {
                float4 rn = normals4(philox4x32_10(noise_ctr(nz, (unsigned)(k >> 2), PURPOSE_LOWRANK, 0), noise_key(nz)));
                xi = (double)pick(rn, k & 3);
            }
            if (NOISE == NOISE_INJECTED) xi = nz.buf[k];
            u[k] = lr.sigma_sqrt[k] * xi - t;
        }
    }
    if (!SOLVE) return;
    __syncthreads();
    // z = S^{-1} u: thread (g, k) of g < tpr sums the columns q = g, g + tpr, ...
    // of row k (loads of one column contiguous over k), in batches of 8
    // loads issued together; the tpr partial sums are then added in order g.
    if (pre) {  // the same sums from the preloaded slice (one batch of rows: m <= 64)
        double t0 = 0.0, t1 = 0.0;
        if (g < tpr) {
#pragma unroll
            for (int i0 = 0; i0 < 16; i0 += 8) {
                if (i0 + 7 < cnt) {
#pragma unroll
                    for (int r = 0; r < 8; r += 2) {
                        t0 = fma(pv[i0 + r], u[g + (i0 + r) * tpr], t0);
                        t1 = fma(pv[i0 + r + 1], u[g + (i0 + r + 1) * tpr], t1);
                    }
                } else {
#pragma unroll
                    for (int r = 0; r < 8; ++r)
                        if (i0 + r < cnt) t0 = fma(pv[i0 + r], u[g + (i0 + r) * tpr], t0);
                }
            }
            acc[g * rows + kk] = t0 + t1;
        }
        __syncthreads();
        if (threadIdx.x < rows) {
            double zk = 0.0;
            for (int h = 0; h < tpr; ++h) zk += acc[h * rows + threadIdx.x];
            if (zs) zs[threadIdx.x] = zk;
            if (publish) {
                lr.z[threadIdx.x] = zk;
                if (lr.zf) lr.zf[threadIdx.x] = (float)zk;
            }
        }
        __syncthreads();
        return;
    }
    for (int k0 = 0; k0 < m; k0 += rows) {
        const int k = k0 + kk;
        double t0 = 0.0, t1 = 0.0;
        if (g < tpr && k < m) {
            int q = g;
            for (; q + 7 * tpr < m; q += 8 * tpr) {
                double sv[8];
#pragma unroll
                for (int r = 0; r < 8; ++r) sv[r] = __ldg(lr.SinvT + (i64)(q + r * tpr) * m + k);
#pragma unroll
                for (int r = 0; r < 8; r += 2) {
                    t0 = fma(sv[r], u[q + r * tpr], t0);
                    t1 = fma(sv[r + 1], u[q + (r + 1) * tpr], t1);
                }
            }
            for (; q < m; q += tpr) t0 = fma(__ldg(lr.SinvT + (i64)q * m + k), u[q], t0);
            acc[g * rows + kk] = t0 + t1;
        }
        __syncthreads();
        if (threadIdx.x < rows && k0 + threadIdx.x < m) {
            double zk = 0.0;
            for (int h = 0; h < tpr; ++h) zk += acc[h * rows + threadIdx.x];
            if (zs) zs[k0 + threadIdx.x] = zk;
            if (publish) {
                lr.z[k0 + threadIdx.x] = zk;
                if (lr.zf) lr.zf[k0 + threadIdx.x] = (float)zk;
            }
        }
        __syncthreads();
    }
}

// lr_solve_cta for the FP32 chain: the same sums, in the same order and the
// same thread layout, in float-float arithmetic (partial sums as float2
// pairs, S^{-1} and Sigma^{1/2} from their float-float copies).  z goes to
// zsf (shared, m floats, rounded to FP32) and, if `publish`, to lr.z (the
// float-float value in FP64) and lr.zf.  u and acc are shared scratch of m
// and 256 float2.
template <int NOISE, bool SOLVE>
__device__ __forceinline__ void lr_solve_cta_ff(const LowRankArg &lr, int P, const NoiseArgs &nz, float2 *u,
                                                float2 *acc, float *zsf, bool publish) {
    const int m = lr.m;
    const int rows = m < 256 ? m : 256;
    const int tpr = 256 / rows;
    const int g = threadIdx.x / rows, kk = threadIdx.x % rows;
    const int cnt = g < tpr ? (m - g + tpr - 1) / tpr : 0;
    const bool pre = SOLVE && m <= 64;
    const float2 *part = reinterpret_cast<const float2 *>(lr.part);
    float2 pv[16];
    if (pre) {
#pragma unroll
        for (int i = 0; i < 16; ++i)
            pv[i] = i < cnt ? __ldg(lr.SinvT_ff + (i64)(g + i * tpr) * m + kk) : make_float2(0.f, 0.f);
    }
    for (int k = threadIdx.x; k < m; k += blockDim.x) {
        float2 pp[8];
        ff32 t{0.f, 0.f};
        for (int q0 = 0; q0 < P; q0 += 8) {
#pragma unroll
            for (int r = 0; r < 8; ++r) pp[r] = q0 + r < P ? __ldcg(part + (i64)k * P + q0 + r) : make_float2(0.f, 0.f);
#pragma unroll
            for (int r = 0; r < 8; ++r)
                if (q0 + r < P) t = ff_add(t, ff_of(pp[r]));
        }
        if (publish) lr.y[k] = ff_to_double(t);
        if (SOLVE) {
            float xi = 0.f;
            if (NOISE == NOISE_PHILOX) {
                float4 rn = normals4(philox4x32_10(noise_ctr(nz, (unsigned)(k >> 2), PURPOSE_LOWRANK, 0), noise_key(nz)));
                xi = pick(rn, k & 3);
            }
            if (NOISE == NOISE_INJECTED) xi = (float)nz.buf[k];
            const ff32 uk = ff_add(ff_mul(ff_of(lr.sigma_sqrt_ff[k]), ff32{xi, 0.f}), ff_neg(t));
            u[k] = make_float2(uk.hi, uk.lo);
        }
    }
    if (!SOLVE) return;
    __syncthreads();
    auto finish = [&](int k, ff32 zk) {
        if (zsf) zsf[k] = ff_to_float(zk);
        if (publish) {
            lr.z[k] = ff_to_double(zk);
            if (lr.zf) lr.zf[k] = ff_to_float(zk);
        }
    };
    if (pre) {
        ff32 t0{0.f, 0.f}, t1{0.f, 0.f};
        if (g < tpr) {
#pragma unroll
            for (int i = 0; i < 16; i += 2) {
                if (i < cnt) t0 = ff_add(t0, ff_mul(ff_of(pv[i]), ff_of(u[g + i * tpr])));
                if (i + 1 < cnt) t1 = ff_add(t1, ff_mul(ff_of(pv[i + 1]), ff_of(u[g + (i + 1) * tpr])));
            }
            const ff32 s = ff_add(t0, t1);
            acc[g * rows + kk] = make_float2(s.hi, s.lo);
        }
        __syncthreads();
        if (threadIdx.x < rows) {
            ff32 zk{0.f, 0.f};
            for (int h = 0; h < tpr; ++h) zk = ff_add(zk, ff_of(acc[h * rows + threadIdx.x]));
            finish(threadIdx.x, zk);
        }
        __syncthreads();
        return;
    }
    for (int k0 = 0; k0 < m; k0 += rows) {
        const int k = k0 + kk;
        if (g < tpr && k < m) {
            ff32 t0{0.f, 0.f}, t1{0.f, 0.f};
            int q = g;
            for (; q + 7 * tpr < m; q += 8 * tpr) {
                float2 sv[8];
#pragma unroll
                for (int r = 0; r < 8; ++r) sv[r] = __ldg(lr.SinvT_ff + (i64)(q + r * tpr) * m + k);
#pragma unroll
                for (int r = 0; r < 8; r += 2) {
                    t0 = ff_add(t0, ff_mul(ff_of(sv[r]), ff_of(u[q + r * tpr])));
                    t1 = ff_add(t1, ff_mul(ff_of(sv[r + 1]), ff_of(u[q + (r + 1) * tpr])));
                }
            }
            for (; q < m; q += tpr) t0 = ff_add(t0, ff_mul(ff_of(__ldg(lr.SinvT_ff + (i64)q * m + k)), ff_of(u[q])));
            const ff32 s = ff_add(t0, t1);
            acc[g * rows + kk] = make_float2(s.hi, s.lo);
        }
        __syncthreads();
        if (threadIdx.x < rows && k0 + threadIdx.x < m) {
            ff32 zk{0.f, 0.f};
            for (int h = 0; h < tpr; ++h) zk = ff_add(zk, ff_of(acc[h * rows + threadIdx.x]));
            finish(k0 + threadIdx.x, zk);
        }
        __syncthreads();
    }
}

// The low-rank solve of a chain in precision T: FP64 for the FP64 chain,
// float-float for the FP32 chain (its partial sums are float-float pairs).
// u and acc: shared scratch of m and 256 doubles; z goes to zs (m doubles of
// shared memory, holding m floats for the FP32 chain) unless it is null.
template <typename T, int NOISE, bool SOLVE>
__device__ __forceinline__ void lr_solve_chain(const LowRankArg &lr, int P, const NoiseArgs &nz, double *u,
                                               double *acc, double *zs, bool publish) {
    if (sizeof(T) == 4)
        lr_solve_cta_ff<NOISE, SOLVE>(lr, P, nz, reinterpret_cast<float2 *>(u), reinterpret_cast<float2 *>(acc),
                                      reinterpret_cast<float *>(zs), publish);
    else
        lr_solve_cta<NOISE, SOLVE>(lr, P, nz, u, acc, zs, publish);
}

template <typename T, int NOISE, bool SOLVE>
__global__ void __launch_bounds__(256) k_lr_solve(LowRankArg lr, int P, NoiseArgs nz) {
    pdl_begin();
    extern __shared__ double dyn[];
    lr_solve_chain<T, NOISE, SOLVE>(lr, P, nz, dyn, dyn + lr.m, nullptr, true);
}

// Partial sums and the solve in one launch: the last CTA to finish (block
// counter, reset by that CTA) forms y -- and with SOLVE z -- from the
// partial sums in the same fixed order as k_lr_solve, so the result does
// not depend on block timing.  The thread that wrote the CTA's partial sum
// counts it with an acquire-release atomic, which orders that write before
// the count and, in the last CTA, the other CTAs' sums before the barrier
// after which its threads read them.
template <typename T, int NOISE, bool SOLVE>
__device__ __forceinline__ void bt_solve_body(const T *__restrict__ x, const LowRankArg &lr, const NoiseArgs &nz, int j,
                                              int p, int P, bool wait = false) {
    __shared__ double sh[32];
    __shared__ bool last;
    bt_partial_cta<T>(x, lr, sh, j, p, P, wait);
    if (threadIdx.x == 0) {
        // one acquire-release count at GPU scope: it publishes this CTA's
        // partial sum (written by this thread) and, in the last CTA, makes
        // every other CTA's visible before the barrier below
        unsigned prev;
        asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(prev) : "l"(lr.counter) : "memory");
        last = prev == (unsigned)(lr.m * P) - 1u;
        if (last) *lr.counter = 0u;
    }
    __syncthreads();
    if (!last) return;
    // every other CTA has exited: the next kernel (the correction) can load
    // its rows of C while this CTA forms z
    pdl_trigger();
    extern __shared__ double dyn[];
    lr_solve_chain<T, NOISE, SOLVE>(lr, P, nz, dyn, dyn + lr.m, nullptr, true);
}

template <typename T, int NOISE, bool SOLVE>
__global__ void __launch_bounds__(256) k_bt_solve(const T *__restrict__ x, LowRankArg lr, NoiseArgs nz) {
    bt_solve_body<T, NOISE, SOLVE>(x, lr, nz, blockIdx.x, blockIdx.y, gridDim.y, true);
}

// Support rows of C = M^{-1} B as x += C z reads them: the rows with one
// entry -- nearly all, since the measurement balls rarely overlap -- as
// (row, column, value) triples, the others in CSR form.  Padded row indices
// are 32-bit (levels of fewer than 2^32 padded points).
struct CorrRows {
    i64 n1 = 0, nm = 0;            // rows with one entry / with several
    const unsigned *r1 = nullptr;  // n1 padded row indices
    const int *c1 = nullptr;       // their columns
    const void *v1 = nullptr;      // their values (type T)
    const unsigned *rm = nullptr;  // nm padded row indices
    const int *pm = nullptr;       // nm + 1 offsets into cm / vm
    const int *cm = nullptr;
    const void *vm = nullptr;
};

// x[row] += C z over the multi-entry row r: the products added to zero in
// entry order, then to the state
template <typename T, typename ZT>
__device__ __forceinline__ void corr_multi_row(T *__restrict__ x, const CorrRows &C, i64 r, const ZT *z) {
    const T *vm = static_cast<const T *>(C.vm);
    T acc = T(0);
    for (int e = C.pm[r]; e < C.pm[r + 1]; ++e) acc += vm[e] * (T)z[C.cm[e]];
    const unsigned row = C.rm[r];
    x[row] = x[row] + acc;
}

// Four single-entry rows of a thread, r0 + j stride (j < 4): row index,
// column, value and state loaded together; the update is the multi-entry
// arithmetic with one product.  The state of rows loaded before the wait
// for the previous kernel is read through L2 (see k_lr_scatter).
template <typename T>
struct CorrQuad {
    unsigned row[4];
    int col[4];
    T val[4], xv[4];
    __device__ __forceinline__ void load(const T *__restrict__ x, const CorrRows &C, i64 r0, i64 stride,
                                         bool before_wait) {
        const T *v1 = static_cast<const T *>(C.v1);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const i64 r = r0 + j * stride;
            const bool ok = r < C.n1;
            row[j] = ok ? C.r1[r] : 0u;
            col[j] = ok ? C.c1[r] : 0;
            val[j] = ok ? v1[r] : T(0);
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
            xv[j] = r0 + j * stride < C.n1 ? (before_wait ? __ldcg(x + row[j]) : x[row[j]]) : T(0);
    }
    template <typename ZT>
    __device__ __forceinline__ void apply(T *__restrict__ x, const CorrRows &C, i64 r0, i64 stride,
                                          const ZT *z) const {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (r0 + j * stride >= C.n1) continue;
            T acc = T(0);
            acc += val[j] * (T)z[col[j]];
            x[row[j]] = xv[j] + acc;
        }
    }
};

// One multi-entry row r (two entries at least) with its row index, entry
// range, first two entries and state loaded together, before the wait for
// the previous kernel where the caller says so; the update is
// corr_multi_row's arithmetic.
template <typename T>
struct CorrMulti {
    unsigned row;
    int e0, e1, col0, col1;
    T val0, val1, xv;
    __device__ __forceinline__ void load(const T *__restrict__ x, const CorrRows &C, i64 r, bool before_wait) {
        const T *vm = static_cast<const T *>(C.vm);
        row = C.rm[r];
        e0 = C.pm[r];
        e1 = C.pm[r + 1];
        col0 = C.cm[e0];
        col1 = C.cm[e0 + 1];
        val0 = vm[e0];
        val1 = vm[e0 + 1];
        xv = before_wait ? __ldcg(x + row) : x[row];
    }
    template <typename ZT>
    __device__ __forceinline__ void apply(T *__restrict__ x, const CorrRows &C, const ZT *z) const {
        const T *vm = static_cast<const T *>(C.vm);
        T acc = T(0);
        acc += val0 * (T)z[col0];
        acc += val1 * (T)z[col1];
        for (int e = e0 + 2; e < e1; ++e) acc += vm[e] * (T)z[C.cm[e]];
        x[row] = xv + acc;
    }
};

// Low-rank solve and correction in one launch: every CTA forms z itself
// (the same arithmetic in the same order in every CTA, so all agree) and
// adds C z on its share of the support rows of C = M^{-1} B, four rows per
// thread and iteration with their loads issued together.  A thread's first
// four rows do not depend on the partial sums the kernel before writes, so
// they are loaded before the wait.
template <typename T, int NOISE>
__global__ void __launch_bounds__(256) k_lr_apply(T *__restrict__ x, LowRankArg lr, int P, NoiseArgs nz, CorrRows C) {
    const i64 stride = (i64)gridDim.x * blockDim.x;
    const i64 t0 = (i64)blockIdx.x * blockDim.x + threadIdx.x;
    CorrQuad<T> q;
    CorrMulti<T> mr;
    if (t0 < C.n1) q.load(x, C, t0, stride, true);
    if (t0 < C.nm) mr.load(x, C, t0, true);
    pdl_begin();
    extern __shared__ double dyn[];
    const int m = lr.m;
    lr_solve_chain<T, NOISE, true>(lr, P, nz, dyn + m, dyn + 2 * m, dyn, blockIdx.x == 0);
    // z (m values of type T at the start of dyn) is complete after the last
    // __syncthreads of the solve
    const T *zs = reinterpret_cast<const T *>(dyn);
    for (i64 r0 = t0; r0 < C.n1; r0 += 4 * stride) {
        q.apply(x, C, r0, stride, zs);
        if (r0 + 4 * stride < C.n1) q.load(x, C, r0 + 4 * stride, stride, false);
    }
    for (i64 r = t0; r < C.nm; r += stride) {
        if (r != t0) mr.load(x, C, r, false);
        mr.apply(x, C, zs);
    }
}

// x[row] += sum_e C_e z_{col_e} over the support rows of C = M^{-1} B, with
// the coefficients z of k_lr_solve (ZT = float: the FP32 chain's rounded
// copy), four rows per thread and iteration with their loads issued together.
// Only z comes from the kernel just before (k_bt_solve); the row indices,
// columns, values and the state of a thread's first four rows do not, so
// they are loaded before the wait for that kernel.  The state was written by
// a kernel before k_bt_solve, which had completed when every CTA of
// k_bt_solve passed its own wait, i.e. before this grid started; it is read
// through L2 (ld.global.cg), the level at which those writes are visible.
template <typename T, typename ZT>
__global__ void __launch_bounds__(256) k_lr_scatter(T *__restrict__ x, CorrRows C, const ZT *__restrict__ z) {
    const i64 stride = (i64)gridDim.x * blockDim.x;
    const i64 t0 = (i64)blockIdx.x * blockDim.x + threadIdx.x;
    CorrQuad<T> q;
    CorrMulti<T> mr;
    if (t0 < C.n1) q.load(x, C, t0, stride, true);
    if (t0 < C.nm) mr.load(x, C, t0, true);
    pdl_begin();
    for (i64 r0 = t0; r0 < C.n1; r0 += 4 * stride) {
        q.apply(x, C, r0, stride, z);
        if (r0 + 4 * stride < C.n1) q.load(x, C, r0 + 4 * stride, stride, false);
    }
    for (i64 r = t0; r < C.nm; r += stride) {
        if (r != t0) mr.load(x, C, r, false);
        mr.apply(x, C, z);
    }
}

// ------------------------------------------------- residual + restriction
// f_c(P_c) = sum_{a in {-1,0,1}^d} r(a) (f - A_0 x)(2 i_c + a),
// r(a) = prod {1/2, 1, 1/2}: IntergridOperator::restrict
// (intergrid_operator.hh:74-88) of the residual f - A_0 x
// (multigridmc_sampler.cc:124-126), with the stencil part of A.
template <typename T, int NPT, int VAR = 0>
__global__ void __launch_bounds__(256) k_resid_restrict(const T *__restrict__ x, const T *__restrict__ f,
                                                         T *__restrict__ fc, T *__restrict__ xc, Grid3 gf, Grid3 gc, StencilArg<T> s,
                                                         int dim, VarField<T> vf) {
    if (gf.pdl) pdl_begin();
    i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
    i64 nc = (i64)gc.N0 * gc.N1 * gc.N2;
    if (t >= nc) return;
    int a = (int)(t % gc.N0), b = (int)((t / gc.N0) % gc.N1), c = (int)(t / ((i64)gc.N0 * gc.N1));
    // fine 0-based coordinates of the centre 2 (a+1) - 1
    int fa = 2 * a + 1, fb = dim > 1 ? 2 * b + 1 : 0, fc_ = dim > 2 ? 2 * c + 1 : 0;
    const int zlo = dim > 2 ? -1 : 0, ylo = dim > 1 ? -1 : 0;
    T acc = T(0);
    for (int az = zlo; az <= -zlo; ++az)
        for (int ay = ylo; ay <= -ylo; ++ay)
            for (int ax = -1; ax <= 1; ++ax) {
                T wr = T((ax ? 0.5 : 1.0) * (ay ? 0.5 : 1.0) * (az ? 0.5 : 1.0));
                i64 P = gf.pad(fa + ax, fb + ay, fc_ + az);
                T res = T(0);
                if (VAR) {
                    res = stencil_row<T, NPT, false, VAR>(x, gf, s, P, vf);
                } else if (NPT == 7) {
                    res = s.w[4] * x[P - gf.sz] + s.w[10] * x[P - gf.sy] + s.w[12] * x[P - 1] + s.w[13] * x[P] +
                          s.w[14] * x[P + 1] + s.w[16] * x[P + gf.sy] + s.w[22] * x[P + gf.sz];
                } else {
#pragma unroll
                    for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
                        for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
                            for (int dx = -1; dx <= 1; ++dx)
                                res += s.w[(dz + 1) * 9 + (dy + 1) * 3 + (dx + 1)] * x[P + dz * gf.sz + dy * gf.sy + dx];
                }
                acc += wr * (f[P] - res);
            }
    fc[gc.pad(a, b, c)] = acc;
    if (xc) xc[gc.pad(a, b, c)] = T(0);  // the coarse sample starts from zero
}

// 3D-tiled variant: a CTA owns RR_TX x RR_TY x RR_TZ coarse points.  It
// stages the x values of the tile's fine footprint plus a one-point halo in
// shared memory (all loads issued at once), computes each fine residual of
// the footprint once and restricts.
constexpr int RR_TX = 16, RR_TY = 4, RR_TZ = 4;
constexpr int RR_FW = 2 * RR_TX + 1, RR_FH = 2 * RR_TY + 1, RR_FD = 2 * RR_TZ + 1;  // residual footprint, 33 x 9 x 9
constexpr int RR_XW = RR_FW + 2, RR_XH = RR_FH + 2, RR_XD = RR_FD + 2;             // x with halo
constexpr int RR_THREADS = 320;  // >= RR_FW * RR_FH = 297 footprint columns and RR_TX * RR_TY * RR_TZ = 256 coarse points
constexpr int RR_RZ = RR_TZ * RR_FH * RR_FW;  // z-restricted residuals of a tile

// The arithmetic of one tile, x (footprint plus halo) in shared memory with
// row pitch XP (footprint point (la, lb, lc) at ((lc + 1) RR_XH + lb + 1) XP
// + la + 1), f through fv(la, lb, lc).  Thread t < 297 takes the column
// (la, lb) of the footprint -- warp lb the first 32 columns of row lb, so
// that a warp's shared-memory loads are one contiguous run (no bank
// conflicts), and the tenth warp the last column of every row: the 9
// residuals along z stay in registers (the x loads of a 7-point column slide
// along z) and are restricted in z, r_z = r(2 cz) / 2 + r(2 cz + 1) +
// r(2 cz + 2) / 2, into rz.  Then thread t < 256 takes one coarse point: the
// 3 x 3 in-plane taps of rz with the weights (1/2, 1, 1/2) in y and x.  The
// product of those weights is the trilinear restriction of
// intergrid_operator.hh:74-88.
template <typename T, int NPT, int XP, typename FV>
__device__ __forceinline__ void rr_tile_compute(const T *xs, const FV &fv, T *rz, T *__restrict__ fc,
                                                T *__restrict__ xc, const Grid3 &gf, const Grid3 &gc,
                                                const StencilArg<T> &s, int ca0, int cb0, int cc0) {
    constexpr int SY = XP, SZ = XP * RR_XH;
    const int fa0 = 2 * ca0, fb0 = 2 * cb0, fz0 = 2 * cc0;
    constexpr int RW = RR_FW - 1;  // 32 columns of a row per warp
    for (int t = threadIdx.x; t < RR_FW * RR_FH; t += blockDim.x) {
        const int lb = t < RW * RR_FH ? t / RW : t - RW * RR_FH;
        const int la = t < RW * RR_FH ? t - lb * RW : RW;
        const bool col_in = fa0 + la < gf.N0 && fb0 + lb < gf.N1;
        const T *xq = xs + (lb + 1) * SY + (la + 1);
        // r_z(cz) = (r(2 cz) / 2 + r(2 cz + 1)) + r(2 cz + 2) / 2, formed as
        // the residuals come, so that only two of them are live at a time
        T rprev = T(0), part = T(0);
#pragma unroll
        for (int lc = 0; lc < RR_FD; ++lc) {
            T v = T(0);
            if (col_in && fz0 + lc < gf.N2) {
                const int q = (lc + 1) * SZ;
                T res;
                if (NPT == 7) {
                    res = s.w[4] * xq[q - SZ] + s.w[10] * xq[q - SY] + s.w[12] * xq[q - 1] + s.w[13] * xq[q] +
                          s.w[14] * xq[q + 1] + s.w[16] * xq[q + SY] + s.w[22] * xq[q + SZ];
                } else {
                    res = T(0);
#pragma unroll
                    for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
                        for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
                            for (int dx = -1; dx <= 1; ++dx)
                                res += s.w[(dz + 1) * 9 + (dy + 1) * 3 + (dx + 1)] * xq[q + dz * SZ + dy * SY + dx];
                }
                v = fv(la, lb, lc) - res;
            }
            if (lc & 1) {
                part = T(0.5) * rprev + v;
            } else {
                if (lc > 0) rz[((lc / 2 - 1) * RR_FH + lb) * RR_FW + la] = part + T(0.5) * v;
                rprev = v;
            }
        }
    }
    __syncthreads();
    if (threadIdx.x >= RR_TX * RR_TY * RR_TZ) return;
    const int la = threadIdx.x % RR_TX, lb = (threadIdx.x / RR_TX) % RR_TY, lc = threadIdx.x / (RR_TX * RR_TY);
    const int ca = ca0 + la, cb = cb0 + lb, cc = cc0 + lc;
    if (ca >= gc.N0 || cb >= gc.N1 || cc >= gc.N2) return;
    T acc = T(0);
#pragma unroll
    for (int ay = 0; ay < 3; ++ay)
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            const T wr = T((ax == 1 ? 1.0 : 0.5) * (ay == 1 ? 1.0 : 0.5));
            acc += wr * rz[(lc * RR_FH + 2 * lb + ay) * RR_FW + 2 * la + ax];
        }
    fc[gc.pad(ca, cb, cc)] = acc;
    if (xc) xc[gc.pad(ca, cb, cc)] = T(0);  // the coarse sample starts from zero
}

template <typename T>
constexpr size_t rr_smem_bytes() {
    return sizeof(T) * (RR_XW * RR_XH * RR_XD + RR_RZ);
}

template <typename T, int NPT>
__device__ __forceinline__ void resid_restrict_tiled_body(const T *__restrict__ x, const T *__restrict__ f,
                                                          T *__restrict__ fc, T *__restrict__ xc, const Grid3 &gf,
                                                          const Grid3 &gc, const StencilArg<T> &s, unsigned char *smem,
                                                          int bx, int by, int bz) {
    T *xs = reinterpret_cast<T *>(smem);  // [RR_XD][RR_XH][RR_XW]
    T *rz = xs + RR_XW * RR_XH * RR_XD;   // [RR_TZ][RR_FH][RR_FW]
    const int ca0 = bx * RR_TX, cb0 = by * RR_TY, cc0 = bz * RR_TZ;
    // fine 0-based origin of the footprint: the centre of coarse ca0 is fine
    // 2 ca0 + 1, its lower neighbour 2 ca0
    const int fa0 = 2 * ca0, fb0 = 2 * cb0, fz0 = 2 * cc0;
    // one warp per row of the box (no index divisions per element; a row is
    // one contiguous run of x)
    const int lane = threadIdx.x & 31;
    for (int row = threadIdx.x >> 5; row < RR_XH * RR_XD; row += RR_THREADS / 32) {
        const int lb = row % RR_XH, lc = row / RR_XH;
        const int gb = fb0 - 1 + lb, gz = fz0 - 1 + lc;
        const bool rin = gb >= 0 && gb < gf.N1 && gz >= 0 && gz < gf.N2;
        const T *xr = x + (rin ? gf.pad(fa0 - 1, gb, gz) : 0);
        for (int la = lane; la < RR_XW; la += 32) {
            const int ga = fa0 - 1 + la;
            xs[row * RR_XW + la] = rin && ga >= 0 && ga < gf.N0 ? xr[la] : T(0);
        }
    }
    __syncthreads();
    rr_tile_compute<T, NPT, RR_XW>(
        xs, [&](int la, int lb, int lc) { return f[gf.pad(fa0 + la, fb0 + lb, fz0 + lc)]; }, rz, fc, xc, gf, gc, s,
        ca0, cb0, cc0);
}

template <typename T, int NPT>
__global__ void __launch_bounds__(RR_THREADS) k_resid_restrict_tiled(const T *__restrict__ x, const T *__restrict__ f,
                                                                      T *__restrict__ fc, T *__restrict__ xc, Grid3 gf, Grid3 gc,
                                                                      StencilArg<T> s) {
    if (gf.pdl) pdl_begin();
    extern __shared__ __align__(16) unsigned char rr_smem[];
    resid_restrict_tiled_body<T, NPT>(x, f, fc, xc, gf, gc, s, rr_smem, blockIdx.x, blockIdx.y, blockIdx.z);
}

// ---------------------------------------------- bulk tensor copies (TMA)
__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// 3D tiled copy of the tensor map's box at element coordinates (x, y, z)
// into shared memory; completion is counted on `bar` in bytes.
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z,
                                            unsigned long long *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<u64>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ u64 global_ns() {
    u64 t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Wait for phase `parity` of `bar`, giving up after limit_ns nanoseconds.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, unsigned parity, u64 limit_ns) {
    const u64 t0 = global_ns();
    while (!mbar_try_wait(bar, parity))
        if (global_ns() - t0 > limit_ns) return false;
    return true;
}

constexpr u64 TILE_WAIT_NS = 200000000ull;  // 0.2 s: a tile copy that has not landed by then is reported
constexpr unsigned ERR_TILE_TIMEOUT = 2u;    // error bit: a tile copy wait ran out

// TMA variant of the residual-restriction (rows of x and f that are
// multiples of 16 bytes): thread 0 issues two 3D bulk tensor copies of the
// padded arrays -- x over the footprint plus a one-point halo, f over the
// footprint -- with rows widened to RR_BW elements (the copy's x coordinate
// 2 * 16 * blockIdx.x stays 16-byte aligned); points outside the arrays read
// as zero, like the ghost layer.  Then rr_tile_compute.
constexpr int RR_BW = 36;

template <typename T>
__host__ __device__ constexpr size_t rr_tma_xbytes() {
    return (sizeof(T) * RR_BW * RR_XH * RR_XD + 127) / 128 * 128;
}
template <typename T>
__host__ __device__ constexpr size_t rr_tma_fbytes() {
    return (sizeof(T) * RR_BW * RR_FH * RR_FD + 15) / 16 * 16;
}
template <typename T>
__host__ __device__ constexpr size_t rr_tma_smem_bytes() {
    return rr_tma_xbytes<T>() + rr_tma_fbytes<T>() + sizeof(T) * RR_RZ;
}

// The arithmetic of one tile once its x and f boxes are in shared memory
// (rr_tile_compute; the f box's footprint point (la, lb, lc) at
// (lc RR_FH + lb) RR_BW + la + 1).
template <typename T, int NPT>
__device__ __forceinline__ void resid_restrict_tile(const T *xs, const T *fs, T *rz, T *__restrict__ fc,
                                                    T *__restrict__ xc, const Grid3 &gf, const Grid3 &gc,
                                                    const StencilArg<T> &s, int ca0, int cb0, int cc0) {
    rr_tile_compute<T, NPT, RR_BW>(
        xs, [&](int la, int lb, int lc) { return fs[(lc * RR_FH + lb) * RR_BW + la + 1]; }, rz, fc, xc, gf, gc, s,
        ca0, cb0, cc0);
}

template <typename T, int NPT>
__global__ void __launch_bounds__(RR_THREADS) k_resid_restrict_tma(const __grid_constant__ CUtensorMap xmap,
                                                                   const __grid_constant__ CUtensorMap fmap,
                                                                   T *__restrict__ fc, T *__restrict__ xc, Grid3 gf, Grid3 gc,
                                                                   StencilArg<T> s, unsigned *__restrict__ err) {
    if (gf.pdl) pdl_begin();
    extern __shared__ __align__(1024) unsigned char rr_tma_smem[];
    __shared__ unsigned long long bar;
    T *xs = reinterpret_cast<T *>(rr_tma_smem);                      // [RR_XD][RR_XH][RR_BW]
    T *fs = reinterpret_cast<T *>(rr_tma_smem + rr_tma_xbytes<T>()); // [RR_FD][RR_FH][RR_BW]
    T *rz = reinterpret_cast<T *>(rr_tma_smem + rr_tma_xbytes<T>() + rr_tma_fbytes<T>());
    const int ca0 = blockIdx.x * RR_TX, cb0 = blockIdx.y * RR_TY, cc0 = blockIdx.z * RR_TZ;
    const int fa0 = 2 * ca0, fb0 = 2 * cb0, fz0 = 2 * cc0;
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_expect_tx(&bar, (unsigned)(sizeof(T) * RR_BW * (RR_XH * RR_XD + RR_FH * RR_FD)));
        // padded coordinates: fine vertex a sits at a + 1
        tma_load_3d(xs, &xmap, fa0, fb0, fz0, &bar);         // fine (fa0-1, fb0-1, fz0-1) ...
        tma_load_3d(fs, &fmap, fa0, fb0 + 1, fz0 + 1, &bar); // fine (fa0-1, fb0, fz0) ...
    }
    const bool ok = mbar_wait_bounded(&bar, 0, TILE_WAIT_NS);
    if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) atomicOr(err, ERR_TILE_TIMEOUT);
        mbar_wait_bounded(&bar, 0, TILE_WAIT_NS);  // let copies in flight land before the CTA exits
        return;
    }
    resid_restrict_tile<T, NPT>(xs, fs, rz, fc, xc, gf, gc, s, ca0, cb0, cc0);
}

// dst[row] += sign * sum_e B_e y_{col_e} / Sigma_{col_e} over the rows of B
// (row-compressed): the B Sigma^{-1} B^T x part of A x.
template <typename T>
__global__ void __launch_bounds__(256) k_add_Bq(T *__restrict__ dst, i64 nrows, const i64 *__restrict__ rows,
                                                 const i64 *__restrict__ ptr, const int *__restrict__ col,
                                                 const double *__restrict__ val, const double *__restrict__ y,
                                                 const double *__restrict__ sigma_inv, double sign) {
    pdl_begin();
    for (i64 r = (i64)blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += (i64)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (i64 e = ptr[r]; e < ptr[r + 1]; ++e) acc += val[e] * (y[col[e]] * sigma_inv[col[e]]);
        dst[rows[r]] += (T)(sign * acc);
    }
}

// --------------------------------------------------------- prolongation
// x += alpha P x_c (intergrid_operator.hh:106-120): every fine vertex
// gathers its <= 2^d coarse parents, weight 1 (even coordinate) or 1/2 for
// each of the two parents (odd coordinate).
template <typename T>
__device__ __forceinline__ void prolong_add_body(T *__restrict__ x, const T *__restrict__ xc, const Grid3 &gf,
                                                 const Grid3 &gc, T alpha, int dim, int bx, int by, int bz_from_top) {
    // coarse cell (i, j, k), 0 <= i <= Nc0 etc., owns the fine vertices with
    // 1-based coordinates 2 i + {0, 1} (those inside the interior); its
    // corners are the coarse vertices i, i+1 (1-based, ghosts are zero)
    // planes from the top: the residual-restriction before ends there, and
    // the sweep after starts at the bottom, which this kernel writes last
    // (both find their first planes in L2)
    const int i = bx * blockDim.x + threadIdx.x;
    const int j = dim > 1 ? by : 0, k = dim > 2 ? bz_from_top : 0;
    if (i > gc.N0) return;
    const int ny = dim > 1 ? 2 : 1, nz = dim > 2 ? 2 : 1;
    T cv[2][2][2];
#pragma unroll
    for (int dz = 0; dz < 2; ++dz)
#pragma unroll
        for (int dy = 0; dy < 2; ++dy)
#pragma unroll
            for (int dx = 0; dx < 2; ++dx) {
                const int ci = i + dx, cj = dim > 1 ? j + dy : 1, ck = dim > 2 ? k + dz : 1;
                const bool use = (dy < ny) && (dz < nz);
                cv[dz][dy][dx] = use ? xc[(i64)ck * gc.sz + (i64)cj * gc.sy + ci] : T(0);
            }
#pragma unroll
    for (int oz = 0; oz < 2; ++oz) {
        if (oz >= nz) break;
        const int fk = dim > 2 ? 2 * k + oz : 1;
        if (fk < 1 || fk > gf.N2) continue;
#pragma unroll
        for (int oy = 0; oy < 2; ++oy) {
            if (oy >= ny) break;
            const int fj = dim > 1 ? 2 * j + oy : 1;
            if (fj < 1 || fj > gf.N1) continue;
#pragma unroll
            for (int ox = 0; ox < 2; ++ox) {
                const int fi = 2 * i + ox;
                if (fi < 1 || fi > gf.N0) continue;
                // even coordinate: the vertex itself (weight 1); odd: half
                // of each neighbour
                T acc = T(0);
#pragma unroll
                for (int dz = 0; dz < 2; ++dz) {
                    const T wz = dim > 2 ? (oz == 0 ? (dz == 0 ? T(1) : T(0)) : T(0.5)) : (dz == 0 ? T(1) : T(0));
                    if (wz == T(0)) continue;
#pragma unroll
                    for (int dy = 0; dy < 2; ++dy) {
                        const T wy = dim > 1 ? (oy == 0 ? (dy == 0 ? T(1) : T(0)) : T(0.5)) : (dy == 0 ? T(1) : T(0));
                        if (wy == T(0)) continue;
#pragma unroll
                        for (int dx = 0; dx < 2; ++dx) {
                            const T wx = ox == 0 ? (dx == 0 ? T(1) : T(0)) : T(0.5);
                            if (wx == T(0)) continue;
                            acc += wx * wy * wz * cv[dz][dy][dx];
                        }
                    }
                }
                const i64 P = (i64)fk * gf.sz + (i64)fj * gf.sy + fi;
                x[P] += alpha * acc;
            }
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(128) k_prolong_add(T *__restrict__ x, const T *__restrict__ xc, Grid3 gf, Grid3 gc,
                                                      T alpha, int dim) {
    if (gf.pdl) pdl_begin();
    prolong_add_body<T>(x, xc, gf, gc, alpha, dim, blockIdx.x, blockIdx.y, (int)(gridDim.z - 1 - blockIdx.z));
}

// ----------------------------------------------------- stencil apply
// y = A_0 x (LinearOperator::apply without the low-rank term).
template <typename T, int VAR = 0>
__global__ void __launch_bounds__(256) k_apply_stencil(const T *__restrict__ x, T *__restrict__ y, Grid3 g,
                                                        StencilArg<T> s, VarField<T> vf) {
    if (g.pdl) pdl_begin();
    i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
    i64 n = (i64)g.N0 * g.N1 * g.N2;
    if (t >= n) return;
    int a = (int)(t % g.N0), b = (int)((t / g.N0) % g.N1), c = (int)(t / ((i64)g.N0 * g.N1));
    i64 P = g.pad(a, b, c);
    T res = T(0);
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx)
                res += vweight<T, VAR>(s, vf, P, (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1)) * x[P + dz * g.sz + dy * g.sy + dx];
    y[P] = res;
}

// ---------------------------------------------------- layout conversion
template <typename T>
__global__ void __launch_bounds__(256) k_unpack(const double *__restrict__ src, T *__restrict__ dst, Grid3 g) {
    if (g.pdl) pdl_begin();
    const int a = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y, c = blockIdx.z;
    if (a >= g.N0) return;
    dst[g.pad(a, b, c)] = (T)src[((i64)c * g.N1 + b) * g.N0 + a];
}

// Both inputs of Sampler::apply in one pass (two independent read streams
// per thread).
template <typename T>
__global__ void __launch_bounds__(256) k_unpack2(const double *__restrict__ f_src, const double *__restrict__ x_src,
                                                 T *__restrict__ f_dst, T *__restrict__ x_dst, Grid3 g) {
    if (g.pdl) pdl_begin();
    const int a = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y, c = blockIdx.z;
    if (a >= g.N0) return;
    const i64 i = ((i64)c * g.N1 + b) * g.N0 + a, P = g.pad(a, b, c);
    const double fv = f_src[i], xv = x_src[i];
    f_dst[P] = (T)fv;
    x_dst[P] = (T)xv;
}

template <typename T>
__global__ void __launch_bounds__(256) k_pack(const T *__restrict__ src, double *__restrict__ dst, Grid3 g) {
    if (g.pdl) pdl_begin();
    const int a = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y, c = blockIdx.z;
    if (a >= g.N0) return;
    dst[((i64)c * g.N1 + b) * g.N0 + a] = (double)src[g.pad(a, b, c)];
}

// ------------------------------------------------- coarse Cholesky sample
// CholeskySampler::apply (cholesky_sampler.hh:52-66) with the dense
// natural-order factor Q = L L^T: g = L^{-1} f, x = L^{-T} (xi + g).
// Parity form: column-oriented substitution in one CTA (same operation
// order as the oracle, one rounding per operation).
template <typename T, int NOISE>
__global__ void __launch_bounds__(1024) k_chol_subst(const T *__restrict__ f, T *__restrict__ x, Grid3 g,
                                                      const double *__restrict__ L, double *__restrict__ gv,
                                                      NoiseArgs nz) {
    if (g.pdl) pdl_begin();
    const i64 n = (i64)g.N0 * g.N1 * g.N2;
    for (i64 i = threadIdx.x; i < n; i += blockDim.x) {
        int a = (int)(i % g.N0), b = (int)((i / g.N0) % g.N1), c = (int)(i / ((i64)g.N0 * g.N1));
        gv[i] = (double)f[g.pad(a, b, c)];
    }
    __syncthreads();
    __shared__ double piv;
    for (i64 i = 0; i < n; ++i) {  // forward: L g = f
        if (threadIdx.x == 0) {
            piv = gv[i] / L[i * n + i];
            gv[i] = piv;
        }
        __syncthreads();
        const double p = piv;
        for (i64 k = i + 1 + threadIdx.x; k < n; k += blockDim.x) gv[k] = __dsub_rn(gv[k], __dmul_rn(L[k * n + i], p));
        __syncthreads();
    }
    for (i64 i = threadIdx.x; i < n; i += blockDim.x) {  // xi + g
        double xi = 0.0;
        if (NOISE == NOISE_INJECTED) xi = nz.buf[i];
        if (NOISE == NOISE_PHILOX) {
            float4 r = normals4(philox4x32_10(noise_ctr(nz, (unsigned)(i >> 2), PURPOSE_COARSE, 0), noise_key(nz)));
            xi = (double)pick(r, (int)(i & 3));
        }
        gv[i] = __dadd_rn(xi, gv[i]);
    }
    __syncthreads();
    for (i64 i = n - 1; i >= 0; --i) {  // backward: L^T x = xi + g
        if (threadIdx.x == 0) {
            piv = gv[i] / L[i * n + i];
            gv[i] = piv;
        }
        __syncthreads();
        const double p = piv;
        for (i64 k = threadIdx.x; k < i; k += blockDim.x) gv[k] = __dsub_rn(gv[k], __dmul_rn(L[i * n + k], p));
        __syncthreads();
    }
    for (i64 i = threadIdx.x; i < n; i += blockDim.x) {
        int a = (int)(i % g.N0), b = (int)((i / g.N0) % g.N1), c = (int)(i / ((i64)g.N0 * g.N1));
        x[g.pad(a, b, c)] = (T)gv[i];
    }
}

// Throughput form with the explicit inverse factor Linv = L^{-1}, stored
// row-major in the matrix type MT (double for the FP64 chain, float for the
// FP32 chain) with a leading dimension ld that is a multiple of 16 bytes and
// explicit zeros outside the triangle (and in columns n..ld-1), so that rows
// are read in aligned 16-byte vectors and a vector that straddles the
// diagonal multiplies zeros.  One warp per row; rows i and n-1-i go to
// neighbouring warps, so that every CTA gets the same number of non-zeros.
template <typename MT>
struct Vec16;
template <>
struct Vec16<float> {
    typedef float4 type;
    static constexpr int N = 4;
    static __device__ __forceinline__ float dot(float4 a, const float *v) {
        return a.x * v[0] + a.y * v[1] + a.z * v[2] + a.w * v[3];
    }
};
template <>
struct Vec16<double> {
    typedef double2 type;
    static constexpr int N = 2;
    static __device__ __forceinline__ double dot(double2 a, const double *v) { return a.x * v[0] + a.y * v[1]; }
};

// sum over vectors q0..q1-1 of row . vs, lanes strided, four vectors in flight
template <typename MT>
__device__ __forceinline__ MT warp_row_dot(const MT *__restrict__ row, const MT *vs, int q0, int q1, int lane) {
    typedef typename Vec16<MT>::type V;
    constexpr int NV = Vec16<MT>::N;
    const V *r = reinterpret_cast<const V *>(row);
    MT a0 = MT(0), a1 = MT(0), a2 = MT(0), a3 = MT(0);
    int q = q0 + lane;
    for (; q + 96 < q1; q += 128) {
        V v0 = __ldg(r + q), v1 = __ldg(r + q + 32), v2 = __ldg(r + q + 64), v3 = __ldg(r + q + 96);
        a0 += Vec16<MT>::dot(v0, vs + NV * q);
        a1 += Vec16<MT>::dot(v1, vs + NV * (q + 32));
        a2 += Vec16<MT>::dot(v2, vs + NV * (q + 64));
        a3 += Vec16<MT>::dot(v3, vs + NV * (q + 96));
    }
    for (; q < q1; q += 32) a0 += Vec16<MT>::dot(__ldg(r + q), vs + NV * q);
    MT acc = (a0 + a1) + (a2 + a3);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    return acc;
}

// v = xi + Linv f (row i: vectors 0 .. i / NV)
template <typename T, typename MT, int NOISE>
__device__ __forceinline__ void chol_gemv_lower_body(const T *__restrict__ f, const Grid3 &g, const MT *__restrict__ Linv,
                                                     int ld, MT *__restrict__ v, const NoiseArgs &nz,
                                                     unsigned char *chol_sm, int bx, int nbx) {
    MT *fs = reinterpret_cast<MT *>(chol_sm);
    const int n = g.N0 * g.N1 * g.N2;
    for (int i = threadIdx.x; i < ld; i += blockDim.x) {
        MT val = MT(0);
        if (i < n) {
            const int a = i % g.N0, t = i / g.N0;
            val = (MT)f[g.pad(a, t % g.N1, t / g.N1)];
        }
        fs[i] = val;
    }
    __syncthreads();
    constexpr int NV = Vec16<MT>::N;
    const int lane = threadIdx.x & 31;
    const int warps = nbx * (blockDim.x >> 5);
    for (int ii = bx * (blockDim.x >> 5) + (threadIdx.x >> 5); ii < n; ii += warps) {
        const int i = (ii & 1) ? n - 1 - (ii >> 1) : (ii >> 1);
        const MT acc = warp_row_dot<MT>(Linv + (i64)i * ld, fs, 0, i / NV + 1, lane);
        if (lane == 0) {
            double xi = 0.0;
            if (NOISE == NOISE_INJECTED) xi = nz.buf[i];
            if (NOISE == NOISE_PHILOX) {
                float4 r = normals4(philox4x32_10(noise_ctr(nz, (unsigned)(i >> 2), PURPOSE_COARSE, 0), noise_key(nz)));
                xi = (double)pick(r, i & 3);
            }
            v[i] = (MT)xi + acc;
        }
    }
}

template <typename T, typename MT, int NOISE>
__global__ void __launch_bounds__(256) k_chol_gemv_lower(const T *__restrict__ f, Grid3 g, const MT *__restrict__ Linv,
                                                          int ld, MT *__restrict__ v, NoiseArgs nz) {
    if (g.pdl) pdl_begin();
    extern __shared__ __align__(16) unsigned char chol_sm[];
    chol_gemv_lower_body<T, MT, NOISE>(f, g, Linv, ld, v, nz, chol_sm, blockIdx.x, gridDim.x);
}

// ... x = Linv^T v (row j of Linv^T: vectors j / NV .. ld / NV - 1).
template <typename T, typename MT>
__device__ __forceinline__ void chol_gemv_upper_body(const MT *__restrict__ v, const Grid3 &g,
                                                     const MT *__restrict__ LinvT, int ld, T *__restrict__ x,
                                                     unsigned char *chol_sm, int bx, int nbx) {
    MT *vs = reinterpret_cast<MT *>(chol_sm);
    const int n = g.N0 * g.N1 * g.N2;
    for (int i = threadIdx.x; i < ld; i += blockDim.x) vs[i] = i < n ? v[i] : MT(0);
    __syncthreads();
    constexpr int NV = Vec16<MT>::N;
    const int lane = threadIdx.x & 31;
    const int warps = nbx * (blockDim.x >> 5);
    for (int jj = bx * (blockDim.x >> 5) + (threadIdx.x >> 5); jj < n; jj += warps) {
        const int j = (jj & 1) ? n - 1 - (jj >> 1) : (jj >> 1);
        const MT acc = warp_row_dot<MT>(LinvT + (i64)j * ld, vs, j / NV, ld / NV, lane);
        if (lane == 0) {
            const int a = j % g.N0, t = j / g.N0;
            x[g.pad(a, t % g.N1, t / g.N1)] = (T)acc;
        }
    }
}

template <typename T, typename MT>
__global__ void __launch_bounds__(256) k_chol_gemv_upper(const MT *__restrict__ v, Grid3 g,
                                                          const MT *__restrict__ LinvT, int ld, T *__restrict__ x) {
    if (g.pdl) pdl_begin();
    extern __shared__ __align__(16) unsigned char chol_sm[];
    chol_gemv_upper_body<T, MT>(v, g, LinvT, ld, x, chol_sm, blockIdx.x, gridDim.x);
}

// ------------------------------------------------------------- adjoint
// y += alpha x over whole padded arrays (ghosts are zero in both).
template <typename T>
__global__ void __launch_bounds__(256) k_axpy(T *__restrict__ y, const T *__restrict__ x, T alpha, i64 n) {
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) y[i] += alpha * x[i];
}

// out_k = Sigma_k sum_j (S^{-1})_{jk} q_j: the transposed m x m solve of the
// low-rank correction, scaled by Sigma so that k_add_Bq (which divides by
// Sigma) applies B S^{-T} q.  One thread per k; SinvT row k is column k of
// S^{-1}.
__global__ void __launch_bounds__(256) k_sinvt_q(const double *__restrict__ SinvT, const double *__restrict__ q,
                                                 const double *__restrict__ sigma_sqrt, double *__restrict__ out, int m) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m) return;
    double t = 0.0;
    for (int j = 0; j < m; ++j) t = fma(SinvT[(i64)k * m + j], q[j], t);
    out[k] = sigma_sqrt[k] * sigma_sqrt[k] * t;
}

// ------------------------------------------------- deterministic solver
// One iteration of LoopSolver::apply (loop_solver.cc:24-42) keeps the
// iterate x, the right hand side b and the residual r in FP64 on level 0,
// whatever the type T of the hierarchy that applies the multigrid
// preconditioner: with an FP32 hierarchy the loop is iterative refinement
// and still converges to FP64 accuracy.
//
// r = b - A_0 x over the interior (the low-rank term is added afterwards by
// k_add_Bq with sign -1).
template <int NPT, int VAR = 0>
__global__ void __launch_bounds__(256) k_solve_resid(const double *__restrict__ x, const double *__restrict__ b,
                                                     double *__restrict__ r, Grid3 g, StencilArg<double> s,
                                                     VarField<double> vf) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x, bb = blockIdx.y, c = blockIdx.z;
    if (a >= g.N0) return;
    const i64 P = g.pad(a, bb, c);
    r[P] = b[P] - stencil_row<double, NPT, false, VAR>(x, g, s, P, vf);
}

// Per CTA: SOLVE_ROWS rows (b, c) of the interior.  The partial sums of
// |r|^2 go to part[blockIdx.x] (a fixed grid, so the norm is
// reproducible); the preconditioner gets f = (T) r and the zero initial
// state of MultigridPreconditioner::solve (multigrid_preconditioner.cc:76).
constexpr int SOLVE_ROWS = 8;
template <typename T>
__global__ void __launch_bounds__(256) k_solve_rhs(const double *__restrict__ r, T *__restrict__ f,
                                                   T *__restrict__ x, Grid3 g, double *__restrict__ part) {
    __shared__ double sh[32];
    const i64 nrows = (i64)g.N1 * g.N2;
    double acc = 0.0;
    for (int q = 0; q < SOLVE_ROWS; ++q) {
        const i64 row = (i64)blockIdx.x * SOLVE_ROWS + q;
        if (row >= nrows) break;
        const int bb = (int)(row % g.N1), c = (int)(row / g.N1);
        for (int a = threadIdx.x; a < g.N0; a += blockDim.x) {
            const i64 P = g.pad(a, bb, c);
            const double v = r[P];
            acc += v * v;
            f[P] = (T)v;
            x[P] = T(0);
        }
    }
    acc = block_sum<256>(acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

// |r|^2 = the sum of the partial sums, in one CTA.
__global__ void __launch_bounds__(256) k_solve_norm(const double *__restrict__ part, int np, double *__restrict__ out) {
    __shared__ double sh[32];
    double acc = 0.0;
    for (int i = threadIdx.x; i < np; i += blockDim.x) acc += part[i];
    acc = block_sum<256>(acc, sh);
    if (threadIdx.x == 0) *out = acc;
}

// x += P r: the preconditioner's result (type T) added to the FP64 iterate
// over whole padded arrays (ghosts are zero in both).
template <typename T>
__global__ void __launch_bounds__(256) k_solve_update(double *__restrict__ x, const T *__restrict__ dx, i64 n) {
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) x[i] += (double)dx[i];
}

// ------------------------------------------------------ exact sampler
// A draw eta ~ N(0, A_0) for a symmetric stencil with non-positive
// off-diagonal weights and a non-negative diagonal surplus
// c_0 = w_c - sum_k |w_k|:  x^T A_0 x = c_0 |x|^2 + sum over edges (p, q) of
// c_k (x_q - x_p)^2, one edge per pair of stencil neighbours in each of the
// 13 directions k of positive linear offset, c_k = -w_k, and one boundary
// edge (outside value zero) wherever a neighbour lies outside the lattice
// (which keeps the diagonal of the Dirichlet operator).  So
//   eta_p = sqrt(c_0) xi_p + sum_k sqrt(c_k) (xi_{k, p - o_k} - xi_{k, p}),
// with independent normals xi on the points and on the edges (edge (r, r +
// o_k) keyed by its lower end r, which may be a ghost position).  Philox
// keys: the sampler's seed; counter (edge or point id, purpose EXACT,
// direction k in the level byte, the step counter).  b += eta.
struct EdgeWeights {
    double c0;        // sqrt(c_0)
    double ck[13];    // sqrt(c_k) for the directions of positive offset
    int off[13][3];   // (dx, dy, dz) of direction k
};

__device__ __forceinline__ double exact_normal(const NoiseArgs &nz, int k, unsigned id) {
    NoiseArgs a = nz;
    a.level = (unsigned)k;
    return (double)normals4(philox4x32_10(noise_ctr(a, id, PURPOSE_EXACT, 0), noise_key(a))).x;
}

// cdiag (may be null): per-point centre weights, c_0 = cdiag[P] - offsum.
template <int NPT>
__global__ void __launch_bounds__(256) k_prior_perturbation(double *__restrict__ b, Grid3 g, EdgeWeights ew,
                                                            NoiseArgs nz, const double *__restrict__ cdiag,
                                                            double offsum) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x, bb = blockIdx.y, c = blockIdx.z;
    if (a >= g.N0) return;
    // ids over positions (-1 .. N) in every direction
    const unsigned X = (unsigned)g.N0 + 2u, Y = (unsigned)g.N1 + 2u;
    auto id = [&](int pa, int pb, int pc) { return ((unsigned)(pc + 1) * Y + (unsigned)(pb + 1)) * X + (unsigned)(pa + 1); };
    const double c0 = cdiag ? sqrt(fmax(cdiag[g.pad(a, bb, c)] - offsum, 0.0)) : ew.c0;
    double eta = c0 * exact_normal(nz, 0, id(a, bb, c));
#pragma unroll
    for (int k = 0; k < 13; ++k) {
        const int dx = ew.off[k][0], dy = ew.off[k][1], dz = ew.off[k][2];
        if (NPT == 7 && (dx != 0) + (dy != 0) + (dz != 0) > 1) continue;
        if (ew.ck[k] == 0.0) continue;
        eta += ew.ck[k] * (exact_normal(nz, k + 1, id(a - dx, bb - dy, c - dz)) - exact_normal(nz, k + 1, id(a, bb, c)));
    }
    b[g.pad(a, bb, c)] += eta;
}

// y_j = Sigma_j^{1/2} xi_j with m more normals (direction byte 14), so that
// k_add_Bq (which divides by Sigma) adds B Sigma^{-1/2} xi: the low-rank
// part of eta ~ N(0, A_0 + B Sigma^{-1} B^T).
__global__ void __launch_bounds__(256) k_lowrank_perturbation(NoiseArgs nz, const double *__restrict__ sigma_sqrt, int m,
                                                              double *__restrict__ y) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    y[j] = sigma_sqrt[j] * exact_normal(nz, 14, (unsigned)j);
}

// ------------------------------------------------ parameter adjoint
// Derivatives of one step (noise fixed) with respect to the fine stencil's
// centre weight s (for the FD prior, s = h^d kappa^2 + const, so
// d/dkappa^2 = h^d d/ds) and to log Sigma_k.  A sweep is
// x'' = x + M_f^{-1}(c - A x) with M_f = M + B Sigma^{-1} B^T,
// M = D / omega + (A_0's part before the point in the sweep order) and
// c = f + sd xi + B Sigma^{-1/2} xi'; with u = M_f^{-T} x-bar'' it adds
//   u^T dc - u^T dN x - u^T dM_f x''   (N = A_0 - M)
// to the gradient.  dA_0/ds on level l is the Galerkin stencil E_l of the
// unit centre weight; the noise part c - f = M x'' + N x + B Sigma^{-1} B^T x''
// - f is rebuilt from the sweep's input and output states, so the point
// normals need not be stored.
struct PgradStencils {
    double a[27];  // the level's A_0
    double e[27];  // E_l = dA_0 / ds
    float af[27], ef[27];  // the same rounded to FP32 (neighbour sums of FP32 chains)
};

template <typename T>
__device__ __forceinline__ T pg_a(const PgradStencils &st, int k);
template <>
__device__ __forceinline__ float pg_a<float>(const PgradStencils &st, int k) { return st.af[k]; }
template <>
__device__ __forceinline__ double pg_a<double>(const PgradStencils &st, int k) { return st.a[k]; }
template <typename T>
__device__ __forceinline__ T pg_e(const PgradStencils &st, int k);
template <>
__device__ __forceinline__ float pg_e<float>(const PgradStencils &st, int k) { return st.ef[k]; }
template <>
__device__ __forceinline__ double pg_e<double>(const PgradStencils &st, int k) { return st.e[k]; }

// Colour of interior point (a, b, c) in the multicolour order (2 colours:
// parity of a + b + c; 2^dim colours: one parity bit per direction).
__device__ __forceinline__ int point_colour(int ncol, int a, int b, int c) {
    return ncol == 2 ? ((a + b + c) & 1) : ((a & 1) | ((b & 1) << 1) | ((c & 1) << 2));
}

// Per CTA of SOLVE_ROWS rows, the eight sums over the level's points p
// (part[j * gridDim.x + blockIdx.x]):
//   0: u_p sum_{q before p} A_pq v_q    1: u_p sum_{q after p} A_pq w_q
//   2: u_p sum_{q before p} E_pq v_q    3: u_p sum_{q before p} E_pq w_q
//   4: u_p sum_{q after p} E_pq w_q     5: u_p v_p   6: u_p w_p   7: u_p f_p
// (v = the sweep's output, w = its input; off-diagonal neighbours only, the
// 6 axis neighbours of a 7-point level or all 26).  "Before" is the order
// of the sweep of direction `forward`: by linear index for the
// lexicographic order (ncol = 0), by colour otherwise.  The neighbour sums
// run in the chain's type T, the u_p-weighted sums in FP64.  Without
// off-diagonal entries in E (HAS_E false: the fine level's E is the unit
// centre weight) sums 2 to 4 are zero and skipped.
template <typename T, int NPT, bool HAS_E>
__global__ void __launch_bounds__(256) k_pgrad_stencil(const T *__restrict__ u, const T *__restrict__ v,
                                                       const T *__restrict__ w, const T *__restrict__ f, Grid3 g,
                                                       PgradStencils st, int ncol, int forward,
                                                       double *__restrict__ part) {
    __shared__ double sh[32];
    const i64 nrows = (i64)g.N1 * g.N2;
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int q = 0; q < SOLVE_ROWS; ++q) {
        const i64 row = (i64)blockIdx.x * SOLVE_ROWS + q;
        if (row >= nrows) break;
        const int bb = (int)(row % g.N1), c = (int)(row / g.N1);
        for (int a = threadIdx.x; a < g.N0; a += blockDim.x) {
            const i64 P = g.pad(a, bb, c);
            const T up = u[P];
            if (up == T(0)) continue;
            const int cp = ncol ? point_colour(ncol, a, bb, c) : 0;
            T lav = 0, uaw = 0, lev = 0, lew = 0, uew = 0;
#pragma unroll
            for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
                for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
                    for (int dx = -1; dx <= 1; ++dx) {
                        const int nzo = (dx != 0) + (dy != 0) + (dz != 0);
                        if (nzo == 0 || (NPT == 7 && nzo > 1)) continue;
                        const int k = (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1);
                        const T wa = pg_a<T>(st, k), we = pg_e<T>(st, k);
                        bool before;
                        if (ncol == 0) {
                            const bool lower = dz < 0 || (dz == 0 && (dy < 0 || (dy == 0 && dx < 0)));
                            before = forward ? lower : !lower;
                        } else {
                            const int cq = point_colour(ncol, a + dx, bb + dy, c + dz);
                            before = forward ? cq < cp : cq > cp;
                        }
                        const i64 Q = P + dz * g.sz + dy * g.sy + dx;
                        const T wq = w[Q];
                        if (before) {
                            const T vq = v[Q];
                            lav += wa * vq;
                            if (HAS_E) {
                                lev += we * vq;
                                lew += we * wq;
                            }
                        } else {
                            uaw += wa * wq;
                            if (HAS_E) uew += we * wq;
                        }
                    }
            const double ud = (double)up;
            acc[0] += ud * (double)lav;
            acc[1] += ud * (double)uaw;
            if (HAS_E) {
                acc[2] += ud * (double)lev;
                acc[3] += ud * (double)lew;
                acc[4] += ud * (double)uew;
            }
            acc[5] += ud * (double)v[P];
            acc[6] += ud * (double)w[P];
            acc[7] += ud * (double)f[P];
        }
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const double t = block_sum<256>(acc[j], sh);
        if (threadIdx.x == 0) part[(i64)j * gridDim.x + blockIdx.x] = t;
        __syncthreads();
    }
}

// Adds one event's contribution to the gradients (one CTA).  Sums the eight
// partial streams of k_pgrad_stencil (np values each) into S0..S7 and, with Bu = B^T u,
// Bv = B^T v and the low-rank normals xi' of the sweep:
// sweep (mode 0), kd = dsd/ds / sd = E_c / (2 A_c):
//   g_s += kd [S0 + A_c/omega S5 + S1 + A_c (1 - 1/omega) S6 - S7
//              + sum_k Bu_k Bv_k / Sigma_k - sum_k Bu_k xi'_k / Sigma_k^{1/2}]
//          - [S2 + S4 + E_c S6 + E_c/omega (S5 - S6)]
//   g_k += Bu_k (Bv_k / Sigma_k - xi'_k / (2 Sigma_k^{1/2}))
// -u^T dA v with v = w (mode 1: the residual f - A x with u = P f_c-bar,
// and the coarse mean Q^{-1} f with u = Q^{-1} x-bar):
//   g_s -= S3 + S4 + E_c S6;   g_k += Bu_k Bv_k / Sigma_k
struct PgradCoef {
    double kd, omega, ac, ec;
    int mode;
};
__global__ void __launch_bounds__(256) k_pgrad_combine(const double *__restrict__ part, int np,
                                                       const double *__restrict__ Bu, const double *__restrict__ Bv,
                                                       const double *__restrict__ xi,
                                                       const double *__restrict__ sigma_inv,
                                                       const double *__restrict__ sigma_sqrt, int m, PgradCoef cf,
                                                       double *__restrict__ g_s, double *__restrict__ g_sig) {
    __shared__ double sh[32];
    double S[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        double a = 0.0;
        for (int i = threadIdx.x; i < np; i += blockDim.x) a += part[(i64)j * np + i];
        S[j] = block_sum<256>(a, sh);
        __syncthreads();
    }
    double q1 = 0.0, q2 = 0.0;
    for (int k = threadIdx.x; k < m; k += blockDim.x) {
        q1 += Bu[k] * Bv[k] * sigma_inv[k];
        if (cf.mode == 0) q2 += Bu[k] * xi[k] / sigma_sqrt[k];
        g_sig[k] += cf.mode == 0 ? Bu[k] * (Bv[k] * sigma_inv[k] - 0.5 * xi[k] / sigma_sqrt[k])
                                 : Bu[k] * Bv[k] * sigma_inv[k];
    }
    q1 = block_sum<256>(q1, sh);
    __syncthreads();
    q2 = block_sum<256>(q2, sh);
    if (threadIdx.x == 0) {
        double c;
        if (cf.mode == 0)
            c = cf.kd * (S[0] + cf.ac / cf.omega * S[5] + S[1] + cf.ac * (1.0 - 1.0 / cf.omega) * S[6] - S[7] + q1 - q2) -
                (S[2] + S[4] + cf.ec * S[6] + cf.ec / cf.omega * (S[5] - S[6]));
        else
            c = -(S[3] + S[4] + cf.ec * S[6]);
        *g_s += c;
    }
}

// The low-rank normals xi'_k of one sweep (as the low-rank kernels draw
// them), and the n coarse normals of the Cholesky sample, compact.
template <int NOISE>
__global__ void __launch_bounds__(256) k_lowrank_normals(NoiseArgs nz, int m, double *__restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m) return;
    double xi = 0.0;
    if (NOISE == NOISE_PHILOX) {
        float4 rn = normals4(philox4x32_10(noise_ctr(nz, (unsigned)(k >> 2), PURPOSE_LOWRANK, 0), noise_key(nz)));
        xi = (double)pick(rn, k & 3);
    }
    if (NOISE == NOISE_INJECTED) xi = nz.buf[k];
    out[k] = xi;
}

template <int NOISE>
__global__ void __launch_bounds__(256) k_coarse_normals(NoiseArgs nz, int n, double *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double xi = 0.0;
    if (NOISE == NOISE_PHILOX) {
        float4 r = normals4(philox4x32_10(noise_ctr(nz, (unsigned)(i >> 2), PURPOSE_COARSE, 0), noise_key(nz)));
        xi = (double)pick(r, i & 3);
    }
    if (NOISE == NOISE_INJECTED) xi = nz.buf[i];
    out[i] = xi;
}

// The coarse Cholesky sample x = Q^{-1} f + L^{-T} xi, Q = L L^T: with
// dL = L Phi(L^{-1} dQ L^{-T}), Phi(X) = strict lower part + half the
// diagonal, x-bar^T dx = -w1^T dQ mu - xi^T Phi(L^{-1} dQ L^{-T}) w2
// (mu = Q^{-1} f, w1 = Q^{-1} x-bar, w2 = L^{-1} x-bar).
//
// s-term: part[blockIdx.x] = sum over its rows i of xi_i (Phi(X_E) w2)_i,
// X_E = L^{-1} E_c L^{-T} stored like the inverse factor (row-major, ld a
// multiple of 16 bytes, zeros above the diagonal); one warp per row.
template <typename MT>
__global__ void __launch_bounds__(256) k_pgrad_coarse_phi(const MT *__restrict__ Phi, int ld,
                                                          const MT *__restrict__ w2, const double *__restrict__ xi,
                                                          int n, double *__restrict__ part) {
    extern __shared__ __align__(16) unsigned char chol_sm[];
    __shared__ double sh[32];
    MT *ws = reinterpret_cast<MT *>(chol_sm);
    for (int i = threadIdx.x; i < ld; i += blockDim.x) ws[i] = i < n ? w2[i] : MT(0);
    __syncthreads();
    constexpr int NV = Vec16<MT>::N;
    const int lane = threadIdx.x & 31;
    const int warps = gridDim.x * (blockDim.x >> 5);
    double acc = 0.0;
    for (int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
        const MT r = warp_row_dot<MT>(Phi + (i64)i * ld, ws, 0, i / NV + 1, lane);
        if (lane == 0) acc += xi[i] * (double)r;
    }
    acc = block_sum<256>(acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

// *target += scale * sum(part[0 .. np))
__global__ void __launch_bounds__(256) k_accum_sum(const double *__restrict__ part, int np, double scale,
                                                   double *__restrict__ target) {
    __shared__ double sh[32];
    double acc = 0.0;
    for (int i = threadIdx.x; i < np; i += blockDim.x) acc += part[i];
    acc = block_sum<256>(acc, sh);
    if (threadIdx.x == 0) *target += scale * acc;
}

// log Sigma_k term of the coarse sample's L^{-T} xi part (dQ = -b_k b_k^T /
// Sigma_k, u = L^{-1} b_k, column k of U):
//   g_k += (1 / Sigma_k) sum_j u_j w2_j (sum_{i > j} u_i xi_i + u_j xi_j / 2).
// One CTA per k; the suffix sums run over chunks of 256 indices from the
// end, a block scan inside each chunk.
template <typename MT>
__global__ void __launch_bounds__(256) k_pgrad_coarse_sigma(const double *__restrict__ U, const MT *__restrict__ w2,
                                                            const double *__restrict__ xi,
                                                            const double *__restrict__ sigma_inv,
                                                            double *__restrict__ g_sig, int n) {
    __shared__ double wsum[8];
    __shared__ double sh[32];
    __shared__ double carry;
    const int k = blockIdx.x;
    const double *u = U + (i64)k * n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0.0;
    __syncthreads();
    double acc = 0.0;
    for (int base = ((n - 1) / 256) * 256; base >= 0; base -= 256) {
        const int j = base + threadIdx.x;
        const double uj = j < n ? u[j] : 0.0, xj = j < n ? xi[j] : 0.0, wj = j < n ? (double)w2[j] : 0.0;
        const double v = uj * xj;
        double incl = v;  // sum over the lanes at or above this one
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double t = __shfl_down_sync(0xffffffffu, incl, o);
            if (lane + o < 32) incl += t;
        }
        if (lane == 0) wsum[warp] = incl;
        __syncthreads();
        double above = 0.0;
        for (int q = warp + 1; q < 8; ++q) above += wsum[q];
        acc += wj * uj * (carry + above + (incl - v) + 0.5 * v);
        __syncthreads();
        if (threadIdx.x == 0) {
            double tot = 0.0;
            for (int q = 0; q < 8; ++q) tot += wsum[q];
            carry += tot;
        }
        __syncthreads();
    }
    acc = block_sum<256>(acc, sh);
    if (threadIdx.x == 0) g_sig[k] += sigma_inv[k] * acc;
}

// ------------------------------------------------------------ step end
// Observables z_p = b_p^T x of measure_sampling_time (sampling_time.cc:40),
// one CTA per probe p (probe p's entries are bptr[p]..bptr[p+1]), stored at
// obs[k * nprobe + p] for step k while k < capacity; a non-finite value
// raises the error flag.  The last CTA to finish advances the observation
// count and the step counter that keys the Philox streams.  Runs after
// every other kernel of the step.
template <typename T>
__device__ __forceinline__ void step_end_body(const T *__restrict__ x, int nprobe, const i64 *__restrict__ bptr,
                                              const i64 *__restrict__ bidx, const double *__restrict__ bval,
                                              double *__restrict__ obs, i64 capacity, u64 *__restrict__ obs_count,
                                              u64 *__restrict__ d_step, unsigned *__restrict__ err,
                                              unsigned *__restrict__ done, int p, int nblocks) {
    __shared__ double sh[32];
    __shared__ bool last;
    if (nprobe > 0 && p < nprobe) {
        double acc = 0.0;
        for (i64 e = bptr[p] + threadIdx.x; e < bptr[p + 1]; e += blockDim.x) acc += bval[e] * (double)x[bidx[e]];
        acc = block_sum<256>(acc, sh);
        if (threadIdx.x == 0) {
            const u64 k = *obs_count;
            if ((i64)k < capacity) obs[k * nprobe + p] = acc;
            if (!isfinite(acc)) atomicOr(err, 1u);
        }
    }
    __threadfence();
    if (threadIdx.x == 0) last = (atomicAdd(done, 1u) == (unsigned)nblocks - 1u);
    __syncthreads();
    if (last && threadIdx.x == 0) {
        if (nprobe > 0) *obs_count += 1ull;
        *d_step += 1ull;
        *done = 0u;
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_step_end(const T *__restrict__ x, int nprobe, const i64 *__restrict__ bptr,
                                                   const i64 *__restrict__ bidx, const double *__restrict__ bval,
                                                   double *__restrict__ obs, i64 capacity, u64 *__restrict__ obs_count,
                                                   u64 *__restrict__ d_step, unsigned *__restrict__ err,
                                                   unsigned *__restrict__ done) {
    pdl_begin();
    step_end_body<T>(x, nprobe, bptr, bidx, bval, obs, capacity, obs_count, d_step, err, done, blockIdx.x, gridDim.x);
}

// ------------------------------------------- low-rank Cholesky sampler
// The sampler's solves with the block factor of A_0 and its low-rank
// products are dense FP64 matrix-vector products of three kinds.

// y_i = yadd_i + alpha sum_j A_ij v_j over a row-major rows x cols block
// (leading dimension lda): one warp per row, lanes over the columns, a
// warp-shuffle sum.  LOWER: the block is lower triangular (columns j <= i).
// y may alias yadd (each row reads its own entry before writing it).
template <bool LOWER>
__global__ void __launch_bounds__(256) k_dgemv_rows(const double *__restrict__ A, i64 rows, i64 cols, i64 lda,
                                                    const double *__restrict__ v, const double *yadd, double alpha,
                                                    double *y) {
    const i64 i = ((i64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= rows) return;
    const i64 jmax = LOWER ? min(i + 1, cols) : cols;
    const double *Ai = A + i * lda;
    double a0 = 0.0, a1 = 0.0;
    i64 j = lane;
    for (; j + 32 < jmax; j += 64) {
        a0 = fma(Ai[j], v[j], a0);
        a1 = fma(Ai[j + 32], v[j + 32], a1);
    }
    if (j < jmax) a0 = fma(Ai[j], v[j], a0);
    double acc = a0 + a1;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) y[i] = (yadd ? yadd[i] : 0.0) + alpha * acc;
}

// Partial sums of (A^T v)_j over row chunk blockIdx.y (rows [c rch,
// (c + 1) rch)): part[c cols + j], one thread per column (coalesced row
// reads).  LOWER: A is lower triangular, rows i >= j only.
template <bool LOWER>
__global__ void __launch_bounds__(256) k_dgemv_cols_partial(const double *__restrict__ A, i64 rows, i64 cols, i64 lda,
                                                            const double *__restrict__ v, int rch,
                                                            double *__restrict__ part) {
    const i64 j = (i64)blockIdx.x * blockDim.x + threadIdx.x;
    const int c = blockIdx.y;
    if (j >= cols) return;
    i64 i0 = (i64)c * rch;
    const i64 i1 = min(rows, i0 + rch);
    if (LOWER && i0 < j) i0 = j;
    double acc = 0.0;
    for (i64 i = i0; i < i1; ++i) acc = fma(A[i * lda + j], v[i], acc);
    part[(i64)c * cols + j] = acc;
}

// y_j = yadd_j + alpha sum_c part[c cols + j], chunks in order (the result
// does not depend on block timing).  y may alias yadd.
__global__ void __launch_bounds__(256) k_dgemv_cols_finish(const double *__restrict__ part, int nch, i64 cols,
                                                           const double *yadd, double alpha, double *y) {
    const i64 j = (i64)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= cols) return;
    double acc = 0.0;
    for (int c = 0; c < nch; ++c) acc += part[(i64)c * cols + j];
    y[j] = (yadd ? yadd[j] : 0.0) + alpha * acc;
}

// xi_i ~ N(0, 1): Philox (counter: vertex group i / 4, purpose
// PURPOSE_CHOLESKY, the sampler's step counter) or the injected normals
template <int NOISE>
__global__ void __launch_bounds__(256) k_cholesky_normals(NoiseArgs nz, i64 n, double *__restrict__ xi) {
    const i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (NOISE == NOISE_INJECTED) {
        xi[i] = nz.buf[i];
    } else {
        const float4 r = normals4(philox4x32_10(noise_ctr(nz, (unsigned)(i >> 2), PURPOSE_CHOLESKY, 0), noise_key(nz)));
        xi[i] = (double)pick(r, (int)(i & 3));
    }
}

__global__ void k_counter_advance(u64 *__restrict__ step) { *step += 1ull; }

// ------------------------------------------------------- batched chains
// Chains of one lattice geometry stepped together (FP32-mixed chains with
// Philox noise): every launch of the step covers all chains of the group --
// blockIdx.z (or blockIdx.y) picks the chain for the regular work, a job
// table for the ragged low-rank work -- and each chain keeps its own arrays,
// stencils, low-rank data, Philox key and step counter.  The kernels call
// the one-chain kernels' bodies, so a chain stepped in a batch draws the
// same normals and computes the same values, bit for bit, as when it is
// stepped alone.

// One chain on one level.
struct BatchLevelArg {
    float *x, *f;
    const float *fsplit;  // level 0: the colour-split f (colour k at fsplit + k * fhalf), else null
    i64 fhalf;
    float *xc, *fc;       // the next level's state and right hand side (null on the coarsest level)
    StencilArg<float> s;
};
static_assert(sizeof(StencilArg<float>) == 32 * sizeof(float), "stencil argument: 32 floats");

// One chain: noise key, step counter, coarse Cholesky factors, observables.
struct BatchChainArg {
    u64 seed;
    u64 *d_step;
    const float *Linv, *LinvT;
    float *gv;
    int nprobe;
    const i64 *bptr, *bidx;
    const double *bval;
    double *obs;
    i64 capacity;
    u64 *obs_count;
    unsigned *err, *done;
};

// Low-rank data of one chain on one level and sweep direction: the B^T x
// arguments and C = M^{-1} B by rows.
struct BatchLowRank {
    LowRankArg lr;
    CorrRows C;  // x += C z rows (FP32 values)
};

// B^T x work unit: chain, column j, part p of P.
struct BtJob {
    int chain, j, p, P;
};
// Row range [r0, r1) of one chain's sparse rows.
struct RowJob {
    int chain;
    i64 r0, r1;
};
// B_c Sigma^{-1} y rows of one chain's coarse level (the residual's
// low-rank term), destination its coarse f.
struct BatchAddBq {
    i64 nrows;
    const i64 *rows, *ptr;
    const int *col;
    const double *val, *y, *sigma_inv;
    float *dst;
};

__device__ __forceinline__ void load_stencil_shared(StencilArg<float> &dst, const StencilArg<float> &src) {
    const int t = (threadIdx.z * blockDim.y + threadIdx.y) * blockDim.x + threadIdx.x;
    if (t < 32) reinterpret_cast<float *>(&dst)[t] = reinterpret_cast<const float *>(&src)[t];
    __syncthreads();
}

__device__ __forceinline__ NoiseArgs batch_noise(const BatchChainArg &c, unsigned invocation, unsigned level) {
    NoiseArgs nz;
    nz.buf = nullptr;
    nz.seed = c.seed;
    nz.d_step = c.d_step;
    nz.invocation = invocation;
    nz.level = level;
    return nz;
}

// red-black colour pass of the 7-point level, grid.z = chains x planes
template <int NOISE, bool V8, bool FS>
__global__ void __launch_bounds__(RBP_THREADS) k_sweep_rb_vec_batch(const BatchLevelArg *__restrict__ la,
                                                                    const BatchChainArg *__restrict__ ca, Grid3 g,
                                                                    int colour, int reverse, unsigned invocation,
                                                                    unsigned level) {
    __shared__ StencilArg<float> ss;
    const int chain = blockIdx.z / g.N2, bz = blockIdx.z - chain * g.N2;
    const BatchLevelArg &a = la[chain];
    load_stencil_shared(ss, a.s);
    const NoiseArgs nz = batch_noise(ca[chain], invocation, level);
    const float *fsc = FS ? a.fsplit + colour * a.fhalf : nullptr;
    sweep_rb_vec_body<NOISE, false, V8, FS>(a.x, a.f, g, ss, colour, reverse, nz, nullptr, fsc, blockIdx.x, blockIdx.y,
                                            bz);
}

// one colour of an 8-colour level, grid.z = chains x colour planes
template <int NOISE>
__global__ void __launch_bounds__(RBP_THREADS) k_sweep_c27_batch(const BatchLevelArg *__restrict__ la,
                                                                 const BatchChainArg *__restrict__ ca, Grid3 g,
                                                                 int colour, int ncz, unsigned invocation,
                                                                 unsigned level) {
    __shared__ StencilArg<float> ss;
    const int chain = blockIdx.z / ncz, bz = blockIdx.z - chain * ncz;
    const BatchLevelArg &a = la[chain];
    load_stencil_shared(ss, a.s);
    const NoiseArgs nz = batch_noise(ca[chain], invocation, level);
    sweep_c27_body<float, false, NOISE, 0>(a.x, a.f, g, ss, colour, nz, VarField<float>{nullptr, 0}, blockIdx.x,
                                           blockIdx.y, bz);
}

// B^T x partial sums with the per-chain solve in each chain's last CTA
// (SOLVE: the low-rank correction's coefficients; otherwise y = B^T x of the
// residual), one CTA per job
template <int NOISE, bool SOLVE>
__global__ void __launch_bounds__(256) k_bt_solve_batch(const BatchLevelArg *__restrict__ la,
                                                        const BatchLowRank *__restrict__ lrs,
                                                        const BatchChainArg *__restrict__ ca,
                                                        const BtJob *__restrict__ jobs, unsigned invocation,
                                                        unsigned level) {
    const BtJob jb = jobs[blockIdx.x];
    const LowRankArg lr = lrs[jb.chain].lr;
    const NoiseArgs nz = batch_noise(ca[jb.chain], invocation, level);
    bt_solve_body<float, NOISE, SOLVE>(la[jb.chain].x, lr, nz, jb.j, jb.p, jb.P);
}

// x += C z over a row range of one chain (the per-row arithmetic of
// k_lr_scatter)
__global__ void __launch_bounds__(256) k_lr_scatter_batch(const BatchLevelArg *__restrict__ la,
                                                          const BatchLowRank *__restrict__ lrs,
                                                          const RowJob *__restrict__ jobs) {
    const RowJob jb = jobs[blockIdx.x];
    const BatchLowRank &c = lrs[jb.chain];
    const CorrRows &C = c.C;
    float *x = la[jb.chain].x;
    const float *z = c.lr.zf;
    const float *v1 = static_cast<const float *>(C.v1);
    for (i64 r = jb.r0 + threadIdx.x; r < jb.r1; r += blockDim.x) {
        if (r < C.n1) {
            const unsigned row = C.r1[r];
            float acc = 0.f;
            acc += v1[r] * z[C.c1[r]];
            x[row] = x[row] + acc;
        } else {
            corr_multi_row(x, C, r - C.n1, z);
        }
    }
}

// f_c -= B_c Sigma^{-1} y over a row range of one chain (the per-row
// arithmetic of k_add_Bq with sign -1)
__global__ void __launch_bounds__(256) k_add_Bq_batch(const BatchAddBq *__restrict__ bq,
                                                      const RowJob *__restrict__ jobs) {
    const RowJob jb = jobs[blockIdx.x];
    const BatchAddBq &a = bq[jb.chain];
    for (i64 r = jb.r0 + threadIdx.x; r < jb.r1; r += blockDim.x) {
        double acc = 0.0;
        for (i64 e = a.ptr[r]; e < a.ptr[r + 1]; ++e) acc += a.val[e] * (a.y[a.col[e]] * a.sigma_inv[a.col[e]]);
        a.dst[a.rows[r]] += (float)(-1.0 * acc);
    }
}

// residual + restriction, grid.z = chains x coarse tiles in z
template <int NPT>
// Six CTAs per SM: the batched residual-restriction (plain loads, one CTA per
// tile of one chain) gains more from occupancy than it loses to the spills
// this forces (512 chains of 32^3-128^3 cells: 23.1k -> 25.8k samples/s
// against 24.9k with four CTAs per SM, one box).
#ifndef MGMC_RR_BATCH_MINB
#define MGMC_RR_BATCH_MINB 6
#endif
__global__ void __launch_bounds__(RR_THREADS, MGMC_RR_BATCH_MINB) k_resid_restrict_batch(const BatchLevelArg *__restrict__ la, Grid3 gf,
                                                                      Grid3 gc, int tz) {
    __shared__ StencilArg<float> ss;
    extern __shared__ __align__(16) unsigned char rr_smem_b[];
    const int chain = blockIdx.z / tz, bz = blockIdx.z - chain * tz;
    const BatchLevelArg &a = la[chain];
    load_stencil_shared(ss, a.s);
    resid_restrict_tiled_body<float, NPT>(a.x, a.f, a.fc, a.xc, gf, gc, ss, rr_smem_b, blockIdx.x, blockIdx.y, bz);
}

// x += alpha P x_c, grid.z = chains x (coarse planes + 1)
__global__ void __launch_bounds__(128) k_prolong_batch(const BatchLevelArg *__restrict__ la, Grid3 gf, Grid3 gc,
                                                       float alpha, int dim, int nzc) {
    const int chain = blockIdx.z / nzc, bz = blockIdx.z - chain * nzc;
    const BatchLevelArg &a = la[chain];
    prolong_add_body<float>(a.x, a.xc, gf, gc, alpha, dim, blockIdx.x, blockIdx.y, nzc - 1 - bz);
}

// coarse Cholesky sample, grid.y = chains
template <int NOISE>
__global__ void __launch_bounds__(256) k_chol_lower_batch(const BatchLevelArg *__restrict__ la,
                                                          const BatchChainArg *__restrict__ ca, Grid3 g, int ld,
                                                          unsigned invocation, unsigned level) {
    extern __shared__ __align__(16) unsigned char chol_sm_b[];
    const BatchChainArg &c = ca[blockIdx.y];
    const NoiseArgs nz = batch_noise(c, invocation, level);
    chol_gemv_lower_body<float, float, NOISE>(la[blockIdx.y].f, g, c.Linv, ld, c.gv, nz, chol_sm_b, blockIdx.x,
                                              gridDim.x);
}

__global__ void __launch_bounds__(256) k_chol_upper_batch(const BatchLevelArg *__restrict__ la,
                                                          const BatchChainArg *__restrict__ ca, Grid3 g, int ld) {
    extern __shared__ __align__(16) unsigned char chol_sm_b[];
    const BatchChainArg &c = ca[blockIdx.y];
    chol_gemv_upper_body<float, float>(c.gv, g, c.LinvT, ld, la[blockIdx.y].x, chol_sm_b, blockIdx.x, gridDim.x);
}

// observables and step counters, grid.y = chains
__global__ void __launch_bounds__(256) k_step_end_batch(const BatchLevelArg *__restrict__ la,
                                                        const BatchChainArg *__restrict__ ca) {
    const BatchChainArg &c = ca[blockIdx.y];
    step_end_body<float>(la[blockIdx.y].x, c.nprobe, c.bptr, c.bidx, c.bval, c.obs, c.capacity, c.obs_count, c.d_step,
                         c.err, c.done, blockIdx.x, gridDim.x);
}

}  // namespace mgmc
