// kernels.cuh -- sm_103a kernels of the Multigrid Monte Carlo step.
//
// Data layout (every level): padded lexicographic arrays with shared ghost
// rows/planes, see Geometry in setup.h.  A point with 0-based interior
// coordinates (a, b, c) lives at P = (c+1) sz + (b+1) sy + (a+1); ghosts are
// zero, so stencil loads need no boundary tests.
//
// Kernels (one V-cycle at level l uses them in this order):
//   k_sweep_colour      multicolour SOR / Gibbs sweep of one colour
//   k_sweep_wavefront   lexicographic SOR sweep as a hyperplane wavefront
//                       (one CTA; parity mode)
//   k_bt_x_z            y = B^T x and the m x m low-rank solve
//   k_lr_scatter        x += C z over the rows of C = M^{-1} B
//   k_resid_restrict    f_c = R (f - A_0 x)  (fused residual + restriction)
//   k_sub_Bq            f_c -= B_c Sigma^{-1} y
//   k_prolong_add       x += alpha P x_c
//   k_chol_*            coarse-level FP64 Cholesky sample
//   k_step_end          observable z = b^T x, step counter
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace mgmc {

typedef long long i64;
typedef unsigned long long u64;

// ------------------------------------------------------------- geometry
struct Grid3 {
    int N0, N1, N2;  // interior vertices per direction
    i64 sy, sz;      // padded strides
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
};

// ---------------------------------------------------------------- noise
enum { NOISE_NONE = 0, NOISE_PHILOX = 1, NOISE_INJECTED = 2 };
enum { PURPOSE_POINT = 0, PURPOSE_LOWRANK = 1, PURPOSE_COARSE = 2 };

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

// Two Box-Muller pairs in FP32 (Box & Muller 1958).  u1 is in (0, 1]: the
// product of a value <= 2^32 with 2^-32 plus 2^-33 rounds to at most 1.0f,
// so the logarithm is never positive.
__device__ __forceinline__ float4 normals4(uint4 r) {
    const float two_m32 = 2.3283064365386963e-10f;  // 2^-32
    const float two_m33 = 1.1641532182693481e-10f;  // 2^-33
    float u1a = __fmaf_rn(__uint2float_rn(r.x), two_m32, two_m33);
    float u1b = __fmaf_rn(__uint2float_rn(r.z), two_m32, two_m33);
    float ra = sqrtf(-2.0f * logf(u1a));
    float rb = sqrtf(-2.0f * logf(u1b));
    float sa, ca, sb, cb;
    sincospif(__uint2float_rz(r.y) * (2.0f * two_m32), &sa, &ca);
    sincospif(__uint2float_rz(r.w) * (2.0f * two_m32), &sb, &cb);
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
template <typename T, int NPT, bool EXACT>
__device__ __forceinline__ void sor_point(T *__restrict__ x, const T *__restrict__ f, const Grid3 &g,
                                          const StencilArg<T> &s, i64 P, bool noisy, T xi) {
    typedef Ar<EXACT> A;
    T res = T(0);
    if (NPT == 7) {
        const int ks[7] = {4, 10, 12, 13, 14, 16, 22};
        const i64 os[7] = {-g.sz, -g.sy, -1, 0, 1, g.sy, g.sz};
#pragma unroll
        for (int q = 0; q < 7; ++q) res = A::add(res, A::mul(s.w[ks[q]], x[P + os[q]]));
    } else {
#pragma unroll
        for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
            for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
                for (int dx = -1; dx <= 1; ++dx)
                    res = A::add(res, A::mul(s.w[(dz + 1) * 9 + (dy + 1) * 3 + (dx + 1)], x[P + dz * g.sz + dy * g.sy + dx]));
    }
    T cval = f[P];
    if (noisy) cval = A::add(A::mul(s.sd, xi), cval);
    T xo = x[P];
    if (EXACT)
        x[P] = A::add(xo, A::mul(s.omega, A::sub(cval, res)) / s.diag);
    else
        x[P] = xo + s.omega_diag * (cval - res);
}

// --------------------------------------------------- multicolour sweep
// Thread = (8-point x-group g, row (b, c)); it updates the <= 4 points of
// the colour in that group.  ncolour == 2: colour (a + b + c) & 1;
// otherwise the colour bits are (a & 1, b & 1, c & 1).
template <typename T, int NPT, bool EXACT, int NOISE>
__global__ void __launch_bounds__(256) k_sweep_colour(T *__restrict__ x, const T *__restrict__ f, Grid3 g,
                                                       StencilArg<T> s, int colour, int ncolour, NoiseArgs nz) {
    const int G0 = (g.N0 + 7) >> 3;
    i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
    int grp = (int)(t % G0);
    i64 row = t / G0;
    int b, c, p;
    if (ncolour == 2) {
        if (row >= (i64)g.N1 * g.N2) return;
        b = (int)(row % g.N1);
        c = (int)(row / g.N1);
        p = (colour + b + c) & 1;
    } else {
        int pb = (colour >> 1) & 1, pc = (colour >> 2) & 1;
        int nb = (g.N1 - pb + 1) >> 1, ncc = (g.N2 - pc + 1) >> 1;
        if (row >= (i64)nb * ncc) return;
        b = 2 * (int)(row % nb) + pb;
        c = 2 * (int)(row / nb) + pc;
        p = colour & 1;
    }
    float4 nrm = make_float4(0.f, 0.f, 0.f, 0.f);
    if (NOISE == NOISE_PHILOX) nrm = point_normals(nz, g, 8 * grp + p, b, c);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        int a = 8 * grp + p + 2 * q;
        if (a >= g.N0) break;
        T xi = T(0);
        if (NOISE == NOISE_PHILOX) xi = (T)pick(nrm, q);
        if (NOISE == NOISE_INJECTED) xi = (T)nz.buf[g.compact(a, b, c)];
        sor_point<T, NPT, EXACT>(x, f, g, s, g.pad(a, b, c), NOISE != NOISE_NONE, xi);
    }
}

// ------------------------------------------- fused red-black SOR sweep
// Both colours of a red-black SOR sweep in one pass over HBM (axis-only
// stencils, i.e. the fine FD level).  A CTA owns an x-y tile of RB_TX x RB_TY
// interior columns and a range of z-planes; it streams the planes through
// shared memory and, plane by plane,
//   1. computes the first colour's new values F on the tile plus a
//      one-point halo (the halo is recomputed by the neighbouring CTAs:
//      every CTA reads only old values, so no inter-CTA ordering exists),
//   2. computes the second colour from F and writes both colours.
// Old state and new state live in different buffers (xin -> xout), so
// halos read by other CTAs are never overwritten.  With in-kernel noise the
// normal of a point is a function of its coordinates only (Philox block per
// (x, y) column and group of 4 planes), so recomputed halo points get the
// same noise.  In exact mode the arithmetic is sor_point's: identical to
// the per-colour kernels and to the oracle's multicolour sweep.
constexpr int RB_TX = 30, RB_TY = 14;          // interior tile
constexpr int RB_W1 = RB_TX + 2, RB_H1 = RB_TY + 2;  // tile + halo 1 (F)
constexpr int RB_W2 = RB_TX + 4, RB_H2 = RB_TY + 4;  // tile + halo 2 (old x)
constexpr int RB_THREADS = RB_W1 * RB_H1;       // 512: one thread per halo-1 column

__device__ __forceinline__ float4 column_normals(const NoiseArgs &nz, const Grid3 &g, int a, int b, int cq) {
    u64 sc = (*nz.d_step) * 4096ull + nz.invocation;
    uint4 ctr = make_uint4((unsigned)((u64)b * g.N0 + a), (PURPOSE_POINT << 28) | (nz.level << 24) | (unsigned)cq,
                           (unsigned)sc, (unsigned)(sc >> 32));
    return normals4(philox4x32_10(ctr, noise_key(nz)));
}

template <typename T, bool EXACT>
__device__ __forceinline__ T rb_update(T xo, T xm, T xp, T ym, T yp, T zm, T zp, const StencilArg<T> &s, T fv,
                                       bool noisy, T xi) {
    typedef Ar<EXACT> A;
    // ascending linear index: z-, y-, x-, centre, x+, y+, z+
    T res = A::mul(s.w[4], zm);
    res = A::add(res, A::mul(s.w[10], ym));
    res = A::add(res, A::mul(s.w[12], xm));
    res = A::add(res, A::mul(s.w[13], xo));
    res = A::add(res, A::mul(s.w[14], xp));
    res = A::add(res, A::mul(s.w[16], yp));
    res = A::add(res, A::mul(s.w[22], zp));
    T cval = fv;
    if (noisy) cval = A::add(A::mul(s.sd, xi), cval);
    if (EXACT) return A::add(xo, A::mul(s.omega, A::sub(cval, res)) / s.diag);
    return xo + s.omega_diag * (cval - res);
}

template <typename T, bool EXACT, int NOISE>
__global__ void __launch_bounds__(RB_THREADS, 2) k_sweep_rb(const T *__restrict__ xin, T *__restrict__ xout,
                                                           const T *__restrict__ f, Grid3 g, StencilArg<T> s,
                                                           int first, int cz, NoiseArgs nz) {
    __shared__ T xo[3][RB_H2][RB_W2];
    __shared__ T Fr[3][RB_H1][RB_W1];
    const int a0 = blockIdx.x * RB_TX, b0 = blockIdx.y * RB_TY;
    const int c0 = blockIdx.z * cz, c1 = min(c0 + cz, g.N2);
    const int tx = threadIdx.x % RB_W1, ty = threadIdx.x / RB_W1;
    const int a = a0 - 1 + tx, b = b0 - 1 + ty;  // this thread's halo-1 column
    const bool col_in = (a >= 0 && a < g.N0 && b >= 0 && b < g.N1);
    const bool col_tile = col_in && tx >= 1 && tx <= RB_TX && ty >= 1 && ty <= RB_TY;
    auto slot = [](int c) { return ((c % 3) + 3) % 3; };
    // load old plane c (halo-2 region; ghosts read from the padded array,
    // positions beyond the ghost frame set to zero)
    auto load_plane = [&](int c) {
        T(*dst)[RB_W2] = xo[slot(c)];
        for (int i = threadIdx.x; i < RB_H2 * RB_W2; i += RB_THREADS) {
            int la = i % RB_W2, lb = i / RB_W2;
            int ga = a0 - 2 + la, gb = b0 - 2 + lb;
            T v = T(0);
            if (c >= 0 && c < g.N2 && ga >= 0 && ga < g.N0 && gb >= 0 && gb < g.N1) v = xin[g.pad(ga, gb, c)];
            dst[lb][la] = v;
        }
    };
    float4 nb_cur = make_float4(0.f, 0.f, 0.f, 0.f), nb_prev = nb_cur;
    int q_cur = -1000, q_prev = -1000;
    auto normal_at = [&](int c) -> T {
        int q = c >> 2;
        if (q == q_cur) return (T)pick(nb_cur, c & 3);
        if (q == q_prev) return (T)pick(nb_prev, c & 3);
        nb_prev = nb_cur;
        q_prev = q_cur;
        nb_cur = column_normals(nz, g, a, b, q);
        q_cur = q;
        return (T)pick(nb_cur, c & 3);
    };
    load_plane(c0 - 2);
    load_plane(c0 - 1);
    for (int kk = c0 - 1; kk <= c1; ++kk) {
        load_plane(kk + 1);
        __syncthreads();
        // 1. first colour of plane kk on the halo-1 region
        {
            T fval = T(0);
            if (kk >= 0 && kk < g.N2 && col_in && ((a + b + kk) & 1) == first) {
                const int lx = tx + 1, ly = ty + 1;
                const T(*P0)[RB_W2] = xo[slot(kk)];
                T xi = T(0);
                if (NOISE == NOISE_PHILOX) xi = normal_at(kk);
                if (NOISE == NOISE_INJECTED) xi = (T)nz.buf[g.compact(a, b, kk)];
                fval = rb_update<T, EXACT>(P0[ly][lx], P0[ly][lx - 1], P0[ly][lx + 1], P0[ly - 1][lx], P0[ly + 1][lx],
                                           xo[slot(kk - 1)][ly][lx], xo[slot(kk + 1)][ly][lx], s, f[g.pad(a, b, kk)],
                                           NOISE != NOISE_NONE, xi);
            }
            Fr[slot(kk)][ty][tx] = fval;  // zero off the first colour / outside
        }
        __syncthreads();
        // 2. finalise plane kk-1 on the tile
        const int c = kk - 1;
        if (c >= c0 && c < c1 && col_tile) {
            T out;
            if (((a + b + c) & 1) == first) {
                out = Fr[slot(c)][ty][tx];
            } else {
                const T(*F0)[RB_W1] = Fr[slot(c)];
                T xi = T(0);
                if (NOISE == NOISE_PHILOX) xi = normal_at(c);
                if (NOISE == NOISE_INJECTED) xi = (T)nz.buf[g.compact(a, b, c)];
                out = rb_update<T, EXACT>(xo[slot(c)][ty + 1][tx + 1], F0[ty][tx - 1], F0[ty][tx + 1], F0[ty - 1][tx],
                                          F0[ty + 1][tx], Fr[slot(c - 1)][ty][tx], Fr[slot(c + 1)][ty][tx], s,
                                          f[g.pad(a, b, c)], NOISE != NOISE_NONE, xi);
            }
            xout[g.pad(a, b, c)] = out;
        }
        __syncthreads();
    }
}

// ------------------------------------------------ lexicographic wavefront
// Lexicographic order as hyperplanes t = a + hb b + hc c: every neighbour
// that precedes a point lexicographically lies on an earlier hyperplane
// ((1,1,1) for axis stencils, (1,2,4) for 27-point stencils), points on one
// hyperplane are independent.  One CTA, one __syncthreads per hyperplane.
template <typename T, int NPT, bool EXACT, int NOISE>
__global__ void __launch_bounds__(1024) k_sweep_wavefront(T *__restrict__ x, const T *__restrict__ f, Grid3 g,
                                                           StencilArg<T> s, int forward, int hb, int hc, NoiseArgs nz) {
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

// Low-rank arguments of one level and sweep direction.
struct LowRankArg {
    int m;
    const i64 *Bptr;    // m+1, CSC of B (padded indices)
    const i64 *Bidx;
    const double *Bval;
    const double *Sinv; // m x m, (Sigma + B^T M^{-1} B)^{-1}
    const double *G;    // m x m, B^T M^{-1} B
    const double *sinv_sqrt; // Sigma^{-1/2}
    double *y;          // m scratch: B^T x
    double *z;          // m scratch: coefficients of C
    unsigned *counter;  // block-completion counter (self-resetting)
};

// y_j = sum_i B_ij x_i (one block per column j).  The last block to finish
// then forms
//   w = Sigma^{-1/2} xi',  z = w - S^{-1} (y + G w)
// (with_noise == 0: z = -S^{-1} y, the smoother's correction
// x -= Bbar B^T x of sor_smoother.cc:47-51, Bbar = C S^{-1}).
template <typename T, int NOISE, bool SOLVE>
__global__ void __launch_bounds__(256) k_bt_x_z(const T *__restrict__ x, LowRankArg lr, NoiseArgs nz) {
    __shared__ double sh[32];
    __shared__ bool last;
    const int j = blockIdx.x;
    double acc = 0.0;
    for (i64 e = lr.Bptr[j] + threadIdx.x; e < lr.Bptr[j + 1]; e += blockDim.x) acc += lr.Bval[e] * (double)x[lr.Bidx[e]];
    acc = block_sum<256>(acc, sh);
    if (threadIdx.x == 0) lr.y[j] = acc;
    if (!SOLVE) return;
    __threadfence();
    if (threadIdx.x == 0) {
        unsigned done = atomicAdd(lr.counter, 1u);
        last = (done == (unsigned)gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    extern __shared__ double dyn[];
    double *w = dyn, *v = dyn + lr.m;
    const int m = lr.m;
    for (int k = threadIdx.x; k < m; k += blockDim.x) {
        double xi = 0.0;
        if (NOISE == NOISE_PHILOX) {
            float4 r = normals4(philox4x32_10(noise_ctr(nz, (unsigned)(k >> 2), PURPOSE_LOWRANK, 0), noise_key(nz)));
            xi = (double)pick(r, k & 3);
        }
        if (NOISE == NOISE_INJECTED) xi = nz.buf[k];
        w[k] = lr.sinv_sqrt[k] * xi;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < m; k += blockDim.x) {
        double s = ((volatile double *)lr.y)[k];
        for (int q = 0; q < m; ++q) s += lr.G[(i64)k * m + q] * w[q];
        v[k] = s;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < m; k += blockDim.x) {
        double s = 0.0;
        for (int q = 0; q < m; ++q) s += lr.Sinv[(i64)k * m + q] * v[q];
        lr.z[k] = w[k] - s;
    }
    if (threadIdx.x == 0) *lr.counter = 0u;
}

// x[row] += sum_e C_e z_{col_e} over the support rows of C = M^{-1} B.
template <typename T>
__global__ void __launch_bounds__(256) k_lr_scatter(T *__restrict__ x, i64 nrows, const i64 *__restrict__ rows,
                                                     const i64 *__restrict__ ptr, const int *__restrict__ col,
                                                     const T *__restrict__ val, const double *__restrict__ z) {
    for (i64 r = (i64)blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += (i64)gridDim.x * blockDim.x) {
        T acc = T(0);
        for (i64 e = ptr[r]; e < ptr[r + 1]; ++e) acc += val[e] * (T)z[col[e]];
        x[rows[r]] += acc;
    }
}

// ------------------------------------------------- residual + restriction
// f_c(P_c) = sum_{a in {-1,0,1}^d} r(a) (f - A_0 x)(2 i_c + a),
// r(a) = prod {1/2, 1, 1/2}: IntergridOperator::restrict
// (intergrid_operator.hh:74-88) of the residual f - A_0 x
// (multigridmc_sampler.cc:124-126), with the stencil part of A.
template <typename T, int NPT>
__global__ void __launch_bounds__(256) k_resid_restrict(const T *__restrict__ x, const T *__restrict__ f,
                                                         T *__restrict__ fc, Grid3 gf, Grid3 gc, StencilArg<T> s,
                                                         int dim) {
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
                if (NPT == 7) {
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
}

// dst[row] += sign * sum_e B_e y_{col_e} / Sigma_{col_e} over the rows of B
// (row-compressed): the B Sigma^{-1} B^T x part of A x.
template <typename T>
__global__ void __launch_bounds__(256) k_add_Bq(T *__restrict__ dst, i64 nrows, const i64 *__restrict__ rows,
                                                 const i64 *__restrict__ ptr, const int *__restrict__ col,
                                                 const double *__restrict__ val, const double *__restrict__ y,
                                                 const double *__restrict__ sigma_inv, double sign) {
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
__global__ void __launch_bounds__(256) k_prolong_add(T *__restrict__ x, const T *__restrict__ xc, Grid3 gf, Grid3 gc,
                                                      T alpha, int dim) {
    i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
    i64 n = (i64)gf.N0 * gf.N1 * gf.N2;
    if (t >= n) return;
    int co[3] = {(int)(t % gf.N0) + 1, (int)((t / gf.N0) % gf.N1) + 1, (int)(t / ((i64)gf.N0 * gf.N1)) + 1};
    int lo[3], np[3];
    T wt[3];
    for (int d = 0; d < 3; ++d) {
        if (d >= dim) {
            lo[d] = 1;
            np[d] = 1;
            wt[d] = T(1);
        } else if ((co[d] & 1) == 0) {
            lo[d] = co[d] >> 1;
            np[d] = 1;
            wt[d] = T(1);
        } else {
            lo[d] = co[d] >> 1;
            np[d] = 2;
            wt[d] = T(0.5);
        }
    }
    T acc = T(0);
    for (int k = 0; k < np[2]; ++k)
        for (int j = 0; j < np[1]; ++j)
            for (int i = 0; i < np[0]; ++i)
                acc += wt[0] * wt[1] * wt[2] * xc[(i64)(lo[2] + k) * gc.sz + (i64)(lo[1] + j) * gc.sy + (lo[0] + i)];
    i64 P = (i64)co[2] * gf.sz + (i64)co[1] * gf.sy + co[0];
    x[P] += alpha * acc;
}

// ----------------------------------------------------- stencil apply
// y = A_0 x (LinearOperator::apply without the low-rank term).
template <typename T>
__global__ void __launch_bounds__(256) k_apply_stencil(const T *__restrict__ x, T *__restrict__ y, Grid3 g,
                                                        StencilArg<T> s) {
    i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
    i64 n = (i64)g.N0 * g.N1 * g.N2;
    if (t >= n) return;
    int a = (int)(t % g.N0), b = (int)((t / g.N0) % g.N1), c = (int)(t / ((i64)g.N0 * g.N1));
    i64 P = g.pad(a, b, c);
    T res = T(0);
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) res += s.w[(dz + 1) * 9 + (dy + 1) * 3 + (dx + 1)] * x[P + dz * g.sz + dy * g.sy + dx];
    y[P] = res;
}

// ---------------------------------------------------- layout conversion
template <typename T>
__global__ void k_unpack(const double *__restrict__ src, T *__restrict__ dst, Grid3 g) {
    i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
    i64 n = (i64)g.N0 * g.N1 * g.N2;
    if (t >= n) return;
    int a = (int)(t % g.N0), b = (int)((t / g.N0) % g.N1), c = (int)(t / ((i64)g.N0 * g.N1));
    dst[g.pad(a, b, c)] = (T)src[t];
}

template <typename T>
__global__ void k_pack(const T *__restrict__ src, double *__restrict__ dst, Grid3 g) {
    i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
    i64 n = (i64)g.N0 * g.N1 * g.N2;
    if (t >= n) return;
    int a = (int)(t % g.N0), b = (int)((t / g.N0) % g.N1), c = (int)(t / ((i64)g.N0 * g.N1));
    dst[t] = (double)src[g.pad(a, b, c)];
}

template <typename T>
__global__ void k_zero_interior(T *__restrict__ x, Grid3 g) {
    i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
    i64 n = (i64)g.N0 * g.N1 * g.N2;
    if (t >= n) return;
    int a = (int)(t % g.N0), b = (int)((t / g.N0) % g.N1), c = (int)(t / ((i64)g.N0 * g.N1));
    x[g.pad(a, b, c)] = T(0);
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

// Throughput form with the explicit inverse factor Linv = L^{-1}:
// v = xi + Linv f (warp per row, row i has i+1 non-zeros) ...
template <typename T, int NOISE>
__global__ void __launch_bounds__(256) k_chol_gemv_lower(const T *__restrict__ f, Grid3 g, const double *__restrict__ Linv,
                                                          double *__restrict__ v, NoiseArgs nz) {
    extern __shared__ double fs[];
    const i64 n = (i64)g.N0 * g.N1 * g.N2;
    for (i64 i = threadIdx.x; i < n; i += blockDim.x) {
        int a = (int)(i % g.N0), b = (int)((i / g.N0) % g.N1), c = (int)(i / ((i64)g.N0 * g.N1));
        fs[i] = (double)f[g.pad(a, b, c)];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const i64 warps = (i64)gridDim.x * (blockDim.x >> 5);
    for (i64 i = (i64)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
        const double *row = Linv + i * n;
        double acc = 0.0;
        for (i64 k = lane; k <= i; k += 32) acc += row[k] * fs[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) {
            double xi = 0.0;
            if (NOISE == NOISE_INJECTED) xi = nz.buf[i];
            if (NOISE == NOISE_PHILOX) {
                float4 r = normals4(philox4x32_10(noise_ctr(nz, (unsigned)(i >> 2), PURPOSE_COARSE, 0), noise_key(nz)));
                xi = (double)pick(r, (int)(i & 3));
            }
            v[i] = xi + acc;
        }
    }
}

// ... x = Linv^T v (row j of Linv^T has non-zeros j..n-1).
template <typename T>
__global__ void __launch_bounds__(256) k_chol_gemv_upper(const double *__restrict__ v, Grid3 g,
                                                          const double *__restrict__ LinvT, T *__restrict__ x) {
    extern __shared__ double vs[];
    const i64 n = (i64)g.N0 * g.N1 * g.N2;
    for (i64 i = threadIdx.x; i < n; i += blockDim.x) vs[i] = v[i];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const i64 warps = (i64)gridDim.x * (blockDim.x >> 5);
    for (i64 j = (i64)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); j < n; j += warps) {
        const double *row = LinvT + j * n;
        double acc = 0.0;
        for (i64 k = j + lane; k < n; k += 32) acc += row[k] * vs[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) {
            int a = (int)(j % g.N0), b = (int)((j / g.N0) % g.N1), c = (int)(j / ((i64)g.N0 * g.N1));
            x[g.pad(a, b, c)] = (T)acc;
        }
    }
}

// ------------------------------------------------------------ step end
// Observable z = b^T x of measure_sampling_time (sampling_time.cc:40),
// stored at obs[count] while count < capacity; a non-finite value raises
// the error flag.  Then the step counter that keys the Philox streams
// advances.  One CTA; runs after every other kernel of the step.
template <typename T>
__global__ void __launch_bounds__(256) k_step_end(const T *__restrict__ x, i64 nb, const i64 *__restrict__ bidx,
                                                   const double *__restrict__ bval, double *__restrict__ obs,
                                                   i64 capacity, u64 *__restrict__ obs_count,
                                                   u64 *__restrict__ d_step, unsigned *__restrict__ err) {
    __shared__ double sh[32];
    double acc = 0.0;
    for (i64 e = threadIdx.x; e < nb; e += blockDim.x) acc += bval[e] * (double)x[bidx[e]];
    acc = block_sum<256>(acc, sh);
    if (threadIdx.x == 0) {
        if (nb > 0) {
            u64 k = *obs_count;
            if ((i64)k < capacity) obs[k] = acc;
            *obs_count = k + 1;
            if (!isfinite(acc)) atomicOr(err, 1u);
        }
        *d_step += 1ull;
    }
}

}  // namespace mgmc
