// kernels.cuh -- sm_103a kernels of the Multigrid Monte Carlo step.
//
// Data layout (every level): padded lexicographic arrays with shared ghost
// rows/planes, see Geometry in setup.h.  A point with 0-based interior
// coordinates (a, b, c) lives at P = (c+1) sz + (b+1) sy + (a+1); ghosts are
// zero, so stencil loads need no boundary tests.
//
// Kernels (one V-cycle at level l uses them in this order):
//   k_sweep_rb          red-black SOR sweep of the fine 7-point level, both
//                       colours in one pass (multicolour order)
//   k_sweep_planes      8-colour SOR sweep of a 27-point level, one launch per
//                       plane parity (multicolour order)
//   k_sweep_wavefront   lexicographic SOR sweep as a hyperplane wavefront
//                       (one CTA; parity mode)
//   k_bt_x_z            y = B^T x and the m x m low-rank solve
//   k_lr_scatter        x += C z over the rows of C = M^{-1} B
//   k_resid_restrict_tiled  f_c = R (f - A_0 x)  (fused residual + restriction)
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
constexpr int RB_TX = 62, RB_TY = 14;                 // interior tile
constexpr int RB_W1 = RB_TX + 2, RB_H1 = RB_TY + 2;  // tile + halo 1 (F): 64 x 16
constexpr int RB_W2 = RB_TX + 4, RB_H2 = RB_TY + 4;  // tile + halo 2 (old x): 66 x 18
constexpr int RB_THREADS = (RB_W1 / 2) * RB_H1;       // 512: one thread per pair of halo-1 columns
constexpr int RB_NLD = (RB_W2 * RB_H2 + RB_THREADS - 1) / RB_THREADS;

__device__ __forceinline__ float4 column_normals(const NoiseArgs &nz, const Grid3 &g, int a, int b, int cq) {
    u64 sc = (*nz.d_step) * 4096ull + nz.invocation;
    uint4 ctr = make_uint4((unsigned)((u64)b * g.N0 + a), (PURPOSE_POINT << 28) | (nz.level << 24) | (unsigned)cq,
                           (unsigned)sc, (unsigned)(sc >> 32));
    return normals4(philox4x32_10(ctr, noise_key(nz)));
}

// Normals of one lattice column, four planes per Philox block; planes are
// requested in (nearly) ascending order, so two cached blocks suffice.
struct ColumnNoise {
    float4 cur, prev;
    int qcur, qprev;
    __device__ void init() {
        qcur = qprev = -1000;
        cur = prev = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __device__ __forceinline__ float get(const NoiseArgs &nz, const Grid3 &g, int a, int b, int c) {
        int q = c >> 2;
        if (q == qcur) return pick(cur, c & 3);
        if (q == qprev) return pick(prev, c & 3);
        prev = cur;
        qprev = qcur;
        cur = column_normals(nz, g, a, b, q);
        qcur = q;
        return pick(cur, c & 3);
    }
};

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

// Thread = pair of adjacent halo-1 columns (one of each colour on every
// plane), so both colours' work is spread evenly over the lanes.  Per plane
// kk:  [A] first colour of plane kk on the halo-1 region,  [B] sync,
// [C] second colour of plane kk-1 and both colours written out,  [D] the
// old plane kk+2 (loaded into registers one plane earlier) stored to shared
// memory,  [E] plane kk+3 loaded into registers,  [F] sync.  The global
// load latency is hidden behind one plane of work.
template <typename T>
constexpr size_t rb_smem_bytes() {
    return sizeof(T) * (4 * RB_H2 * RB_W2 + 3 * RB_H1 * RB_W1);
}

template <typename T, bool EXACT, int NOISE>
__global__ void __launch_bounds__(RB_THREADS, 2) k_sweep_rb(const T *__restrict__ xin, T *__restrict__ xout,
                                                           const T *__restrict__ f, Grid3 g, StencilArg<T> s,
                                                           int first, int cz, NoiseArgs nz) {
    extern __shared__ __align__(16) unsigned char rb_smem[];
    T(*xo)[RB_H2][RB_W2] = reinterpret_cast<T(*)[RB_H2][RB_W2]>(rb_smem);
    T(*Fr)[RB_H1][RB_W1] = reinterpret_cast<T(*)[RB_H1][RB_W1]>(rb_smem + sizeof(T) * 4 * RB_H2 * RB_W2);
    const int a0 = blockIdx.x * RB_TX, b0 = blockIdx.y * RB_TY;
    const int c0 = blockIdx.z * cz, c1 = min(c0 + cz, g.N2);
    const int px = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int b = b0 - 1 + ty;
    const bool row_in = b >= 0 && b < g.N1;
    const bool row_tile = row_in && ty >= 1 && ty <= RB_TY;
    int ac[2];
    bool cin[2], ctile[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int tx = 2 * px + h;
        ac[h] = a0 - 1 + tx;
        cin[h] = row_in && ac[h] >= 0 && ac[h] < g.N0;
        ctile[h] = row_tile && cin[h] && tx >= 1 && tx <= RB_TX;
    }
    ColumnNoise cn[2];
    cn[0].init();
    cn[1].init();
    T pre[RB_NLD];
    auto fetch = [&](int c) {
#pragma unroll
        for (int j = 0; j < RB_NLD; ++j) {
            const int i = threadIdx.x + j * RB_THREADS;
            T v = T(0);
            if (i < RB_W2 * RB_H2) {
                const int la = i % RB_W2, lb = i / RB_W2;
                const int ga = a0 - 2 + la, gb = b0 - 2 + lb;
                if (c >= 0 && c < g.N2 && ga >= 0 && ga < g.N0 && gb >= 0 && gb < g.N1) v = xin[g.pad(ga, gb, c)];
            }
            pre[j] = v;
        }
    };
    auto commit = [&](int c) {
#pragma unroll
        for (int j = 0; j < RB_NLD; ++j) {
            const int i = threadIdx.x + j * RB_THREADS;
            if (i < RB_W2 * RB_H2) xo[c & 3][i / RB_W2][i % RB_W2] = pre[j];
        }
    };
    auto s3 = [](int c) { return ((c % 3) + 3) % 3; };
    fetch(c0 - 2);
    commit(c0 - 2);
    fetch(c0 - 1);
    commit(c0 - 1);
    fetch(c0);
    commit(c0);
    fetch(c0 + 1);
    __syncthreads();
    for (int kk = c0 - 1; kk <= c1; ++kk) {
        // [A] first colour of plane kk
        const bool plane_in = kk >= 0 && kk < g.N2;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int tx = 2 * px + h, a = ac[h];
            T fval = T(0);
            if (plane_in && cin[h] && ((a + b + kk) & 1) == first) {
                const int lx = tx + 1, ly = ty + 1;
                T xi = T(0);
                if (NOISE == NOISE_PHILOX) xi = (T)cn[h].get(nz, g, a, b, kk);
                if (NOISE == NOISE_INJECTED) xi = (T)nz.buf[g.compact(a, b, kk)];
                fval = rb_update<T, EXACT>(xo[kk & 3][ly][lx], xo[kk & 3][ly][lx - 1], xo[kk & 3][ly][lx + 1],
                                           xo[kk & 3][ly - 1][lx], xo[kk & 3][ly + 1][lx], xo[(kk - 1) & 3][ly][lx],
                                           xo[(kk + 1) & 3][ly][lx], s, f[g.pad(a, b, kk)], NOISE != NOISE_NONE, xi);
            }
            Fr[s3(kk)][ty][tx] = fval;
        }
        __syncthreads();
        // [C] second colour of plane c = kk-1, both colours written
        const int c = kk - 1;
        if (c >= c0 && c < c1) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                if (!ctile[h]) continue;
                const int tx = 2 * px + h, a = ac[h];
                T out;
                if (((a + b + c) & 1) == first) {
                    out = Fr[s3(c)][ty][tx];
                } else {
                    T xi = T(0);
                    if (NOISE == NOISE_PHILOX) xi = (T)cn[h].get(nz, g, a, b, c);
                    if (NOISE == NOISE_INJECTED) xi = (T)nz.buf[g.compact(a, b, c)];
                    out = rb_update<T, EXACT>(xo[c & 3][ty + 1][tx + 1], Fr[s3(c)][ty][tx - 1], Fr[s3(c)][ty][tx + 1],
                                              Fr[s3(c)][ty - 1][tx], Fr[s3(c)][ty + 1][tx], Fr[s3(c - 1)][ty][tx],
                                              Fr[s3(c + 1)][ty][tx], s, f[g.pad(a, b, c)], NOISE != NOISE_NONE, xi);
                }
                xout[g.pad(a, b, c)] = out;
            }
        }
        // [D], [E]
        commit(kk + 2);
        fetch(kk + 3);
        __syncthreads();
    }
}

// Multicolour sweep of a 2^dim-colour (9- / 27-point) level organised by
// planes: the colours with z-parity p touch no other plane of parity p, so
// one launch updates all planes of one parity, one CTA per plane running the
// plane's four in-plane colours separated by __syncthreads.  The update
// order and the noise are those of the colour-by-colour sweep (colour index
// (a & 1) | (b & 1) << 1 | (c & 1) << 2, ascending forward, descending
// backward), so the chain is the same.
template <typename T, bool EXACT, int NOISE>
__global__ void __launch_bounds__(512) k_sweep_planes(T *__restrict__ x, const T *__restrict__ f, Grid3 g,
                                                       StencilArg<T> s, int zpar, int forward, NoiseArgs nz) {
    const int c = 2 * blockIdx.x + zpar;
    if (c >= g.N2) return;
    const int G0 = (g.N0 + 7) >> 3;
    for (int cc = 0; cc < 4; ++cc) {
        const int col2 = forward ? cc : 3 - cc;
        const int pa = col2 & 1, pb = col2 >> 1;
        const int nb = (g.N1 - pb + 1) >> 1;
        for (int t = threadIdx.x; t < nb * G0; t += blockDim.x) {
            const int grp = t % G0, b = 2 * (t / G0) + pb;
            float4 nrm = make_float4(0.f, 0.f, 0.f, 0.f);
            if (NOISE == NOISE_PHILOX) nrm = point_normals(nz, g, 8 * grp + pa, b, c);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int a = 8 * grp + pa + 2 * q;
                if (a >= g.N0) break;
                T xi = T(0);
                if (NOISE == NOISE_PHILOX) xi = (T)pick(nrm, q);
                if (NOISE == NOISE_INJECTED) xi = (T)nz.buf[g.compact(a, b, c)];
                sor_point<T, 27, EXACT>(x, f, g, s, g.pad(a, b, c), NOISE != NOISE_NONE, xi);
            }
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
    double *part;       // m x gridDim.y scratch: partial sums of B^T x
    unsigned *counter;  // block-completion counter (self-resetting)
};

// y_j = sum_i B_ij x_i with gridDim.y blocks per column j (partial sums in
// `part`, combined in a fixed order by the last block to finish, so the
// result does not depend on block timing).  With SOLVE the same block then
// forms
//   w = Sigma^{-1/2} xi',  z = w - S^{-1} (y + G w)
// (with_noise == 0: z = -S^{-1} y, the smoother's correction
// x -= Bbar B^T x of sor_smoother.cc:47-51, Bbar = C S^{-1}).
template <typename T, int NOISE, bool SOLVE>
__global__ void __launch_bounds__(256) k_bt_x_z(const T *__restrict__ x, LowRankArg lr, NoiseArgs nz) {
    __shared__ double sh[32];
    __shared__ bool last;
    const int j = blockIdx.x, p = blockIdx.y, P = gridDim.y;
    const i64 e0 = lr.Bptr[j], e1 = lr.Bptr[j + 1];
    const i64 len = (e1 - e0 + P - 1) / P;
    const i64 lo = e0 + p * len, hi = min(e1, lo + len);
    double acc = 0.0;
    for (i64 e = lo + threadIdx.x; e < hi; e += blockDim.x) acc += lr.Bval[e] * (double)x[lr.Bidx[e]];
    acc = block_sum<256>(acc, sh);
    if (threadIdx.x == 0) lr.part[j * P + p] = acc;
    __threadfence();
    if (threadIdx.x == 0) {
        unsigned done = atomicAdd(lr.counter, 1u);
        last = (done == gridDim.x * gridDim.y - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    const int m = lr.m;
    for (int k = threadIdx.x; k < m; k += blockDim.x) {
        double t = 0.0;
        for (int q = 0; q < P; ++q) t += ((volatile double *)lr.part)[k * P + q];
        lr.y[k] = t;
    }
    if (threadIdx.x == 0) *lr.counter = 0u;
    if (!SOLVE) return;
    __syncthreads();
    extern __shared__ double dyn[];
    double *w = dyn, *v = dyn + m;
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
        double t = lr.y[k];
        for (int q = 0; q < m; ++q) t += lr.G[(i64)k * m + q] * w[q];
        v[k] = t;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < m; k += blockDim.x) {
        double t = 0.0;
        for (int q = 0; q < m; ++q) t += lr.Sinv[(i64)k * m + q] * v[q];
        lr.z[k] = w[k] - t;
    }
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

// Plane-streaming variant: a CTA owns a tile of RR_TX x RR_TY coarse
// columns and a range of coarse planes.  Fine residual planes are computed
// once each on the (2 RR_TX + 1) x (2 RR_TY + 1) fine footprint of the tile
// and kept in a ring of three planes; every coarse plane then restricts from
// the ring.  x is staged plane by plane with a one-point halo.
constexpr int RR_TX = 16, RR_TY = 8;
constexpr int RR_FW = 2 * RR_TX + 1, RR_FH = 2 * RR_TY + 1;  // fine residual footprint
constexpr int RR_XW = RR_FW + 2, RR_XH = RR_FH + 2;          // x with halo
constexpr int RR_THREADS = 256;

template <typename T, int NPT>
__global__ void __launch_bounds__(RR_THREADS) k_resid_restrict_tiled(const T *__restrict__ x, const T *__restrict__ f,
                                                                      T *__restrict__ fc, Grid3 gf, Grid3 gc,
                                                                      StencilArg<T> s, int czc) {
    __shared__ T xs[3][RR_XH][RR_XW];
    __shared__ T rs[3][RR_FH][RR_FW];
    const int ca0 = blockIdx.x * RR_TX, cb0 = blockIdx.y * RR_TY;
    const int cc0 = blockIdx.z * czc, cc1 = min(cc0 + czc, gc.N2);
    // fine 0-based origin of the footprint: centre of coarse (ca0, cb0) is
    // fine 2 ca0 + 1, its left neighbour 2 ca0
    const int fa0 = 2 * ca0, fb0 = 2 * cb0;
    auto slot = [](int p) { return ((p % 3) + 3) % 3; };
    auto load_x = [&](int p) {
        T(*dst)[RR_XW] = xs[slot(p)];
        for (int i = threadIdx.x; i < RR_XH * RR_XW; i += RR_THREADS) {
            int la = i % RR_XW, lb = i / RR_XW;
            int ga = fa0 - 1 + la, gb = fb0 - 1 + lb;
            T v = T(0);
            if (p >= 0 && p < gf.N2 && ga >= 0 && ga < gf.N0 && gb >= 0 && gb < gf.N1) v = x[gf.pad(ga, gb, p)];
            dst[lb][la] = v;
        }
    };
    auto resid_plane = [&](int p) {  // fine residual of plane p on the footprint
        T(*dst)[RR_FW] = rs[slot(p)];
        for (int i = threadIdx.x; i < RR_FH * RR_FW; i += RR_THREADS) {
            int la = i % RR_FW, lb = i / RR_FW;
            int ga = fa0 + la, gb = fb0 + lb;
            T r = T(0);
            if (p >= 0 && p < gf.N2 && ga < gf.N0 && gb < gf.N1) {
                const int X = la + 1, Y = lb + 1;
                T res;
                if (NPT == 7) {
                    res = s.w[4] * xs[slot(p - 1)][Y][X] + s.w[10] * xs[slot(p)][Y - 1][X] + s.w[12] * xs[slot(p)][Y][X - 1] +
                          s.w[13] * xs[slot(p)][Y][X] + s.w[14] * xs[slot(p)][Y][X + 1] + s.w[16] * xs[slot(p)][Y + 1][X] +
                          s.w[22] * xs[slot(p + 1)][Y][X];
                } else {
                    res = T(0);
#pragma unroll
                    for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
                        for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
                            for (int dx = -1; dx <= 1; ++dx)
                                res += s.w[(dz + 1) * 9 + (dy + 1) * 3 + (dx + 1)] * xs[slot(p + dz)][Y + dy][X + dx];
                }
                r = f[gf.pad(ga, gb, p)] - res;
            }
            dst[lb][la] = r;
        }
    };
    // coarse plane cc needs fine residual planes 2cc, 2cc+1, 2cc+2
    const int p_lo = 2 * cc0, p_hi = 2 * (cc1 - 1) + 2;
    load_x(p_lo - 1);
    load_x(p_lo);
    for (int p = p_lo; p <= p_hi; ++p) {
        load_x(p + 1);
        __syncthreads();
        resid_plane(p);
        __syncthreads();
        if (p >= p_lo + 2 && ((p - p_lo) & 1) == 0) {  // restrict coarse plane (p - 2) / 2
            const int cc = (p - 2) / 2;
            for (int i = threadIdx.x; i < RR_TX * RR_TY; i += RR_THREADS) {
                int la = i % RR_TX, lb = i / RR_TX;
                int ca = ca0 + la, cb = cb0 + lb;
                if (ca >= gc.N0 || cb >= gc.N1) continue;
                T acc = T(0);
#pragma unroll
                for (int az = 0; az < 3; ++az)
#pragma unroll
                    for (int ay = 0; ay < 3; ++ay)
#pragma unroll
                        for (int ax = 0; ax < 3; ++ax) {
                            T wr = T((ax == 1 ? 1.0 : 0.5) * (ay == 1 ? 1.0 : 0.5) * (az == 1 ? 1.0 : 0.5));
                            acc += wr * rs[slot(2 * cc + az)][2 * lb + ay][2 * la + ax];
                        }
                fc[gc.pad(ca, cb, cc)] = acc;
            }
        }
        __syncthreads();
    }
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
__global__ void __launch_bounds__(128) k_prolong_add(T *__restrict__ x, const T *__restrict__ xc, Grid3 gf, Grid3 gc,
                                                      T alpha, int dim) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= gf.N0) return;
    int co[3] = {a + 1, (int)blockIdx.y + 1, (int)blockIdx.z + 1};
    int lo[3], np[3];
    T wt[3];
#pragma unroll
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
    const i64 P = (i64)co[2] * gf.sz + (i64)co[1] * gf.sy + co[0];
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
