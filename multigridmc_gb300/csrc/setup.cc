// setup.cc -- host-side set-up of the multigrid hierarchy.
#include "setup.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace mgmc {

Geometry::Geometry(int dim_, int nx, int ny, int nz) : dim(dim_) {
    c[0] = nx;
    c[1] = dim > 1 ? ny : 2;
    c[2] = dim > 2 ? nz : 2;
    for (int d = 0; d < 3; ++d) N[d] = c[d] - 1;
    n = (int64_t)N[0] * N[1] * N[2];
    sy = c[0];
    sz = (int64_t)c[0] * c[1];
    nalloc = (int64_t)(c[2] + 2) * sz + 32;
}

// Lattice3d::get_coarse_lattice (src/lattice/lattice3d.hh:248-263)
bool Geometry::coarsenable() const {
    for (int d = 0; d < dim; ++d)
        if (c[d] % 2 != 0 || c[d] / 2 <= 1) return false;
    return true;
}

Geometry Geometry::coarse() const { return Geometry(dim, c[0] / 2, c[1] / 2, c[2] / 2); }

double Geometry::cell_volume() const {  // Lattice::cell_volume, src/lattice/lattice.hh:36-44
    double v = 1.0;
    for (int d = 0; d < dim; ++d) v /= c[d];
    return v;
}

static inline int sidx(int dx, int dy, int dz) { return (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1); }

// ShiftedLaplaceFDOperator (src/linear_operator/shiftedlaplace_fd_operator.cc:9-57):
// every operation in the order of the reference so that the FP64 values are
// the reference's bit for bit.
void fd_stencil(const Geometry &g, double kappa_sq, double st[27]) {
    for (int k = 0; k < 27; ++k) st[k] = 0.0;
    double hinv2[3] = {0.0, 0.0, 0.0};
    double cell_volume = 1.0;
    for (int d = 0; d < g.dim; ++d) {
        double h = 1. / double(g.c[d]);
        hinv2[d] = 1. / (h * h);
        cell_volume *= h;
    }
    double diagonal = cell_volume * kappa_sq;
    for (int d = 0; d < g.dim; ++d) {
        int o[3] = {0, 0, 0};
        o[d] = -1;
        st[sidx(o[0], o[1], o[2])] = -cell_volume * hinv2[d];
        o[d] = 1;
        st[sidx(o[0], o[1], o[2])] = -cell_volume * hinv2[d];
        diagonal += 2. * cell_volume * hinv2[d];
    }
    st[13] = diagonal;
}

// 1d weight of the linear intergrid stencil {1/2, 1, 1/2}
// (src/intergrid/intergrid_operator_linear.cc:13-29); inactive directions
// carry the identity.
static inline double rweight(int o, bool active) {
    if (!active) return o == 0 ? 1.0 : 0.0;
    if (o == 0) return 1.0;
    if (o == 1 || o == -1) return 0.5;
    return 0.0;
}

// Galerkin product A_c = R A P for a translation-invariant stencil:
//   W_c(s) = sum_{a,b} r(a) W(b) r(a + b - 2 s).
// With homogeneous Dirichlet boundaries the zero-extended fine field equals
// the reference's truncated stencil rows, so the coarse operator of
// linear_operator.cc:10-23 is this stencil on every coarse vertex.
void galerkin_stencil(int dim, const double fine[27], double coarse[27]) {
    bool act[3] = {dim > 0, dim > 1, dim > 2};
    for (int sz = -1; sz <= 1; ++sz)
        for (int sy = -1; sy <= 1; ++sy)
            for (int sx = -1; sx <= 1; ++sx) {
                double acc = 0.0;
                for (int az = -1; az <= 1; ++az)
                    for (int ay = -1; ay <= 1; ++ay)
                        for (int ax = -1; ax <= 1; ++ax) {
                            double ra = rweight(ax, act[0]) * rweight(ay, act[1]) * rweight(az, act[2]);
                            if (ra == 0.0) continue;
                            for (int bz = -1; bz <= 1; ++bz)
                                for (int by = -1; by <= 1; ++by)
                                    for (int bx = -1; bx <= 1; ++bx) {
                                        double w = fine[sidx(bx, by, bz)];
                                        if (w == 0.0) continue;
                                        double rp = rweight(ax + bx - 2 * sx, act[0]) * rweight(ay + by - 2 * sy, act[1]) *
                                                    rweight(az + bz - 2 * sz, act[2]);
                                        acc += ra * w * rp;
                                    }
                        }
                coarse[sidx(sx, sy, sz)] = acc;
            }
}

int colour_count(int dim, const double st[27]) {
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                int nz = (dx != 0) + (dy != 0) + (dz != 0);
                if (nz > 1 && st[sidx(dx, dy, dz)] != 0.0) return 1 << dim;
            }
    return 2;
}

// ------------------------------------------------ measurement quadrature
// V_d(R) recursion (src/linear_operator/measured_operator.cc:50-66)
static double V_sphere(double radius, int dim) {
    if (dim == 0) return 1.0;
    if (dim == 1) return 2. * radius;
    return 2. * M_PI / double(dim) * radius * radius * V_sphere(radius, dim - 2);
}

static double dist(const double *a, const double *b, int dim) {
    double s = 0.0;
    for (int d = 0; d < dim; ++d) s += (a[d] - b[d]) * (a[d] - b[d]);
    return std::sqrt(s);
}

// measurement_vector (src/linear_operator/measured_operator.cc:69-171) with
// the 2-point Gauss-Legendre rule of src/auxilliary/quadrature.cc:11-56.
// Only cells within the bounding box of the ball are visited; every cell
// outside it fails the reference's overlap test.
std::map<int64_t, double> measurement_vector(const Geometry &g, const double *x0, double radius) {
    std::map<int64_t, double> r;
    const int dim = g.dim;
    if (radius < 1.E-12) {  // nearest vertex, first one wins on ties
        double d_min = double(dim);
        int64_t best = 0;
        for (int64_t ell = 0; ell < g.n; ++ell) {
            int64_t nxy = (int64_t)g.N[0] * g.N[1];
            int64_t idx[3] = {(ell % nxy) % g.N[0] + 1, (ell % nxy) / g.N[0] + 1, ell / nxy + 1};
            double x[3];
            for (int d = 0; d < dim; ++d) x[d] = idx[d] * (1. / double(g.c[d]));
            double dd = dist(x, x0, dim);
            if (dd < d_min) {
                d_min = dd;
                best = ell;
            }
        }
        r[best] = 1.0;
        return r;
    }
    double h[3] = {0, 0, 0};
    for (int d = 0; d < dim; ++d) h[d] = 1. / double(g.c[d]);
    const double cell_volume = g.cell_volume();
    const double normalisation = 1. / V_sphere(radius, dim);
    // quadrature points/weights on [0,1]^d, first direction slowest
    const double q1[2] = {0.5 * (-1.0 / std::sqrt(3.0) + 1.0), 0.5 * (1.0 / std::sqrt(3.0) + 1.0)};
    const int nq = 1 << dim;
    std::vector<std::array<double, 3>> qp(nq);
    std::vector<double> qw(nq);
    for (int q = 0; q < nq; ++q) {
        double w = 1.0;
        for (int d = 0; d < dim; ++d) {
            int bit = (q >> (dim - 1 - d)) & 1;
            qp[q][d] = q1[bit];
            w *= 0.5 * 1.0;
        }
        qw[q] = w;
    }
    int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int d = 0; d < 3; ++d) {
        if (d < dim) {
            lo[d] = std::max(0, (int)std::floor((x0[d] - radius) / h[d]) - 1);
            hi[d] = std::min(g.c[d] - 1, (int)std::floor((x0[d] + radius) / h[d]) + 1);
        }
    }
    for (int cz = lo[2]; cz <= hi[2]; ++cz)
        for (int cy = lo[1]; cy <= hi[1]; ++cy)
            for (int cx = lo[0]; cx <= hi[0]; ++cx) {
                int cc[3] = {cx, cy, cz};
                bool overlap = false;
                double xmin[3] = {2.0, 2.0, 2.0}, xmax[3] = {-1.0, -1.0, -1.0};
                for (int q = 0; q < nq; ++q) {
                    double xc[3];
                    for (int d = 0; d < dim; ++d) {
                        int om = (q >> (dim - 1 - d)) & 1;
                        xc[d] = h[d] * double(cc[d] + om);
                        xmin[d] = std::min(xmin[d], xc[d]);
                        xmax[d] = std::max(xmax[d], xc[d]);
                    }
                    overlap = overlap || (dist(xc, x0, dim) < radius);
                }
                bool centre_in_cell = true;
                for (int d = 0; d < dim; ++d)
                    centre_in_cell = centre_in_cell && (xmin[d] <= x0[d]) && (x0[d] <= xmax[d]);
                overlap = overlap || centre_in_cell;
                if (!overlap) continue;
                for (int a = 0; a < nq; ++a) {  // corners, first direction slowest
                    int alpha[3] = {0, 0, 0};
                    int v[3] = {1, 1, 1};
                    bool interior = true;
                    for (int d = 0; d < dim; ++d) {
                        alpha[d] = (a >> (dim - 1 - d)) & 1;
                        v[d] = cc[d] + alpha[d];
                        if (v[d] <= 0 || v[d] >= g.c[d]) interior = false;
                    }
                    if (!interior) continue;
                    int64_t ell = ((int64_t)(v[2] - 1) * g.N[1] + (v[1] - 1)) * g.N[0] + (v[0] - 1);
                    double local_entry = 0.0;
                    for (int q = 0; q < nq; ++q) {
                        double x[3];
                        for (int d = 0; d < dim; ++d) x[d] = h[d] * (qp[q][d] + double(cc[d]));
                        double xi = dist(x, x0, dim) / radius;
                        if (xi < 1.0) {
                            double phihat = 1.0;
                            for (int d = 0; d < dim; ++d) phihat *= (alpha[d] == 0) ? (1.0 - qp[q][d]) : qp[q][d];
                            local_entry += phihat * qw[q] * cell_volume * normalisation;
                        }
                    }
                    r[ell] += local_entry;
                }
            }
    return r;
}

// B_c = R B (src/linear_operator/linear_operator.cc:19): coarse vertex ic
// gathers fine vertices 2 ic + a with weight prod_d {1/2, 1, 1/2}[a_d].
SparseCols restrict_columns(const Geometry &fine, const SparseCols &B) {
    Geometry cg = fine.coarse();
    SparseCols out;
    out.m = B.m;
    out.ptr.assign(1, 0);
    const int64_t nxy = (int64_t)fine.N[0] * fine.N[1];
    for (int j = 0; j < B.m; ++j) {
        std::map<int64_t, double> col;
        for (int64_t e = B.ptr[j]; e < B.ptr[j + 1]; ++e) {
            int64_t ell = B.row[e];
            int f[3] = {(int)((ell % nxy) % fine.N[0]) + 1, (int)((ell % nxy) / fine.N[0]) + 1, (int)(ell / nxy) + 1};
            // candidate coarse parents in each direction
            int cand[3][2], w2[3][2], nc[3];
            double wt[3][2];
            for (int d = 0; d < 3; ++d) {
                if (d >= fine.dim) {
                    nc[d] = 1;
                    cand[d][0] = 1;
                    wt[d][0] = 1.0;
                    continue;
                }
                if (f[d] % 2 == 0) {
                    nc[d] = 1;
                    cand[d][0] = f[d] / 2;
                    wt[d][0] = 1.0;
                } else {
                    nc[d] = 2;
                    cand[d][0] = (f[d] - 1) / 2;
                    cand[d][1] = (f[d] + 1) / 2;
                    wt[d][0] = wt[d][1] = 0.5;
                }
            }
            (void)w2;
            for (int a = 0; a < nc[0]; ++a)
                for (int b = 0; b < nc[1]; ++b)
                    for (int c = 0; c < nc[2]; ++c) {
                        int ic[3] = {cand[0][a], cand[1][b], cand[2][c]};
                        bool ok = true;
                        for (int d = 0; d < 3; ++d)
                            if (ic[d] <= 0 || ic[d] >= cg.c[d]) ok = false;
                        if (!ok) continue;
                        int64_t cidx = ((int64_t)(ic[2] - 1) * cg.N[1] + (ic[1] - 1)) * cg.N[0] + (ic[0] - 1);
                        col[cidx] += wt[0][a] * wt[1][b] * wt[2][c] * B.val[e];
                    }
        }
        for (auto &kv : col) {
            out.row.push_back(kv.first);
            out.val.push_back(kv.second);
        }
        out.ptr.push_back((int64_t)out.row.size());
    }
    return out;
}

std::vector<double> dense_precision(const Geometry &g, const double st[27], const SparseCols &B,
                                    const std::vector<double> &Sigma) {
    const int64_t n = g.n;
    std::vector<double> Q((size_t)(n * n), 0.0);
    const int64_t nxy = (int64_t)g.N[0] * g.N[1];
    for (int64_t ell = 0; ell < n; ++ell) {
        int v[3] = {(int)((ell % nxy) % g.N[0]) + 1, (int)((ell % nxy) / g.N[0]) + 1, (int)(ell / nxy) + 1};
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    double w = st[sidx(dx, dy, dz)];
                    if (w == 0.0) continue;
                    int u[3] = {v[0] + dx, v[1] + dy, v[2] + dz};
                    bool ok = true;
                    for (int d = 0; d < 3; ++d)
                        if (u[d] <= 0 || u[d] >= g.c[d]) ok = false;
                    if (!ok) continue;
                    int64_t col = ((int64_t)(u[2] - 1) * g.N[1] + (u[1] - 1)) * g.N[0] + (u[0] - 1);
                    Q[ell * n + col] = w;
                }
    }
    for (int j = 0; j < B.m; ++j) {
        double sinv = 1.0 / Sigma[j];
        for (int64_t a = B.ptr[j]; a < B.ptr[j + 1]; ++a)
            for (int64_t b = B.ptr[j]; b < B.ptr[j + 1]; ++b)
                Q[B.row[a] * n + B.row[b]] += B.val[a] * sinv * B.val[b];
    }
    return Q;
}

// Left-looking Cholesky: L_ij = (Q_ij - sum_{k<j} L_ik L_jk) / L_jj with the
// inner sums in ascending k.
bool dense_cholesky(std::vector<double> &Q, int64_t n) {
    bool ok = true;
    for (int64_t j = 0; j < n && ok; ++j) {
        const double *Lj = &Q[j * n];
        double s = Q[j * n + j];
        for (int64_t k = 0; k < j; ++k) s -= Lj[k] * Lj[k];
        if (!(s > 0.0)) {
            ok = false;
            break;
        }
        const double d = std::sqrt(s);
        Q[j * n + j] = d;
#pragma omp parallel for schedule(static) if (n - j > 256)
        for (int64_t i = j + 1; i < n; ++i) {
            double *Li = &Q[i * n];
            double t = Li[j];
            for (int64_t k = 0; k < j; ++k) t -= Li[k] * Lj[k];
            Li[j] = t / d;
        }
    }
    if (!ok) return false;
    for (int64_t i = 0; i < n; ++i)
        for (int64_t j = i + 1; j < n; ++j) Q[i * n + j] = 0.0;
    return true;
}

// Column c of L^{-1} by forward substitution; stored as row c of the
// transposed inverse.
std::vector<double> inverse_factor_transposed(const std::vector<double> &L, int64_t n) {
    std::vector<double> T((size_t)(n * n), 0.0);
#pragma omp parallel for schedule(dynamic, 8) if (n > 256)
    for (int64_t c = 0; c < n; ++c) {
        double *w = &T[c * n];
        w[c] = 1.0 / L[c * n + c];
        for (int64_t i = c + 1; i < n; ++i) {
            const double *Li = &L[i * n];
            double s = 0.0;
            for (int64_t k = c; k < i; ++k) s -= Li[k] * w[k];
            w[i] = s / Li[i];
        }
    }
    return T;
}

std::vector<double> galerkin_field(const Geometry &fine, const double stencil[27], const double *centre,
                                   const double *full) {
    const Geometry crs = fine.coarse();
    const int64_t n = fine.n, nc = crs.n;
    const int *N = fine.N, *Nc = crs.N;
    const bool act[3] = {fine.dim > 0, fine.dim > 1, fine.dim > 2};
    std::vector<double> out((size_t)27 * nc, 0.0);
    auto wgt = [&](int64_t f, int k) -> double {
        if (full) return full[(size_t)k * n + f];
        return k == 13 && centre ? centre[f] : stencil[k];
    };
#pragma omp parallel for schedule(static) if (nc > 4096)
    for (int64_t pc = 0; pc < nc; ++pc) {
        int c[3] = {(int)(pc % Nc[0]), (int)((pc / Nc[0]) % Nc[1]), (int)(pc / ((int64_t)Nc[0] * Nc[1]))};
        double acc[27] = {0};
        int lo[3], hi[3];
        for (int d = 0; d < 3; ++d) {
            lo[d] = act[d] ? -1 : 0;
            hi[d] = act[d] ? 1 : 0;
        }
        for (int rz = lo[2]; rz <= hi[2]; ++rz)
            for (int ry = lo[1]; ry <= hi[1]; ++ry)
                for (int rx = lo[0]; rx <= hi[0]; ++rx) {
                    const int r[3] = {rx, ry, rz};
                    int fp[3];
                    double wr = 1.0;
                    bool in = true;
                    for (int d = 0; d < 3; ++d) {
                        fp[d] = act[d] ? 2 * c[d] + 1 + r[d] : 0;
                        if (r[d]) wr *= 0.5;
                        in = in && fp[d] >= 0 && fp[d] < N[d];
                    }
                    if (!in) continue;
                    const int64_t f = ((int64_t)fp[2] * N[1] + fp[1]) * N[0] + fp[0];
                    for (int k = 0; k < 27; ++k) {
                        const int o[3] = {k % 3 - 1, (k / 3) % 3 - 1, k / 9 - 1};
                        bool ok = true;
                        int gq[3];
                        for (int d = 0; d < 3; ++d) {
                            if (!act[d] && o[d]) ok = false;
                            gq[d] = fp[d] + o[d];
                            ok = ok && gq[d] >= 0 && gq[d] < N[d];
                        }
                        if (!ok) continue;
                        const double a = wgt(f, k);
                        if (a == 0.0) continue;
                        // coarse parents q of the fine neighbour gq: gq = 2 q + 1 + s, s in {-1, 0, 1}
                        int pq[3][2], np_[3];
                        double pw[3][2];
                        for (int d = 0; d < 3; ++d) {
                            if (!act[d]) {
                                np_[d] = 1;
                                pq[d][0] = 0;
                                pw[d][0] = 1.0;
                            } else if (gq[d] % 2 == 1) {
                                np_[d] = 1;
                                pq[d][0] = (gq[d] - 1) / 2;
                                pw[d][0] = 1.0;
                            } else {
                                np_[d] = 2;
                                pq[d][0] = gq[d] / 2 - 1;
                                pq[d][1] = gq[d] / 2;
                                pw[d][0] = pw[d][1] = 0.5;
                            }
                        }
                        for (int iz = 0; iz < np_[2]; ++iz)
                            for (int iy = 0; iy < np_[1]; ++iy)
                                for (int ix = 0; ix < np_[0]; ++ix) {
                                    const int q[3] = {pq[0][ix], pq[1][iy], pq[2][iz]};
                                    bool qin = true;
                                    for (int d = 0; d < 3; ++d) qin = qin && q[d] >= 0 && q[d] < Nc[d];
                                    if (!qin) continue;
                                    const int kc = (q[2] - c[2] + 1) * 9 + (q[1] - c[1] + 1) * 3 + (q[0] - c[0] + 1);
                                    acc[kc] += wr * a * pw[0][ix] * pw[1][iy] * pw[2][iz];
                                }
                    }
                }
        for (int k = 0; k < 27; ++k) out[(size_t)k * nc + pc] = acc[k];
    }
    return out;
}

std::vector<double> fem_field(const Geometry &g, int model, double p0, double p1) {
    const int dim = g.dim;
    const int64_t n = g.n;
    double h[3] = {1, 1, 1}, hinv2[3] = {0, 0, 0};
    double cell_volume = 1.0;
    for (int d = 0; d < dim; ++d) {
        h[d] = 1. / double(g.c[d]);
        hinv2[d] = 1. / (h[d] * h[d]);
        cell_volume *= h[d];
    }
    // quadrature on [0,1]^d, first direction slowest (quadrature.cc:11-56)
    const double q1[2] = {0.5 * (-1.0 / std::sqrt(3.0) + 1.0), 0.5 * (1.0 / std::sqrt(3.0) + 1.0)};
    const int nq = 1 << dim, nb = 1 << dim;
    std::vector<std::array<double, 3>> qp(nq);
    std::vector<double> qw(nq);
    for (int q = 0; q < nq; ++q) {
        double w = 1.0;
        for (int d = 0; d < dim; ++d) {
            qp[q][d] = q1[(q >> (dim - 1 - d)) & 1];
            w *= 0.5 * 1.0;
        }
        qw[q] = w;
    }
    // basis index alpha in {0,1}^d, first direction slowest
    auto bit = [&](int a, int d) { return (a >> (dim - 1 - d)) & 1; };
    auto phi = [&](int a, const std::array<double, 3> &x) {
        double v = 1.0;
        for (int j = 0; j < dim; ++j) v *= bit(a, j) == 0 ? (1.0 - x[j]) : x[j];
        return v;
    };
    auto dphi = [&](int a, int k, const std::array<double, 3> &x) {
        double v = 1.0;
        for (int j = 0; j < dim; ++j)
            v *= j == k ? (bit(a, j) == 0 ? -1.0 : 1.0) : (bit(a, j) == 0 ? (1.0 - x[j]) : x[j]);
        return v;
    };
    std::vector<double> pp((size_t)nb * nb * nq), gg((size_t)nb * nb * nq);
    for (int a = 0; a < nb; ++a)
        for (int b = 0; b < nb; ++b)
            for (int q = 0; q < nq; ++q) {
                pp[((size_t)a * nb + b) * nq + q] = phi(a, qp[q]) * phi(b, qp[q]);
                double s = 0.0;
                for (int k = 0; k < dim; ++k) s += dphi(a, k, qp[q]) * (hinv2[k] * dphi(b, k, qp[q]));
                gg[((size_t)a * nb + b) * nq + q] = s;
            }
    const double L1 = 0.5 * (p1 + p0), L2 = 0.5 * (p1 - p0);
    auto kappa_sq = [&](const double *x) {
        if (model == 0) return p0;
        double lam = L2;
        for (int d = 0; d < dim; ++d) lam *= std::cos(M_PI * x[d]);
        lam += L1;
        return 1. / (lam * lam);
    };
    std::vector<double> field((size_t)27 * n, 0.0);
    const int nc[3] = {g.c[0], dim > 1 ? g.c[1] : 1, dim > 2 ? g.c[2] : 1};
    for (int ck = 0; ck < nc[2]; ++ck)
        for (int cj = 0; cj < nc[1]; ++cj)
            for (int ci = 0; ci < nc[0]; ++ci) {  // cells in the reference's linear order
                const int cell[3] = {ci, cj, ck};
                for (int a = 0; a < nb; ++a)
                    for (int b = 0; b < nb; ++b) {
                        int va[3] = {1, 1, 1}, vb[3] = {1, 1, 1};
                        bool inside = true;
                        for (int d = 0; d < dim; ++d) {
                            va[d] = cell[d] + bit(a, d);
                            vb[d] = cell[d] + bit(b, d);
                            inside = inside && va[d] > 0 && va[d] < g.c[d] && vb[d] > 0 && vb[d] < g.c[d];
                        }
                        if (!inside) continue;
                        double local = 0.0;
                        for (int q = 0; q < nq; ++q) {
                            double x[3] = {0, 0, 0};
                            for (int d = 0; d < dim; ++d) x[d] = h[d] * (qp[q][d] + double(cell[d]));
                            local += (kappa_sq(x) * pp[((size_t)a * nb + b) * nq + q] + gg[((size_t)a * nb + b) * nq + q]) * qw[q];
                        }
                        const int64_t row = ((int64_t)(va[2] - 1) * g.N[1] + (va[1] - 1)) * g.N[0] + (va[0] - 1);
                        const int k = (vb[2] - va[2] + 1) * 9 + (vb[1] - va[1] + 1) * 3 + (vb[0] - va[0] + 1);
                        field[(size_t)k * n + row] += local * cell_volume;
                    }
            }
    return field;
}

std::vector<double> dense_precision_field(const Geometry &g, const std::vector<double> &field, const SparseCols &B,
                                          const std::vector<double> &Sigma) {
    const int64_t n = g.n;
    std::vector<double> Q((size_t)(n * n), 0.0);
    for (int64_t p = 0; p < n; ++p) {
        const int a = (int)(p % g.N[0]), b = (int)((p / g.N[0]) % g.N[1]), c = (int)(p / ((int64_t)g.N[0] * g.N[1]));
        for (int k = 0; k < 27; ++k) {
            const double w = field[(size_t)k * n + p];
            if (w == 0.0) continue;
            const int qa = a + k % 3 - 1, qb = b + (k / 3) % 3 - 1, qc = c + k / 9 - 1;
            if (qa < 0 || qb < 0 || qc < 0 || qa >= g.N[0] || qb >= g.N[1] || qc >= g.N[2]) continue;
            Q[(size_t)p * n + ((int64_t)qc * g.N[1] + qb) * g.N[0] + qa] = w;
        }
    }
    for (int j = 0; j < B.m; ++j) {
        const double sinv = 1.0 / Sigma[j];
        for (int64_t e = B.ptr[j]; e < B.ptr[j + 1]; ++e)
            for (int64_t f = B.ptr[j]; f < B.ptr[j + 1]; ++f)
                Q[(size_t)B.row[e] * n + B.row[f]] += B.val[e] * sinv * B.val[f];
    }
    return Q;
}

std::vector<double> cholesky_phi_sandwich(const std::vector<double> &T, const Geometry &g, const double E[27]) {
    const int64_t n = g.n;
    // Y = E L^{-T}: row p of Y sums the rows q of L^{-T} (= rows of T) over
    // the stencil neighbours q of p
    std::vector<double> Y((size_t)(n * n), 0.0);
#pragma omp parallel for schedule(static) if (n > 256)
    for (int64_t p = 0; p < n; ++p) {
        const int a = (int)(p % g.N[0]), b = (int)((p / g.N[0]) % g.N[1]), c = (int)(p / ((int64_t)g.N[0] * g.N[1]));
        double *y = &Y[(size_t)p * n];
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    const double w = E[(dz + 1) * 9 + (dy + 1) * 3 + (dx + 1)];
                    const int qa = a + dx, qb = b + dy, qc = c + dz;
                    if (w == 0.0 || qa < 0 || qb < 0 || qc < 0 || qa >= g.N[0] || qb >= g.N[1] || qc >= g.N[2]) continue;
                    const int64_t q = ((int64_t)qc * g.N[1] + qb) * g.N[0] + qa;
                    const double *t = &T[(size_t)q * n];
                    for (int64_t j = q; j < n; ++j) y[j] += w * t[j];  // T row q is zero before column q
                }
    }
    // X = L^{-1} Y on and below the diagonal: X[i][j] = sum_{k <= i} L^{-1}[i][k] Y[k][j]
    std::vector<double> Phi((size_t)(n * n), 0.0);
#pragma omp parallel for schedule(dynamic, 8) if (n > 256)
    for (int64_t i = 0; i < n; ++i) {
        double *x = &Phi[(size_t)i * n];
        for (int64_t k = 0; k <= i; ++k) {
            const double l = T[(size_t)k * n + i];  // L^{-1}[i][k]
            if (l == 0.0) continue;
            const double *y = &Y[(size_t)k * n];
            for (int64_t j = 0; j <= i; ++j) x[j] += l * y[j];
        }
        x[i] *= 0.5;
    }
    return Phi;
}

std::vector<double> inverse_factor_times(const std::vector<double> &T, int64_t n, const SparseCols &B) {
    std::vector<double> U((size_t)n * B.m, 0.0);
    for (int k = 0; k < B.m; ++k) {
        double *u = &U[(size_t)k * n];
        for (int64_t e = B.ptr[k]; e < B.ptr[k + 1]; ++e) {
            const int64_t l = B.row[e];
            const double v = B.val[e];
            const double *t = &T[(size_t)l * n];
            for (int64_t i = l; i < n; ++i) u[i] += v * t[i];  // L^{-1}[i][l] = T[l][i], zero for i < l
        }
    }
    return U;
}

std::vector<double> small_inverse(const std::vector<double> &S, int m) {
    std::vector<double> LU = S, inv((size_t)m * m, 0.0);
    std::vector<int> piv(m);
    for (int i = 0; i < m; ++i) piv[i] = i;
    for (int k = 0; k < m; ++k) {
        int p = k;
        for (int i = k + 1; i < m; ++i)
            if (std::fabs(LU[i * m + k]) > std::fabs(LU[p * m + k])) p = i;
        if (p != k) {
            for (int j = 0; j < m; ++j) std::swap(LU[k * m + j], LU[p * m + j]);
            std::swap(piv[k], piv[p]);
        }
        for (int i = k + 1; i < m; ++i) {
            LU[i * m + k] /= LU[k * m + k];
            for (int j = k + 1; j < m; ++j) LU[i * m + j] -= LU[i * m + k] * LU[k * m + j];
        }
    }
    for (int c = 0; c < m; ++c) {
        std::vector<double> y(m);
        for (int i = 0; i < m; ++i) {
            double s = (piv[i] == c) ? 1.0 : 0.0;
            for (int j = 0; j < i; ++j) s -= LU[i * m + j] * y[j];
            y[i] = s;
        }
        for (int i = m - 1; i >= 0; --i) {
            double s = y[i];
            for (int j = i + 1; j < m; ++j) s -= LU[i * m + j] * inv[j * m + c];
            inv[i * m + c] = s / LU[i * m + i];
        }
    }
    return inv;
}

// ----------------------------------------------------- low-rank Cholesky
bool lowrank_cholesky_factors(const Geometry &g, const double st[27], const SparseCols &B,
                              const std::vector<double> &Sigma, LowRankCholeskyFactors &F) {
    const int dim = g.dim;
    const int64_t n = g.n;
    const int nb = g.N[dim - 1];
    const int64_t p = n / nb;
    F.nb = nb;
    F.p = p;
    F.m = B.m;
    // in-block coordinates: (a, b) in 3D, (a) in 2D, none in 1D; the block
    // offset runs along direction dim - 1
    const int n0 = dim >= 2 ? g.N[0] : 1, n1 = dim == 3 ? g.N[1] : 1;
    auto coupling = [&](int64_t i, int64_t j, int off) {
        const int ai = (int)(i % n0), bi = (int)(i / n0), aj = (int)(j % n0), bj = (int)(j / n0);
        const int da = aj - ai, db = bj - bi;
        if (da < -1 || da > 1 || db < -1 || db > 1) return 0.0;
        if (dim == 3) return st[sidx(da, db, off)];
        if (dim == 2) return st[sidx(da, off, 0)];
        return st[sidx(off, 0, 0)];
    };
    std::vector<double> Ain((size_t)(p * p), 0.0), Aoff((size_t)(p * p), 0.0);
    for (int64_t i = 0; i < p; ++i)
        for (int64_t j = 0; j < p; ++j) {
            Ain[i * p + j] = coupling(i, j, 0);
            Aoff[i * p + j] = coupling(i, j, -1);  // row in block k, column in block k - 1
        }
    (void)n1;
    F.D.assign((size_t)(nb * p * p), 0.0);
    F.O.assign((size_t)(nb * p * p), 0.0);
    std::vector<double> S = Ain;
    for (int k = 0; k < nb; ++k) {
        std::vector<double> Lk = S;
        if (!dense_cholesky(Lk, p)) return false;
        const std::vector<double> T = inverse_factor_transposed(Lk, p);  // (L_kk^{-1})^T
        double *Dk = &F.D[(size_t)k * p * p];
#pragma omp parallel for schedule(static) if (p > 256)
        for (int64_t i = 0; i < p; ++i)
            for (int64_t j = 0; j <= i; ++j) Dk[i * p + j] = T[j * p + i];
        if (k + 1 == nb) break;
        double *Ok = &F.O[(size_t)(k + 1) * p * p];
        // L_{k+1,k} = A_{k+1,k} L_kk^{-T}: row i gathers the (few) coupled rows of T
#pragma omp parallel for schedule(static) if (p > 256)
        for (int64_t i = 0; i < p; ++i)
            for (int64_t l = 0; l < p; ++l) {
                const double a = Aoff[i * p + l];
                if (a == 0.0) continue;
                const double *Tl = &T[l * p];
                for (int64_t j = 0; j < p; ++j) Ok[i * p + j] += a * Tl[j];
            }
        // S_{k+1} = A_{k+1,k+1} - L_{k+1,k} L_{k+1,k}^T (lower half, mirrored)
#pragma omp parallel for schedule(dynamic, 16) if (p > 256)
        for (int64_t i = 0; i < p; ++i) {
            const double *Oi = &Ok[i * p];
            for (int64_t j = 0; j <= i; ++j) {
                const double *Oj = &Ok[j * p];
                double d = 0.0;
                for (int64_t l = 0; l < p; ++l) d += Oi[l] * Oj[l];
                S[i * p + j] = Ain[i * p + j] - d;
            }
        }
        for (int64_t i = 0; i < p; ++i)
            for (int64_t j = i + 1; j < p; ++j) S[i * p + j] = S[j * p + i];
    }
    const int m = B.m;
    if (m == 0) return true;
    // V = L^{-1} B block by block: Y_k = D_k (B_k - O_k Y_{k-1}), n x m row-major
    std::vector<double> V((size_t)(n * m), 0.0), Bk((size_t)(p * m));
    for (int j = 0; j < m; ++j)
        for (int64_t e = B.ptr[j]; e < B.ptr[j + 1]; ++e) V[B.row[e] * m + j] = B.val[e];  // B first, in place
    for (int k = 0; k < nb; ++k) {
        double *Yk = &V[(size_t)k * p * m];
        std::copy(Yk, Yk + p * m, Bk.begin());
        if (k > 0) {
            const double *Ok = &F.O[(size_t)k * p * p];
            const double *Yp = &V[(size_t)(k - 1) * p * m];
#pragma omp parallel for schedule(static) if (p > 256)
            for (int64_t i = 0; i < p; ++i)
                for (int64_t l = 0; l < p; ++l) {
                    const double o = Ok[i * p + l];
                    if (o == 0.0) continue;
                    for (int c = 0; c < m; ++c) Bk[i * m + c] -= o * Yp[l * m + c];
                }
        }
        const double *Dk = &F.D[(size_t)k * p * p];
#pragma omp parallel for schedule(static) if (p > 256)
        for (int64_t i = 0; i < p; ++i) {
            for (int c = 0; c < m; ++c) {
                double d = 0.0;
                for (int64_t l = 0; l <= i; ++l) d += Dk[i * p + l] * Bk[l * m + c];
                Yk[i * m + c] = d;
            }
        }
    }
    // Householder QR of V; Q explicit (n x m), R (m x m) with a positive diagonal
    std::vector<double> A = V, tau(m, 0.0), R((size_t)m * m, 0.0);
    std::vector<std::vector<double>> refl(m);
    for (int k = 0; k < m; ++k) {
        double nrm = 0.0;
        for (int64_t i = k; i < n; ++i) nrm += A[i * m + k] * A[i * m + k];
        nrm = std::sqrt(nrm);
        const double a0 = A[(int64_t)k * m + k];
        const double alpha = a0 >= 0.0 ? -nrm : nrm;
        std::vector<double> v((size_t)n, 0.0);
        for (int64_t i = k; i < n; ++i) v[i] = A[i * m + k];
        v[k] = a0 - alpha;
        double vv = 0.0;
        for (int64_t i = k; i < n; ++i) vv += v[i] * v[i];
        if (vv > 0.0) {
            for (int c = k; c < m; ++c) {
                double d = 0.0;
                for (int64_t i = k; i < n; ++i) d += v[i] * A[i * m + c];
                const double sc = 2.0 * d / vv;
                for (int64_t i = k; i < n; ++i) A[i * m + c] -= sc * v[i];
            }
            tau[k] = 2.0 / vv;
        }
        refl[k] = std::move(v);
    }
    for (int i = 0; i < m; ++i)
        for (int c = i; c < m; ++c) R[(size_t)i * m + c] = A[(int64_t)i * m + c];
    F.Q.assign((size_t)(n * m), 0.0);
    for (int c = 0; c < m; ++c) F.Q[(size_t)c * m + c] = 1.0;
    for (int k = m - 1; k >= 0; --k) {
        const std::vector<double> &v = refl[k];
        for (int c = 0; c < m; ++c) {
            double d = 0.0;
            for (int64_t i = k; i < n; ++i) d += v[i] * F.Q[i * m + c];
            const double sc = tau[k] * d;
            for (int64_t i = k; i < n; ++i) F.Q[i * m + c] -= sc * v[i];
        }
    }
    for (int c = 0; c < m; ++c)
        if (R[(size_t)c * m + c] < 0.0) {
            for (int cc = 0; cc < m; ++cc) R[(size_t)c * m + cc] = -R[(size_t)c * m + cc];
            for (int64_t i = 0; i < n; ++i) F.Q[i * m + c] = -F.Q[i * m + c];
        }
    // Id - Lambda = Id - R (Sigma + V^T V)^{-1} R^T and its lower factor W
    std::vector<double> Sm((size_t)m * m, 0.0);
    for (int a = 0; a < m; ++a)
        for (int c = 0; c < m; ++c) {
            double d = 0.0;
            for (int64_t i = 0; i < n; ++i) d += V[i * m + a] * V[i * m + c];
            Sm[(size_t)a * m + c] = d + (a == c ? Sigma[a] : 0.0);
        }
    const std::vector<double> Si = small_inverse(Sm, m);
    std::vector<double> RSi((size_t)m * m, 0.0), W((size_t)m * m, 0.0);
    for (int a = 0; a < m; ++a)
        for (int c = 0; c < m; ++c) {
            double d = 0.0;
            for (int k = 0; k < m; ++k) d += R[(size_t)a * m + k] * Si[(size_t)k * m + c];
            RSi[(size_t)a * m + c] = d;
        }
    for (int a = 0; a < m; ++a)
        for (int c = 0; c < m; ++c) {
            double d = 0.0;
            for (int k = 0; k < m; ++k) d += RSi[(size_t)a * m + k] * R[(size_t)c * m + k];
            W[(size_t)a * m + c] = (a == c ? 1.0 : 0.0) - d;
        }
    if (!dense_cholesky(W, m)) return false;
    F.QW.assign((size_t)(n * m), 0.0);
    F.QWT.assign((size_t)(n * m), 0.0);
#pragma omp parallel for schedule(static) if (n > 4096)
    for (int64_t i = 0; i < n; ++i)
        for (int c = 0; c < m; ++c) {
            double u = 0.0, l = 0.0;
            for (int k = 0; k < m; ++k) {
                u += F.Q[i * m + k] * (W[(size_t)c * m + k] - (k == c ? 1.0 : 0.0));  // (W^T - Id)[k][c]
                l += F.Q[i * m + k] * (W[(size_t)k * m + c] - (k == c ? 1.0 : 0.0));  // (W - Id)[k][c]
            }
            F.QW[i * m + c] = u;
            F.QWT[i * m + c] = l;
        }
    return true;
}

}  // namespace mgmc
