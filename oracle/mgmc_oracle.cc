// mgmc_oracle.cc -- CPU restatement of the MultigridMC sampling path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle against which the
// GB300 library is checked.  Only the test-suite, __graft_entry__.smoke()
// and the cpu_baseline leg of bench.py may load it; the product never links
// or calls it.
//
// Every function restates the behaviour of the reference (eikehmueller/
// MultigridMC) in plain, Eigen-free C++; the reference file:line each one
// follows is given in its comment.  Arithmetic is written in the operation
// order of the reference wherever that order is visible in its source, and
// the library is compiled with -ffp-contract=off so that no FMA contraction
// changes rounding.
//
// Parity status: the reference's sampling path cannot be compiled here
// (Eigen >= 5.0, libconfig++, LAPACKE, googletest absent, no network).  The
// oracle is pinned by the reference's own known-answer and property tests
// (lattice index maps, quadrature, CLCG serial/leapfrog agreement,
// Statistics on an AR(1) process, intergrid adjointness, smoother fixed
// point, sampler mean/covariance against the exact covariance), restated in
// tests/test_oracle_*.py, and its random number generator is compared draw
// by draw (integers, uniforms, normals; serial and leapfrog) with the
// reference's own CLCGenerator compiled from its sources (oracle/
// build_ref.py), the one part of the path that builds without Eigen.
// Pathwise chain values of the reference itself are unpinned: no reference
// binary of the sampler can be run to produce them.
//
// Deviations, both deliberate and documented:
//  * the coarse-level Cholesky sampler factorises in natural order, which is
//    the reference's DenseCholeskySampler (cholesky_sampler.cc:25-37,
//    cholesky_wrapper.cc:128-155); the reference's sparse samplers use an
//    AMD / CHOLMOD ordering whose pathwise sample differs (the distribution
//    does not).
//  * an optional multicolour ordering of the SOR sweep (not in the
//    reference) so that the GPU's multicolour kernels can be checked
//    pathwise; ordering 0 is the reference's lexicographic order.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdio>
#include <deque>
#include <map>
#include <memory>
#include <stdexcept>
#include <vector>
#include <algorithm>
#include <array>
#include <tuple>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

// ---------------------------------------------------------------------------
// Lattice: src/lattice/lattice{1,2,3}d.hh.  n[d] cells per direction for the
// active directions d < dim; vertices are the interior points, lexicographic
// with x fastest (lattice3d.hh:118-141).
// ---------------------------------------------------------------------------
struct Lattice {
    int dim;
    int n[3];
    Lattice(int dim_, int nx, int ny, int nz) : dim(dim_) {
        n[0] = nx;
        n[1] = dim > 1 ? ny : 2;
        n[2] = dim > 2 ? nz : 2;
    }
    int N(int d) const { return n[d] - 1; }  // interior extent
    int64_t nvertex() const { return (int64_t)N(0) * N(1) * N(2); }
    int64_t ncell() const {
        int64_t c = 1;
        for (int d = 0; d < dim; ++d) c *= n[d];
        return c;
    }
    // lattice3d.hh:128-135 (1-based Euclidean vertex index)
    void vertex_euclid(int64_t ell, int idx[3]) const {
        int64_t nxy = (int64_t)N(0) * N(1);
        idx[0] = (int)((ell % nxy) % N(0)) + 1;
        idx[1] = (int)((ell % nxy) / N(0)) + 1;
        idx[2] = (int)(ell / nxy) + 1;
    }
    int64_t vertex_linear(const int idx[3]) const {
        return ((int64_t)(idx[2] - 1) * N(1) + (idx[1] - 1)) * N(0) + (idx[0] - 1);
    }
    bool is_interior(const int idx[3]) const {
        for (int d = 0; d < 3; ++d)
            if (idx[d] <= 0 || idx[d] >= n[d]) return false;
        return true;
    }
    // lattice3d.hh:77-86 cell index maps
    void cell_euclid(int64_t ell, int idx[3]) const {
        int nx = n[0], ny = dim > 1 ? n[1] : 1;
        idx[0] = (int)((ell % ((int64_t)nx * ny)) % nx);
        idx[1] = (int)((ell % ((int64_t)nx * ny)) / nx);
        idx[2] = (int)(ell / ((int64_t)nx * ny));
    }
    // lattice.hh:36-44 (volume /= s[d])
    double cell_volume() const {
        double v = 1.0;
        for (int d = 0; d < dim; ++d) v /= n[d];
        return v;
    }
    // lattice3d.hh:236-246
    void vertex_coordinates(int64_t ell, double x[3]) const {
        int idx[3];
        vertex_euclid(ell, idx);
        for (int d = 0; d < dim; ++d) x[d] = idx[d] * (1. / double(n[d]));
    }
    // lattice3d.hh:224-231 (fine_vertex_idx of a coarse vertex)
    int64_t fine_vertex_idx(int64_t ell) const {
        int idx[3];
        vertex_euclid(ell, idx);
        int64_t fN0 = 2 * n[0] - 1, fN1 = 2 * n[1] - 1;
        if (dim == 1) return 2 * (int64_t)idx[0] - 1;
        if (dim == 2) return (2 * (int64_t)idx[1] - 1) * fN0 + 2 * idx[0] - 1;
        return (2 * (int64_t)idx[2] - 1) * fN0 * fN1 + (2 * (int64_t)idx[1] - 1) * fN0 + 2 * idx[0] - 1;
    }
    // lattice3d.hh:248-263: even extents and >1 coarse cell required
    bool coarsenable() const {
        for (int d = 0; d < dim; ++d)
            if (n[d] % 2 != 0 || n[d] / 2 <= 1) return false;
        return true;
    }
    Lattice coarse() const { return Lattice(dim, n[0] / 2, n[1] / 2, n[2] / 2); }
};

// Colour of a vertex for the optional multicolour ordering (0-based
// interior coordinates, inactive directions contribute 0).
static int vertex_colour(const Lattice &lat, int64_t ell, int ncolour) {
    int idx[3];
    lat.vertex_euclid(ell, idx);
    int a = idx[0] - 1, b = idx[1] - 1, c = idx[2] - 1;
    if (ncolour == 2) return (a + b + c) & 1;
    return (a & 1) | ((b & 1) << 1) | ((c & 1) << 2);
}

// ---------------------------------------------------------------------------
// Sparse matrices.  Csr holds a square symmetric operator with columns sorted
// ascending in every row; for a symmetric matrix this is also Eigen's
// column-major storage that the reference iterates (sor_smoother.cc:59-76).
// Csc holds the n x m measurement matrix B column by column, rows ascending.
// ---------------------------------------------------------------------------
struct Csr {
    int64_t n = 0;
    std::vector<int64_t> ptr;
    std::vector<int64_t> col;
    std::vector<double> val;
    std::vector<double> diag;
    void finish_diag() {
        diag.assign(n, 0.0);
        for (int64_t i = 0; i < n; ++i)
            for (int64_t k = ptr[i]; k < ptr[i + 1]; ++k)
                if (col[k] == i) diag[i] = val[k];
    }
};

struct Csc {
    int64_t nrow = 0;
    int m = 0;
    std::vector<int64_t> ptr;  // m+1
    std::vector<int64_t> row;
    std::vector<double> val;
};

// ---------------------------------------------------------------------------
// LinearOperator: A = A_0 + B Sigma^{-1} B^T (linear_operator.hh:19-26).
// ---------------------------------------------------------------------------
struct LinOp {
    Lattice lat;
    Csr A;
    Csc B;           // n x m
    std::vector<double> Sigma;  // m
    explicit LinOp(const Lattice &l) : lat(l) {}
    int m() const { return B.m; }
    int64_t n() const { return A.n; }
    // linear_operator.hh:78-88: y = A_0 x (+ B (Sigma^{-1} B^T x))
    void apply(const double *x, double *y) const {
        // Eigen's column-major sparse * dense adds val * x[col] into
        // y[row] for col ascending; for the symmetric A that is the row sum
        // over ascending columns, computed here row by row
#pragma omp parallel for schedule(static) if (A.n > 100000)
        for (int64_t i = 0; i < A.n; ++i) {
            double acc = 0.0;
            for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k) acc += A.val[k] * x[A.col[k]];
            y[i] = acc;
        }
        if (m() > 0) {
            std::vector<double> s(m(), 0.0);
            for (int j = 0; j < m(); ++j) {
                double sinv = 1.0 / Sigma[j];
                double acc = 0.0;
                for (int64_t k = B.ptr[j]; k < B.ptr[j + 1]; ++k) acc += (sinv * B.val[k]) * x[B.row[k]];
                s[j] = acc;
            }
            for (int j = 0; j < m(); ++j)
                for (int64_t k = B.ptr[j]; k < B.ptr[j + 1]; ++k) y[B.row[k]] += B.val[k] * s[j];
        }
    }
    // linear_operator.cc:26-34: dense precision A_0 + B Sigma^{-1} B^T
    std::vector<double> precision_dense() const {
        int64_t n_ = n();
        std::vector<double> Q(n_ * n_, 0.0);
        for (int64_t i = 0; i < n_; ++i)
            for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k) Q[i * n_ + A.col[k]] = A.val[k];
        for (int j = 0; j < m(); ++j) {
            double sinv = 1.0 / Sigma[j];
            for (int64_t a = B.ptr[j]; a < B.ptr[j + 1]; ++a)
                for (int64_t b = B.ptr[j]; b < B.ptr[j + 1]; ++b)
                    Q[B.row[a] * n_ + B.row[b]] += B.val[a] * sinv * B.val[b];
        }
        return Q;
    }
};

// Operator from a constant 3^dim stencil with Dirichlet boundaries:
// neighbours outside the interior are omitted, as in
// shiftedlaplace_fd_operator.cc:36-55.  st[(dz+1)*9+(dy+1)*3+(dx+1)].
static std::shared_ptr<LinOp> stencil_operator(const Lattice &lat, const double *st) {
    auto op = std::make_shared<LinOp>(lat);
    int64_t n = lat.nvertex();
    Csr &A = op->A;
    A.n = n;
    A.ptr.assign(n + 1, 0);
    // offsets in ascending linear-index order ((dz, dy, dx) lexicographic)
    std::vector<int> offs;
    for (int k = 0; k < 27; ++k)
        if (st[k] != 0.0) offs.push_back(k);
    A.col.reserve(n * offs.size());
    A.val.reserve(n * offs.size());
    for (int64_t ell = 0; ell < n; ++ell) {
        int idx[3];
        lat.vertex_euclid(ell, idx);
        for (int k : offs) {
            int j[3] = {idx[0] + k % 3 - 1, idx[1] + (k / 3) % 3 - 1, idx[2] + k / 9 - 1};
            if (!lat.is_interior(j)) continue;
            A.col.push_back(lat.vertex_linear(j));
            A.val.push_back(st[k]);
        }
        A.ptr[ell + 1] = (int64_t)A.col.size();
    }
    A.finish_diag();
    op->B.nrow = n;
    op->B.m = 0;
    op->B.ptr.assign(1, 0);
    return op;
}

// shiftedlaplace_fd_operator.cc:9-57: 2d+1 point stencil scaled by the cell
// volume; diag = h^d kappa^2 + sum_d 2 h^d h_d^{-2}, off = -h^d h_d^{-2}.
static void fd_stencil(const Lattice &lat, double kappa_sq, double st[27]) {
    for (int k = 0; k < 27; ++k) st[k] = 0.0;
    double hinv2[3] = {0, 0, 0};
    double cell_volume = 1.0;
    for (int d = 0; d < lat.dim; ++d) {
        double h = 1. / double(lat.n[d]);
        hinv2[d] = 1. / (h * h);
        cell_volume *= h;
    }
    double diagonal = cell_volume * kappa_sq;
    for (int d = 0; d < lat.dim; ++d) {
        double off = -cell_volume * hinv2[d];
        int o[3] = {0, 0, 0};
        o[d] = -1;
        st[(o[2] + 1) * 9 + (o[1] + 1) * 3 + (o[0] + 1)] = off;
        o[d] = +1;
        st[(o[2] + 1) * 9 + (o[1] + 1) * 3 + (o[0] + 1)] = off;
        diagonal += 2. * cell_volume * hinv2[d];
    }
    st[13] = diagonal;
}

// ---------------------------------------------------------------------------
// Measurements: measured_operator.cc:9-171, quadrature.cc:11-56,
// common.hh:29-53.
// ---------------------------------------------------------------------------
static double V_sphere(double radius, int dim) {  // measured_operator.cc:50-66
    if (dim == 0) return 1.0;
    if (dim == 1) return 2. * radius;
    return 2. * M_PI / double(dim) * radius * radius * V_sphere(radius, dim - 2);
}

// cartesian_product(v, n): first factor varies slowest (common.hh:29-53)
template <class T>
static std::vector<std::vector<T>> cartesian_product(const std::vector<T> &v, int n) {
    std::vector<std::vector<T>> prod;
    if (n == 1) {
        for (auto &e : v) prod.push_back({e});
    } else {
        auto prev = cartesian_product(v, n - 1);
        for (auto &s : prev)
            for (auto &e : v) {
                auto sj = s;
                sj.push_back(e);
                prod.push_back(sj);
            }
    }
    return prod;
}

struct Quadrature {  // quadrature.cc:11-56
    std::vector<double> weights;
    std::vector<std::vector<double>> points;
    Quadrature(int dim, int order) {
        std::vector<double> w1, p1;
        if (order == 0) {
            w1 = {2.0};
            p1 = {0.0};
        } else if (order == 1) {
            w1 = {1.0, 1.0};
            p1 = {-1.0 / sqrt(3.0), +1.0 / sqrt(3.0)};
        } else {
            w1 = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
            p1 = {-sqrt(3.0 / 5.0), 0.0, +sqrt(3.0 / 5.0)};
        }
        for (auto &wp : cartesian_product(w1, dim)) {
            double w = 1.0;
            for (double s : wp) w *= 0.5 * s;
            weights.push_back(w);
        }
        for (auto &pp : cartesian_product(p1, dim)) {
            std::vector<double> p(dim);
            for (int j = 0; j < dim; ++j) p[j] = 0.5 * (pp[j] + 1.0);
            points.push_back(p);
        }
    }
};

// ShiftedLaplaceFEMOperator (shiftedlaplace_fem_operator.cc:9-152): Q1
// elements with GaussLegendreQuadrature(dim, 1); every pair (alpha, beta) of
// basis functions of every cell whose corners are interior vertices adds
// sum_q (kappa^2(x_q) phi_a phi_b + grad phi_a . h^{-2} grad phi_b) w_q times
// the cell volume (cells in linear order, alpha and beta in
// cartesian-product order).  model 0: kappa^2 = p0; model 1: periodic
// correlation length, Lambda_min = p0, Lambda_max = p1
// (correlationlength_model.hh:83-112).
static std::shared_ptr<LinOp> fem_operator(const Lattice &lat, int model, double p0, double p1) {
    const int dim = lat.dim;
    double h[3] = {1, 1, 1}, hinv2[3] = {0, 0, 0}, cell_volume = 1.0;
    for (int d = 0; d < dim; ++d) {
        h[d] = 1. / double(lat.n[d]);
        hinv2[d] = 1. / (h[d] * h[d]);
        cell_volume *= h[d];
    }
    Quadrature quad(dim, 1);
    auto basis = cartesian_product(std::vector<int>{0, 1}, dim);
    auto phi = [&](const std::vector<int> &a, const std::vector<double> &x) {
        double v = 1.0;
        for (int j = 0; j < dim; ++j) v *= a[j] == 0 ? (1.0 - x[j]) : x[j];
        return v;
    };
    auto dphi = [&](const std::vector<int> &a, int k, const std::vector<double> &x) {
        double v = 1.0;
        for (int j = 0; j < dim; ++j) v *= j == k ? (a[j] == 0 ? -1.0 : 1.0) : (a[j] == 0 ? (1.0 - x[j]) : x[j]);
        return v;
    };
    std::vector<double> pp, gg;
    for (auto &a : basis)
        for (auto &b : basis)
            for (auto &x : quad.points) {
                pp.push_back(phi(a, x) * phi(b, x));
                double sg = 0.0;
                for (int k = 0; k < dim; ++k) sg += dphi(a, k, x) * (hinv2[k] * dphi(b, k, x));
                gg.push_back(sg);
            }
    const double L1 = 0.5 * (p1 + p0), L2 = 0.5 * (p1 - p0);
    auto kappa_sq = [&](const double *x) {
        if (model == 0) return p0;
        double lam = L2;
        for (int d = 0; d < dim; ++d) lam *= cos(M_PI * x[d]);
        lam += L1;
        return 1. / (lam * lam);
    };
    const int64_t n = lat.nvertex();
    std::vector<std::map<int64_t, double>> rows(n);
    int64_t ncell = 1;
    for (int d = 0; d < dim; ++d) ncell *= lat.n[d];
    for (int64_t cidx = 0; cidx < ncell; ++cidx) {
        int cell[3] = {0, 0, 0};
        int64_t t = cidx;
        for (int d = 0; d < dim; ++d) {
            cell[d] = (int)(t % lat.n[d]);
            t /= lat.n[d];
        }
        size_t count = 0;
        for (auto &a : basis)
            for (auto &b : basis) {
                int va[3] = {1, 1, 1}, vb[3] = {1, 1, 1};
                bool inside = true;
                for (int d = 0; d < dim; ++d) {
                    va[d] = cell[d] + a[d];
                    vb[d] = cell[d] + b[d];
                    inside = inside && va[d] > 0 && va[d] < lat.n[d] && vb[d] > 0 && vb[d] < lat.n[d];
                }
                if (!inside) {
                    count += quad.points.size();
                    continue;
                }
                double local = 0.0;
                for (size_t j = 0; j < quad.points.size(); ++j) {
                    double x[3] = {0, 0, 0};
                    for (int d = 0; d < dim; ++d) x[d] = h[d] * (quad.points[j][d] + double(cell[d]));
                    local += (kappa_sq(x) * pp[count] + gg[count]) * quad.weights[j];
                    count++;
                }
                rows[lat.vertex_linear(va)][lat.vertex_linear(vb)] += local * cell_volume;
            }
    }
    auto op = std::make_shared<LinOp>(lat);
    Csr &A = op->A;
    A.n = n;
    A.ptr.assign(n + 1, 0);
    for (int64_t i = 0; i < n; ++i) {
        for (auto &e : rows[i]) {
            A.col.push_back(e.first);
            A.val.push_back(e.second);
        }
        A.ptr[i + 1] = (int64_t)A.col.size();
    }
    A.finish_diag();
    op->B.nrow = n;
    op->B.m = 0;
    op->B.ptr.assign(1, 0);
    return op;
}

static double norm_diff(const double *a, const double *b, int dim) {
    double s = 0.0;
    for (int d = 0; d < dim; ++d) s += (a[d] - b[d]) * (a[d] - b[d]);
    return sqrt(s);
}

// measured_operator.cc:69-171; entries accumulate in cell order, entries
// whose quadrature contribution is zero are kept (Eigen's coeffRef inserts).
static std::map<int64_t, double> measurement_vector(const Lattice &lat, const double *x0, double radius) {
    std::map<int64_t, double> r;
    int dim = lat.dim;
    if (radius < 1.E-12) {
        double d_min = double(dim);
        int64_t ell_min = 0;
        for (int64_t ell = 0; ell < lat.nvertex(); ++ell) {
            double x[3];
            lat.vertex_coordinates(ell, x);
            double dist = norm_diff(x, x0, dim);
            if (dist < d_min) {
                d_min = dist;
                ell_min = ell;
            }
        }
        r[ell_min] = 1.0;
        return r;
    }
    double h[3] = {0, 0, 0};
    double cell_volume = lat.cell_volume();
    double normalisation = 1. / V_sphere(radius, dim);
    for (int d = 0; d < dim; ++d) h[d] = 1. / double(lat.n[d]);
    Quadrature quad(dim, 1);
    auto basis_idx = cartesian_product(std::vector<int>{0, 1}, dim);
    // cells outside the bounding box of the ball fail the overlap test
    // below; visiting only the box (in ascending cell order) changes nothing
    int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int d = 0; d < dim; ++d) {
        lo[d] = std::max(0, (int)std::floor((x0[d] - radius) / h[d]) - 1);
        hi[d] = std::min(lat.n[d] - 1, (int)std::floor((x0[d] + radius) / h[d]) + 1);
    }
    for (int64_t cell_idx = 0; cell_idx < lat.ncell(); ++cell_idx) {
        int cc[3];
        lat.cell_euclid(cell_idx, cc);
        bool inbox = true;
        for (int d = 0; d < dim; ++d) inbox = inbox && cc[d] >= lo[d] && cc[d] <= hi[d];
        if (!inbox) {
            // jump to the next row of the box
            if (cc[0] < lo[0]) cell_idx += lo[0] - cc[0] - 1;
            else if (cc[0] > hi[0]) cell_idx += lat.n[0] - cc[0] - 1;
            continue;
        }
        bool overlap = false;
        double xmin[3] = {2.0, 2.0, 2.0}, xmax[3] = {-1.0, -1.0, -1.0};
        for (auto &om : basis_idx) {
            double xc[3];
            for (int d = 0; d < dim; ++d) {
                xc[d] = h[d] * double(cc[d] + om[d]);
                xmin[d] = std::min(xmin[d], xc[d]);
                xmax[d] = std::max(xmax[d], xc[d]);
            }
            overlap = overlap || (norm_diff(xc, x0, dim) < radius);
        }
        bool centre_in_cell = true;
        for (int d = 0; d < dim; ++d)
            centre_in_cell = centre_in_cell && (xmin[d] <= x0[d]) && (x0[d] <= xmax[d]);
        overlap = overlap || centre_in_cell;
        if (!overlap) continue;
        for (auto &alpha : basis_idx) {
            int v[3] = {1, 1, 1};
            for (int d = 0; d < dim; ++d) v[d] = cc[d] + alpha[d];
            if (!lat.is_interior(v)) continue;
            int64_t ell = lat.vertex_linear(v);
            double local_entry = 0.0;
            for (size_t j = 0; j < quad.points.size(); ++j) {
                const auto &xhat = quad.points[j];
                double x[3];
                for (int d = 0; d < dim; ++d) x[d] = h[d] * (xhat[d] + double(cc[d]));
                double xi = norm_diff(x, x0, dim) / radius;
                if (xi < 1.0) {
                    double phihat = 1.0;  // f_meas == 1 (measured_operator.hh:62)
                    for (int d = 0; d < dim; ++d) phihat *= (alpha[d] == 0) ? (1.0 - xhat[d]) : xhat[d];
                    local_entry += phihat * quad.weights[j] * cell_volume * normalisation;
                }
            }
            r[ell] += local_entry;
        }
    }
    return r;
}

// ---------------------------------------------------------------------------
// Intergrid operator: intergrid_operator.{hh,cc}, intergrid_operator_linear.cc
// ---------------------------------------------------------------------------
struct Intergrid {
    Lattice fine, crs;
    int S;
    std::vector<double> matrix;
    std::vector<int64_t> colidx;
    explicit Intergrid(const Lattice &f) : fine(f), crs(f.coarse()) {
        int dim = f.dim;
        S = 1;
        for (int d = 0; d < dim; ++d) S *= 3;
        const double st1[3] = {0.5, 1.0, 0.5};
        const int sh1[3] = {-1, 0, +1};
        matrix.resize(S);
        std::vector<std::array<int, 3>> shift(S);
        for (int j = 0; j < S; ++j) {  // intergrid_operator_linear.cc:16-29
            matrix[j] = 1.0;
            std::array<int, 3> s = {0, 0, 0};
            int mu = j;
            for (int d = 0; d < dim; ++d) {
                matrix[j] *= st1[mu % 3];
                s[d] = sh1[mu % 3];
                mu /= 3;
            }
            shift[j] = s;
        }
        int64_t nc = crs.nvertex();
        colidx.resize(nc * S);
        for (int64_t ic = 0; ic < nc; ++ic) {  // intergrid_operator.cc:8-20
            int c[3];
            crs.vertex_euclid(ic, c);
            for (int j = 0; j < S; ++j) {
                int v[3] = {1, 1, 1};
                for (int d = 0; d < dim; ++d) v[d] = 2 * c[d] + shift[j][d];
                colidx[ic * S + j] = fine.vertex_linear(v);
            }
        }
    }
    void restrict_(const double *x, double *xc) const {  // intergrid_operator.hh:74-88
#pragma omp parallel for schedule(static) if (crs.nvertex() > 100000)
        for (int64_t ic = 0; ic < crs.nvertex(); ++ic) {
            double result = 0;
            for (int k = 0; k < S; ++k) result += matrix[k] * x[colidx[ic * S + k]];
            xc[ic] = result;
        }
    }
    void prolongate_add(double alpha, const double *xc, double *x) const {  // :106-120
        for (int64_t ic = 0; ic < crs.nvertex(); ++ic) {
            double xce = xc[ic];
            for (int k = 0; k < S; ++k) x[colidx[ic * S + k]] += alpha * matrix[k] * xce;
        }
    }
};

// linear_operator.cc:10-23: A_c = R A R^T, B_c = R B, Sigma copied.
// Sparse triple product row by row: (R A)[ic, g] accumulates over the
// restriction entries k (ascending) and the CSR entries of each fine row,
// then A_c[ic, jc] accumulates (R A)[ic, g] R[jc, g] over g ascending and
// the parents jc of g in ascending order.  Every operator here is at most a
// 27-point stencil, so the work arrays are small boxes around the coarse
// vertex: (R A)[ic, .] lives within +-2 fine cells of 2 ic and A_c[ic, .]
// within +-1 coarse cells of ic.
static std::shared_ptr<LinOp> coarsen(const LinOp &op, const Intergrid &ig) {
    auto cop = std::make_shared<LinOp>(ig.crs);
    const Lattice &fl = op.lat, &cl = ig.crs;
    int64_t nc = cl.nvertex();
    int S = ig.S;
    Csr &Ac = cop->A;
    Ac.n = nc;
    std::vector<std::vector<int64_t>> colv(nc);
    std::vector<std::vector<double>> valv(nc);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t ic = 0; ic < nc; ++ic) {
        double RA[125];
        bool hitRA[125];
        double AC[27];
        bool hitAC[27];
        for (int q = 0; q < 125; ++q) {
            RA[q] = 0.0;
            hitRA[q] = false;
        }
        for (int q = 0; q < 27; ++q) {
            AC[q] = 0.0;
            hitAC[q] = false;
        }
        int c[3];
        cl.vertex_euclid(ic, c);
        int ctr[3] = {2 * c[0], fl.dim > 1 ? 2 * c[1] : 1, fl.dim > 2 ? 2 * c[2] : 1};
        for (int k = 0; k < S; ++k) {
            int64_t f = ig.colidx[ic * S + k];
            double w = ig.matrix[k];
            for (int64_t e = op.A.ptr[f]; e < op.A.ptr[f + 1]; ++e) {
                int g[3];
                fl.vertex_euclid(op.A.col[e], g);
                int q = (g[2] - ctr[2] + 2) * 25 + (g[1] - ctr[1] + 2) * 5 + (g[0] - ctr[0] + 2);
                RA[q] += w * op.A.val[e];
                hitRA[q] = true;
            }
        }
        // slots in ascending global index order = (z, y, x) lexicographic
        for (int q = 0; q < 125; ++q) {
            if (!hitRA[q]) continue;
            int g[3] = {ctr[0] + q % 5 - 2, ctr[1] + (q / 5) % 5 - 2, ctr[2] + q / 25 - 2};
            // coarse parents jc of g: R[jc, g] = prod_d {1/2, 1, 1/2}[g_d - 2 jc_d]
            int pc[3][2], np_[3];
            double pw[3][2];
            for (int d = 0; d < 3; ++d) {
                if (d >= fl.dim) {
                    np_[d] = 1;
                    pc[d][0] = 1;
                    pw[d][0] = 1.0;
                } else if (g[d] % 2 == 0) {
                    np_[d] = 1;
                    pc[d][0] = g[d] / 2;
                    pw[d][0] = 1.0;
                } else {
                    np_[d] = 2;
                    pc[d][0] = (g[d] - 1) / 2;
                    pc[d][1] = (g[d] + 1) / 2;
                    pw[d][0] = pw[d][1] = 0.5;
                }
            }
            for (int a2 = 0; a2 < np_[2]; ++a2)
                for (int a1 = 0; a1 < np_[1]; ++a1)
                    for (int a0 = 0; a0 < np_[0]; ++a0) {
                        int jc[3] = {pc[0][a0], pc[1][a1], pc[2][a2]};
                        if (!cl.is_interior(jc)) continue;
                        // weight product in the order of intergrid_operator_linear.cc:16-29
                        double w = 1.0;
                        w *= pw[0][a0];
                        if (fl.dim > 1) w *= pw[1][a1];
                        if (fl.dim > 2) w *= pw[2][a2];
                        int qc = (jc[2] - c[2] + 1) * 9 + (jc[1] - c[1] + 1) * 3 + (jc[0] - c[0] + 1);
                        AC[qc] += RA[q] * w;
                        hitAC[qc] = true;
                    }
        }
        for (int qc = 0; qc < 27; ++qc) {
            if (!hitAC[qc]) continue;
            int jc[3] = {c[0] + qc % 3 - 1, c[1] + (qc / 3) % 3 - 1, c[2] + qc / 9 - 1};
            colv[ic].push_back(cl.vertex_linear(jc));
            valv[ic].push_back(AC[qc]);
        }
    }
    Ac.ptr.assign(nc + 1, 0);
    for (int64_t ic = 0; ic < nc; ++ic) Ac.ptr[ic + 1] = Ac.ptr[ic] + (int64_t)colv[ic].size();
    Ac.col.resize(Ac.ptr[nc]);
    Ac.val.resize(Ac.ptr[nc]);
    for (int64_t ic = 0; ic < nc; ++ic) {
        std::copy(colv[ic].begin(), colv[ic].end(), Ac.col.begin() + Ac.ptr[ic]);
        std::copy(valv[ic].begin(), valv[ic].end(), Ac.val.begin() + Ac.ptr[ic]);
    }
    Ac.finish_diag();
    // B_c = R B: coarse vertex ic collects the fine entries 2 ic + a of each
    // column; structural entries are kept even where the sum is zero
    cop->B.nrow = nc;
    cop->B.m = op.B.m;
    cop->B.ptr.assign(1, 0);
    for (int j = 0; j < op.B.m; ++j) {
        std::map<int64_t, std::vector<std::pair<int, double>>> contrib;  // ic -> (k, value)
        for (int64_t e = op.B.ptr[j]; e < op.B.ptr[j + 1]; ++e) {
            int g[3];
            fl.vertex_euclid(op.B.row[e], g);
            for (int dz = -1; dz <= 1; ++dz)
                for (int dy = -1; dy <= 1; ++dy)
                    for (int dx = -1; dx <= 1; ++dx) {
                        if ((fl.dim < 2 && dy) || (fl.dim < 3 && dz)) continue;
                        int f2[3] = {g[0] - dx, g[1] - dy, g[2] - dz};  // candidate 2 ic
                        if ((f2[0] % 2) || (fl.dim > 1 && f2[1] % 2) || (fl.dim > 2 && f2[2] % 2)) continue;
                        int jc[3] = {f2[0] / 2, fl.dim > 1 ? f2[1] / 2 : 1, fl.dim > 2 ? f2[2] / 2 : 1};
                        if (!cl.is_interior(jc)) continue;
                        int k = (dx + 1) + (fl.dim > 1 ? 3 * (dy + 1) : 0) + (fl.dim > 2 ? 9 * (dz + 1) : 0);
                        contrib[cl.vertex_linear(jc)].push_back({k, op.B.val[e]});
                    }
        }
        for (auto &kv : contrib) {
            // restrict(): sum over the stencil entries k in ascending order
            std::sort(kv.second.begin(), kv.second.end(),
                      [](const std::pair<int, double> &a, const std::pair<int, double> &b) { return a.first < b.first; });
            double acc = 0.0;
            for (auto &kvv : kv.second) acc += ig.matrix[kvv.first] * kvv.second;
            cop->B.row.push_back(kv.first);
            cop->B.val.push_back(acc);
        }
        cop->B.ptr.push_back((int64_t)cop->B.row.size());
    }
    cop->Sigma = op.Sigma;
    return cop;
}

// ---------------------------------------------------------------------------
// Random numbers: parallel_random.cc:9-78 (CLCG + Marsaglia polar method).
// ---------------------------------------------------------------------------
struct NormalSource {
    virtual ~NormalSource() = default;
    virtual double draw_normal() = 0;
};

struct CLCG : NormalSource {
    int32_t y1 = 1, y2 = 1;
    const int32_t a1 = 40014, m1 = 2147483563, a2 = 40692, m2 = 2147483399;
    const double m1_inv = 1. / 2147483563.;
    int64_t a1_multistep, a2_multistep;
    bool redraw = true;
    double z_1 = 0, z_2 = 0;
    // parallel_random.cc:35-59 with explicit thread count / id (leapfrog)
    CLCG(int n_threads = 1, int thread_id = 0) {
        a1_multistep = a1;
        a2_multistep = a2;
        for (int j = 1; j < n_threads; ++j) {
            if (j <= thread_id) {
                y1 = (int32_t)(((int64_t)a1 * y1) % m1);
                y2 = (int32_t)(((int64_t)a2 * y2) % m2);
            }
            a1_multistep = (a1_multistep * a1) % m1;
            a2_multistep = (a2_multistep * a2) % m2;
        }
    }
    int32_t draw_int() {  // parallel_random.cc:62-71
        int32_t x = y1 - y2;
        if (x < 1) x += m1 - 1;
        y1 = (int32_t)((a1_multistep * y1) % m1);
        y2 = (int32_t)((a2_multistep * y2) % m2);
        return x;
    }
    double draw_uniform_real() { return draw_int() * m1_inv; }
    double draw_normal() override {  // parallel_random.cc:9-32
        if (redraw) {
            double u1, u2, s;
            do {
                u1 = 2. * draw_uniform_real() - 1.;
                u2 = 2. * draw_uniform_real() - 1.;
                s = u1 * u1 + u2 * u2;
            } while ((s == 0) || (s >= 1));
            double L = sqrt(-2 * log(s) / s);
            z_1 = L * u1;
            z_2 = L * u2;
            redraw = false;
            return z_1;
        }
        redraw = true;
        return z_2;
    }
};

// Injected noise: the k-th call returns data[k] (parity runs).
struct BufferSource : NormalSource {
    std::vector<double> data;
    size_t pos = 0;
    double draw_normal() override {
        if (pos >= data.size()) throw std::runtime_error("injected noise exhausted");
        return data[pos++];
    }
};

// ---------------------------------------------------------------------------
// Dense helpers
// ---------------------------------------------------------------------------
// LU with partial pivoting inverse (Eigen's .inverse() for m > 4 uses
// PartialPivLU; the result agrees to rounding).
static std::vector<double> dense_inverse(const std::vector<double> &A, int m) {
    std::vector<double> LU = A, inv(m * m, 0.0);
    std::vector<int> piv(m);
    for (int i = 0; i < m; ++i) piv[i] = i;
    for (int k = 0; k < m; ++k) {
        int p = k;
        for (int i = k + 1; i < m; ++i)
            if (fabs(LU[i * m + k]) > fabs(LU[p * m + k])) p = i;
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

// Natural-order dense Cholesky A = L L^T (lower, row-major); returns false
// if a pivot is not positive.
static bool dense_cholesky(std::vector<double> &A, int64_t n) {
    for (int64_t j = 0; j < n; ++j) {
        double s = A[j * n + j];
        for (int64_t k = 0; k < j; ++k) s -= A[j * n + k] * A[j * n + k];
        if (!(s > 0.0)) return false;
        double d = sqrt(s);
        A[j * n + j] = d;
        for (int64_t i = j + 1; i < n; ++i) {
            double t = A[i * n + j];
            for (int64_t k = 0; k < j; ++k) t -= A[i * n + k] * A[j * n + k];
            A[i * n + j] = t / d;
        }
        for (int64_t i = 0; i < j; ++i) A[i * n + j] = 0.0;
    }
    return true;
}

// ---------------------------------------------------------------------------
// Sweep ordering.  ordering 0: lexicographic (the reference);
// ordering 1: multicolour -- 2 colours when the stencil couples only axis
// neighbours, 2^dim colours otherwise; colours visited 0..C-1 forward and
// C-1..0 backward, ascending index inside a colour.
// ---------------------------------------------------------------------------
static std::vector<int64_t> sweep_order(const LinOp &op, int ordering, bool forward, std::vector<int> *colour_out) {
    int64_t n = op.n();
    std::vector<int64_t> order(n);
    if (ordering == 0) {
        for (int64_t i = 0; i < n; ++i) order[i] = forward ? i : n - 1 - i;
        if (colour_out) {
            colour_out->assign(n, 0);
            for (int64_t i = 0; i < n; ++i) (*colour_out)[i] = (int)i;  // rank = index
        }
        return order;
    }
    bool diagonal = false;
    for (int64_t i = 0; i < n && !diagonal; ++i) {
        int a[3];
        op.lat.vertex_euclid(i, a);
        for (int64_t k = op.A.ptr[i]; k < op.A.ptr[i + 1]; ++k) {
            int b[3];
            op.lat.vertex_euclid(op.A.col[k], b);
            int nz = (a[0] != b[0]) + (a[1] != b[1]) + (a[2] != b[2]);
            if (nz > 1) {
                diagonal = true;
                break;
            }
        }
    }
    int ncol = diagonal ? (1 << op.lat.dim) : 2;
    std::vector<int> colour(n);
    for (int64_t i = 0; i < n; ++i) colour[i] = vertex_colour(op.lat, i, ncol);
    int64_t p = 0;
    for (int c = 0; c < ncol; ++c) {
        int cc = forward ? c : ncol - 1 - c;
        if (forward) {
            for (int64_t i = 0; i < n; ++i)
                if (colour[i] == cc) order[p++] = i;
        } else {
            for (int64_t i = n - 1; i >= 0; --i)
                if (colour[i] == cc) order[p++] = i;
        }
    }
    if (colour_out) *colour_out = colour;
    return order;
}

// ---------------------------------------------------------------------------
// SOR smoother: sor_smoother.cc:9-78
// ---------------------------------------------------------------------------
// Bbar is a function of (operator, direction, ordering, omega); samplers of
// one hierarchy share it instead of holding the reference's four identical
// pairs per level (ssor_sampler.hh:37-38, multigridmc_sampler.cc:92-95).
typedef std::map<std::tuple<const LinOp *, bool, int, double>, std::shared_ptr<std::vector<double>>> BbarCache;

struct SORSmoother {
    std::shared_ptr<LinOp> op;
    double omega;
    bool forward;
    int ordering;
    std::vector<int64_t> order;
    std::shared_ptr<std::vector<double>> Bbar;  // n x m row-major, dense (sor_smoother.cc:25-35)
    SORSmoother(std::shared_ptr<LinOp> op_, double omega_, bool forward_, int ordering_, BbarCache *cache = nullptr)
        : op(op_), omega(omega_), forward(forward_), ordering(ordering_) {
        order = sweep_order(*op, ordering, forward, nullptr);
        int m = op->m();
        if (m == 0) return;
        auto key = std::make_tuple((const LinOp *)op.get(), forward, ordering, omega);
        if (cache && cache->count(key)) {
            Bbar = (*cache)[key];
            return;
        }
        Bbar = std::make_shared<std::vector<double>>(build_bbar());
        if (cache) (*cache)[key] = Bbar;
    }
    std::vector<double> build_bbar() const {
        const int m = op->m();
        const int64_t n = op->n();
        std::vector<int64_t> pos(n);
        for (int64_t p = 0; p < n; ++p) pos[order[p]] = p;
        std::vector<double> X((size_t)n * m, 0.0);  // (L + D/omega)^{-1} B, row-major
        for (int j = 0; j < m; ++j)
            for (int64_t k = op->B.ptr[j]; k < op->B.ptr[j + 1]; ++k) X[(size_t)op->B.row[k] * m + j] = op->B.val[k];
        // diag entries a + (1-omega)/omega * a (sor_smoother.cc:22-23);
        // substitution along the sweep, earlier entries subtracted in the
        // order they were computed (Eigen's column-oriented triangular solve)
        const double scal = (1. - omega) / omega;
        std::vector<std::pair<int64_t, double>> prev;
        for (int64_t p = 0; p < n; ++p) {
            int64_t i = order[p];
            double dii = op->A.diag[i] + scal * op->A.diag[i];
            prev.clear();
            for (int64_t k = op->A.ptr[i]; k < op->A.ptr[i + 1]; ++k) {
                int64_t c = op->A.col[k];
                if (c != i && pos[c] < p) prev.push_back({pos[c], op->A.val[k]});
            }
            std::sort(prev.begin(), prev.end());
            double *Xi = &X[(size_t)i * m];
            for (auto &e : prev) {
                const double *Xc = &X[(size_t)order[e.first] * m];
                for (int j = 0; j < m; ++j) Xi[j] -= e.second * Xc[j];
            }
            for (int j = 0; j < m; ++j) Xi[j] = Xi[j] / dii;
        }
        // S = Sigma + B^T (L + D/omega)^{-1} B;  Bbar = X S^{-1}
        std::vector<double> S((size_t)m * m, 0.0);
        for (int a = 0; a < m; ++a) {
            for (int b = 0; b < m; ++b) {
                double acc = 0.0;
                for (int64_t k = op->B.ptr[a]; k < op->B.ptr[a + 1]; ++k) acc += op->B.val[k] * X[(size_t)op->B.row[k] * m + b];
                S[a * m + b] = acc;
            }
            S[a * m + a] += op->Sigma[a];
        }
        std::vector<double> Sinv = dense_inverse(S, m);
#pragma omp parallel for schedule(static) if (n > 100000)
        for (int64_t i = 0; i < n; ++i) {
            double row[4096];
            double *Xi = &X[(size_t)i * m];
            for (int b = 0; b < m; ++b) {
                double acc = 0.0;
                for (int a = 0; a < m; ++a) acc += Xi[a] * Sinv[a * m + b];
                row[b] = acc;
            }
            for (int b = 0; b < m; ++b) Xi[b] = row[b];
        }
        return X;
    }
    // sor_smoother.cc:56-78
    void apply_sparse(const double *b, double *x) const {
        const Csr &A = op->A;
        for (int64_t p = 0; p < A.n; ++p) {
            int64_t ell = order[p];
            double residual = 0.0;
            for (int64_t k = A.ptr[ell]; k < A.ptr[ell + 1]; ++k) residual += A.val[k] * x[A.col[k]];
            x[ell] += omega * (b[ell] - residual) / A.diag[ell];
        }
    }
    // sor_smoother.cc:40-54 (nsmooth = 1)
    void apply(const double *b, double *x) const {
        apply_sparse(b, x);
        int m = op->m();
        if (m > 0) {
            std::vector<double> y(m, 0.0);
            for (int j = 0; j < m; ++j) {
                double acc = 0.0;
                for (int64_t k = op->B.ptr[j]; k < op->B.ptr[j + 1]; ++k) acc += op->B.val[k] * x[op->B.row[k]];
                y[j] = acc;
            }
            const int64_t n = op->n();
            const double *Bb = Bbar->data();
#pragma omp parallel for schedule(static) if (n > 100000)
            for (int64_t i = 0; i < n; ++i) {
                double acc = 0.0;
                for (int j = 0; j < m; ++j) acc += Bb[(size_t)i * m + j] * y[j];
                x[i] -= acc;
            }
        }
    }
};

// ---------------------------------------------------------------------------
// Samplers
// ---------------------------------------------------------------------------
struct Sampler {
    virtual ~Sampler() = default;
    virtual void apply(const double *f, double *x) = 0;
};

// sor_sampler.cc:9-59
struct SORSampler : Sampler {
    std::shared_ptr<LinOp> op;
    NormalSource *rng;
    double omega;
    int nsmooth;
    SORSmoother smoother;
    std::vector<double> sqrt_precision_diag, Sigma_inv_sqrt, c_rhs, xi;
    SORSampler(std::shared_ptr<LinOp> op_, NormalSource *rng_, double omega_, int nsmooth_, bool forward, int ordering,
               BbarCache *cache = nullptr)
        : op(op_), rng(rng_), omega(omega_), nsmooth(nsmooth_), smoother(op_, omega_, forward, ordering, cache) {
        int64_t n = op->n();
        sqrt_precision_diag.resize(n);
        for (int64_t ell = 0; ell < n; ++ell)
            sqrt_precision_diag[ell] = sqrt(op->A.diag[ell] * (2. - omega) / omega);
        c_rhs.resize(n);
        xi.resize(op->m());
        Sigma_inv_sqrt.resize(op->m());
        for (int j = 0; j < op->m(); ++j) Sigma_inv_sqrt[j] = sqrt(1.0 / op->Sigma[j]);
    }
    void apply(const double *f, double *x) override {
        int64_t n = op->n();
        for (int k = 0; k < nsmooth; ++k) {
            for (int64_t ell = 0; ell < n; ++ell) {
                double tmp = sqrt_precision_diag[ell];
                c_rhs[ell] = tmp * rng->draw_normal() + f[ell];
            }
            int m = op->m();
            if (m > 0) {
                for (int j = 0; j < m; ++j) xi[j] = rng->draw_normal();
                for (int j = 0; j < m; ++j) {
                    double s = Sigma_inv_sqrt[j] * xi[j];
                    for (int64_t e = op->B.ptr[j]; e < op->B.ptr[j + 1]; ++e) c_rhs[op->B.row[e]] += op->B.val[e] * s;
                }
            }
            smoother.apply(c_rhs.data(), x);
        }
    }
};

// ssor_sampler.{hh,cc}
struct SSORSampler : Sampler {
    SORSampler fwd, bwd;
    int nsmooth;
    SSORSampler(std::shared_ptr<LinOp> op, NormalSource *rng, double omega, int nsmooth_, int ordering,
                BbarCache *cache = nullptr)
        : fwd(op, rng, omega, 1, true, ordering, cache), bwd(op, rng, omega, 1, false, ordering, cache), nsmooth(nsmooth_) {}
    void apply(const double *f, double *x) override {
        for (int k = 0; k < nsmooth; ++k) {
            fwd.apply(f, x);
            bwd.apply(f, x);
        }
    }
};

// cholesky_sampler.hh:52-66 with the dense natural-order factor of
// cholesky_sampler.cc:25-37 / cholesky_wrapper.cc:128-155.
struct CholeskySampler : Sampler {
    std::shared_ptr<LinOp> op;
    NormalSource *rng;
    int64_t n;
    std::vector<double> L, xi, g;
    bool ok;
    CholeskySampler(std::shared_ptr<LinOp> op_, NormalSource *rng_) : op(op_), rng(rng_) {
        n = op->n();
        L = op->precision_dense();
        ok = dense_cholesky(L, n);
        xi.resize(n);
        g.resize(n);
    }
    void apply(const double *f, double *x) override {
        for (int64_t ell = 0; ell < n; ++ell) xi[ell] = rng->draw_normal();
        for (int64_t i = 0; i < n; ++i) {  // L g = f
            double s = f[i];
            for (int64_t k = 0; k < i; ++k) s -= L[i * n + k] * g[k];
            g[i] = s / L[i * n + i];
        }
        for (int64_t i = 0; i < n; ++i) xi[i] = xi[i] + g[i];
        // L^T x = xi + g, column-oriented back substitution: the terms of
        // row i are subtracted in the order the x[k] are computed (k
        // descending), as in Eigen's triangular solvers
        for (int64_t i = n - 1; i >= 0; --i) {
            double s = xi[i];
            for (int64_t k = n - 1; k > i; --k) s -= L[k * n + i] * x[k];
            x[i] = s / L[i * n + i];
        }
    }
};

// cholesky_sampler.cc:41-129 (LowRankCholeskySampler): the sparse part A_0 is
// factored (here by the dense natural-order LL^T), the low-rank term enters
// through V = L^{-1} B, its thin QR V = QR (Householder, R with a positive
// diagonal: the sampler does not depend on the signs of Q's columns), the
// m x m matrix Id - Lambda = Id - R (Sigma + V^T V)^{-1} R^T and its lower
// Cholesky factor W, with Q_W = Q (W^T - Id), Q_W_T = Q (W - Id).  A sample
// draws n normals xi, forms g = L^{-1} f, g += Q_W (Q^T g), xi += g,
// xi += Q_W_T (Q^T xi) and solves L^T x = xi.
struct LowRankCholeskySampler : Sampler {
    std::shared_ptr<LinOp> op;
    NormalSource *rng;
    int64_t n;
    int m;
    std::vector<double> L, Q, QW, QWT, xi, g, t;  // L n x n row-major; Q, QW, QWT n x m row-major
    bool ok = true;
    LowRankCholeskySampler(std::shared_ptr<LinOp> op_, NormalSource *rng_) : op(op_), rng(rng_) {
        n = op->n();
        m = op->m();
        L.assign(n * n, 0.0);
        for (int64_t i = 0; i < n; ++i)
            for (int64_t k = op->A.ptr[i]; k < op->A.ptr[i + 1]; ++k) L[i * n + op->A.col[k]] = op->A.val[k];
        ok = dense_cholesky(L, n);
        xi.resize(n);
        g.resize(n);
        t.resize(std::max(m, 1));
        if (!ok || m == 0) return;
        // V = L^{-1} B, column by column (forward substitution)
        std::vector<double> V(n * m, 0.0), b(n);
        for (int j = 0; j < m; ++j) {
            std::fill(b.begin(), b.end(), 0.0);
            for (int64_t e = op->B.ptr[j]; e < op->B.ptr[j + 1]; ++e) b[op->B.row[e]] = op->B.val[e];
            for (int64_t i = 0; i < n; ++i) {
                double s = b[i];
                for (int64_t k = 0; k < i; ++k) s -= L[i * n + k] * V[k * m + j];
                V[i * m + j] = s / L[i * n + i];
            }
        }
        // Householder QR of V (n x m): reflectors applied to a copy, R from
        // the reduced matrix, Q from the reflectors applied to Id(n x m)
        std::vector<double> A = V, tau(m, 0.0), vk(n);
        std::vector<std::vector<double>> refl(m);
        for (int k = 0; k < m; ++k) {
            double nrm = 0.0;
            for (int64_t i = k; i < n; ++i) nrm += A[i * m + k] * A[i * m + k];
            nrm = sqrt(nrm);
            const double a0 = A[k * m + k];
            const double alpha = a0 >= 0.0 ? -nrm : nrm;
            std::vector<double> v(n, 0.0);
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
            refl[k] = v;
        }
        std::vector<double> R(m * m, 0.0);
        for (int i = 0; i < m; ++i)
            for (int c = i; c < m; ++c) R[i * m + c] = A[i * m + c];
        Q.assign(n * m, 0.0);
        for (int c = 0; c < m; ++c) Q[c * m + c] = 1.0;
        for (int k = m - 1; k >= 0; --k) {
            const std::vector<double> &v = refl[k];
            for (int c = 0; c < m; ++c) {
                double d = 0.0;
                for (int64_t i = k; i < n; ++i) d += v[i] * Q[i * m + c];
                const double sc = tau[k] * d;
                for (int64_t i = k; i < n; ++i) Q[i * m + c] -= sc * v[i];
            }
        }
        // signs: a positive diagonal of R (column c of Q and row c of R flip together)
        for (int c = 0; c < m; ++c)
            if (R[c * m + c] < 0.0) {
                for (int cc = 0; cc < m; ++cc) R[c * m + cc] = -R[c * m + cc];
                for (int64_t i = 0; i < n; ++i) Q[i * m + c] = -Q[i * m + c];
            }
        // Id - Lambda = Id - R (Sigma + V^T V)^{-1} R^T
        std::vector<double> S(m * m, 0.0);
        for (int a = 0; a < m; ++a)
            for (int c = 0; c < m; ++c) {
                double d = 0.0;
                for (int64_t i = 0; i < n; ++i) d += V[i * m + a] * V[i * m + c];
                S[a * m + c] = d + (a == c ? op->Sigma[a] : 0.0);
            }
        const std::vector<double> Si = dense_inverse(S, m);
        std::vector<double> RSi(m * m, 0.0), W(m * m, 0.0);
        for (int a = 0; a < m; ++a)
            for (int c = 0; c < m; ++c) {
                double d = 0.0;
                for (int k = 0; k < m; ++k) d += R[a * m + k] * Si[k * m + c];
                RSi[a * m + c] = d;
            }
        for (int a = 0; a < m; ++a)
            for (int c = 0; c < m; ++c) {
                double d = 0.0;
                for (int k = 0; k < m; ++k) d += RSi[a * m + k] * R[c * m + k];
                W[a * m + c] = (a == c ? 1.0 : 0.0) - d;
            }
        if (!dense_cholesky(W, m)) {
            ok = false;
            return;
        }
        // Q_W = Q (W^T - Id), Q_W_T = Q (W - Id)
        QW.assign(n * m, 0.0);
        QWT.assign(n * m, 0.0);
        for (int64_t i = 0; i < n; ++i)
            for (int c = 0; c < m; ++c) {
                double u = 0.0, l = 0.0;
                for (int k = 0; k < m; ++k) {
                    const double wt = W[c * m + k] - (k == c ? 1.0 : 0.0);  // (W^T - Id)[k][c] = W[c][k] - d
                    const double w = W[k * m + c] - (k == c ? 1.0 : 0.0);   // (W - Id)[k][c]
                    u += Q[i * m + k] * wt;
                    l += Q[i * m + k] * w;
                }
                QW[i * m + c] = u;
                QWT[i * m + c] = l;
            }
    }
    // y += Qx (Q^T v)
    void lowrank_update(const std::vector<double> &Qx, const std::vector<double> &v, std::vector<double> &y) {
        for (int c = 0; c < m; ++c) {
            double d = 0.0;
            for (int64_t i = 0; i < n; ++i) d += Q[i * m + c] * v[i];
            t[c] = d;
        }
        for (int64_t i = 0; i < n; ++i) {
            double d = 0.0;
            for (int c = 0; c < m; ++c) d += Qx[i * m + c] * t[c];
            y[i] += d;
        }
    }
    void apply(const double *f, double *x) override {
        for (int64_t ell = 0; ell < n; ++ell) xi[ell] = rng->draw_normal();
        for (int64_t i = 0; i < n; ++i) {  // L g = f
            double s = f[i];
            for (int64_t k = 0; k < i; ++k) s -= L[i * n + k] * g[k];
            g[i] = s / L[i * n + i];
        }
        if (m > 0) lowrank_update(QW, g, g);
        for (int64_t i = 0; i < n; ++i) xi[i] += g[i];
        if (m > 0) lowrank_update(QWT, xi, xi);
        for (int64_t i = n - 1; i >= 0; --i) {  // L^T x = xi
            double s = xi[i];
            for (int64_t k = n - 1; k > i; --k) s -= L[k * n + i] * x[k];
            x[i] = s / L[i * n + i];
        }
    }
};

struct MGParams {
    int nlevel;
    int smoother;       // 0 = SOR, 1 = SSOR
    int coarse_solver;  // 0 = Cholesky, 1 = SSOR
    int npresmooth, npostsmooth, ncoarsesmooth;
    double omega;
    int cycle;
    double coarse_scaling;
    int ordering;
};

// multigridmc_sampler.cc:8-145
struct MGMCSampler : Sampler {
    MGParams p;
    NormalSource *rng;
    std::vector<std::shared_ptr<LinOp>> ops;
    std::vector<std::unique_ptr<Sampler>> pre, post;
    std::vector<std::unique_ptr<Intergrid>> ig;
    std::unique_ptr<Sampler> coarse;
    std::vector<std::vector<double>> x_ell, f_ell, r_ell;
    BbarCache cache;
    MGMCSampler(std::shared_ptr<LinOp> op, NormalSource *rng_, const MGParams &p_) : p(p_), rng(rng_) {
        std::shared_ptr<LinOp> lin_op = op;
        for (int level = 0; level < p.nlevel; ++level) {
            int64_t n = lin_op->n();
            x_ell.emplace_back(n, 0.0);
            f_ell.emplace_back(n, 0.0);
            r_ell.emplace_back(n, 0.0);
            ops.push_back(lin_op);
            if (p.smoother == 1) {
                pre.emplace_back(new SSORSampler(lin_op, rng, p.omega, p.npresmooth, p.ordering, &cache));
                post.emplace_back(new SSORSampler(lin_op, rng, p.omega, p.npostsmooth, p.ordering, &cache));
            } else {
                pre.emplace_back(new SORSampler(lin_op, rng, p.omega, p.npresmooth, true, p.ordering, &cache));
                post.emplace_back(new SORSampler(lin_op, rng, p.omega, p.npostsmooth, false, p.ordering, &cache));
            }
            if (level < p.nlevel - 1) {
                if (!lin_op->lat.coarsenable()) throw std::runtime_error("cannot coarsen lattice");
                ig.emplace_back(new Intergrid(lin_op->lat));
                lin_op = coarsen(*lin_op, *ig.back());
            }
        }
        if (p.coarse_solver == 0)
            coarse.reset(new CholeskySampler(lin_op, rng));
        else
            coarse.reset(new SSORSampler(lin_op, rng, p.omega, p.ncoarsesmooth, p.ordering, &cache));
    }
    void sample(int level) {
        if (level == p.nlevel - 1) {
            coarse->apply(f_ell[level].data(), x_ell[level].data());
            return;
        }
        int cyc = (level > 0) ? p.cycle : 1;
        for (int j = 0; j < cyc; ++j) {
            pre[level]->apply(f_ell[level].data(), x_ell[level].data());
            ops[level]->apply(x_ell[level].data(), r_ell[level].data());
            int64_t n = ops[level]->n();
            for (int64_t i = 0; i < n; ++i) r_ell[level][i] = f_ell[level][i] - r_ell[level][i];
            ig[level]->restrict_(r_ell[level].data(), f_ell[level + 1].data());
            std::fill(x_ell[level + 1].begin(), x_ell[level + 1].end(), 0.0);
            sample(level + 1);
            ig[level]->prolongate_add(p.coarse_scaling, x_ell[level + 1].data(), x_ell[level].data());
            post[level]->apply(f_ell[level].data(), x_ell[level].data());
        }
    }
    void apply(const double *f, double *x) override {
        int64_t n = ops[0]->n();
        std::copy(f, f + n, f_ell[0].begin());
        std::copy(x, x + n, x_ell[0].begin());
        sample(0);
        std::copy(x_ell[0].begin(), x_ell[0].end(), x);
    }
};

// ---------------------------------------------------------------------------
// Deterministic solvers: cholesky_solver.cc:9-43, multigrid_preconditioner.cc
// :8-108, loop_solver.cc:9-53.
// ---------------------------------------------------------------------------
// CholeskySolver: factor the sparse part A_0 and apply the low-rank term by
// the Woodbury identity, x = y - Bbar B^T y with y = A_0^{-1} b and
// Bbar = A_0^{-1} B (Sigma + B^T A_0^{-1} B)^{-1} (cholesky_solver.cc:9-43).
// The factor is the dense natural-order one (the reference: Eigen's
// SimplicialLLT with AMD ordering; the solution agrees to rounding).
struct CholeskySolver {
    std::shared_ptr<LinOp> op;
    int64_t n;
    std::vector<double> L, Bbar;  // Bbar n x m row-major
    bool ok;
    explicit CholeskySolver(std::shared_ptr<LinOp> op_) : op(op_) {
        n = op->n();
        L.assign(n * n, 0.0);
        for (int64_t i = 0; i < n; ++i)
            for (int64_t k = op->A.ptr[i]; k < op->A.ptr[i + 1]; ++k) L[i * n + op->A.col[k]] = op->A.val[k];
        ok = dense_cholesky(L, n);
        const int m = op->m();
        if (!ok || m == 0) return;
        std::vector<double> AinvB((size_t)n * m), col(n), y(n);
        for (int j = 0; j < m; ++j) {
            std::fill(col.begin(), col.end(), 0.0);
            for (int64_t e = op->B.ptr[j]; e < op->B.ptr[j + 1]; ++e) col[op->B.row[e]] = op->B.val[e];
            solve_A0(col.data(), y.data());
            for (int64_t i = 0; i < n; ++i) AinvB[(size_t)i * m + j] = y[i];
        }
        std::vector<double> S((size_t)m * m, 0.0);  // Sigma + B^T A_0^{-1} B
        for (int a = 0; a < m; ++a) {
            for (int b = 0; b < m; ++b) {
                double acc = 0.0;
                for (int64_t e = op->B.ptr[a]; e < op->B.ptr[a + 1]; ++e) acc += op->B.val[e] * AinvB[(size_t)op->B.row[e] * m + b];
                S[a * m + b] = acc;
            }
            S[a * m + a] += op->Sigma[a];
        }
        std::vector<double> Sinv = dense_inverse(S, m);
        Bbar.assign((size_t)n * m, 0.0);
        for (int64_t i = 0; i < n; ++i)
            for (int b = 0; b < m; ++b) {
                double acc = 0.0;
                for (int a = 0; a < m; ++a) acc += AinvB[(size_t)i * m + a] * Sinv[a * m + b];
                Bbar[(size_t)i * m + b] = acc;
            }
    }
    void solve_A0(const double *b, double *x) const {  // L L^T x = b
        std::vector<double> g(n);
        for (int64_t i = 0; i < n; ++i) {
            double s = b[i];
            for (int64_t k = 0; k < i; ++k) s -= L[i * n + k] * g[k];
            g[i] = s / L[i * n + i];
        }
        for (int64_t i = n - 1; i >= 0; --i) {
            double s = g[i];
            for (int64_t k = n - 1; k > i; --k) s -= L[k * n + i] * x[k];
            x[i] = s / L[i * n + i];
        }
    }
    void apply(const double *b, double *x) const {  // cholesky_solver.cc:29-43
        const int m = op->m();
        if (m == 0) {
            solve_A0(b, x);
            return;
        }
        std::vector<double> y(n), BTy(m, 0.0);
        solve_A0(b, y.data());
        for (int j = 0; j < m; ++j) {
            double acc = 0.0;
            for (int64_t e = op->B.ptr[j]; e < op->B.ptr[j + 1]; ++e) acc += op->B.val[e] * y[op->B.row[e]];
            BTy[j] = acc;
        }
        for (int64_t i = 0; i < n; ++i) {
            double acc = 0.0;
            for (int j = 0; j < m; ++j) acc += Bbar[(size_t)i * m + j] * BTy[j];
            x[i] = y[i] - acc;
        }
    }
};

// MultigridPreconditioner (multigrid_preconditioner.cc:8-108).  The coarse
// solve is the CholeskySolver above (woodbury = true) or the noise-free
// dense natural-order Cholesky sample of the full coarse precision
// (woodbury = false), the form the GPU computes; both give Q_c^{-1} b to
// rounding.
struct MGPreconditioner {
    MGParams p;
    bool woodbury;
    std::vector<std::shared_ptr<LinOp>> ops;
    std::vector<std::unique_ptr<SORSmoother>> fwd, bwd;
    std::vector<std::unique_ptr<Intergrid>> ig;
    std::unique_ptr<CholeskySolver> coarse_w;
    std::unique_ptr<CholeskySampler> coarse_d;
    BufferSource zeros;  // the noise of the dense coarse sample: zero
    std::vector<std::vector<double>> x_ell, b_ell, r_ell;
    BbarCache cache;
    bool ok = true;
    MGPreconditioner(std::shared_ptr<LinOp> op, const MGParams &p_, bool woodbury_) : p(p_), woodbury(woodbury_) {
        std::shared_ptr<LinOp> lin_op = op;
        for (int level = 0; level < p.nlevel; ++level) {
            int64_t n = lin_op->n();
            x_ell.emplace_back(n, 0.0);
            b_ell.emplace_back(n, 0.0);
            r_ell.emplace_back(n, 0.0);
            ops.push_back(lin_op);
            fwd.emplace_back(new SORSmoother(lin_op, p.omega, true, p.ordering, &cache));
            bwd.emplace_back(new SORSmoother(lin_op, p.omega, false, p.ordering, &cache));
            if (level < p.nlevel - 1) {
                if (!lin_op->lat.coarsenable()) throw std::runtime_error("cannot coarsen lattice");
                ig.emplace_back(new Intergrid(lin_op->lat));
                lin_op = coarsen(*lin_op, *ig.back());
            }
        }
        if (woodbury) {
            coarse_w.reset(new CholeskySolver(lin_op));
            ok = coarse_w->ok;
        } else {
            zeros.data.assign((size_t)lin_op->n(), 0.0);
            coarse_d.reset(new CholeskySampler(lin_op, &zeros));
            ok = coarse_d->ok;
        }
    }
    // SORSmoother::apply with nsmooth passes (sor_smoother.cc:40-78): nsmooth
    // times nsmooth sparse sweeps and one low-rank correction
    void sor_smooth(const SORSmoother &s, int nsmooth, const double *b, double *x) {
        for (int k = 0; k < nsmooth; ++k) {
            for (int j = 0; j < nsmooth; ++j) s.apply_sparse(b, x);
            if (s.op->m() > 0) {
                // the low-rank part of SORSmoother::apply alone: x -= Bbar B^T x
                const int m = s.op->m();
                std::vector<double> y(m, 0.0);
                for (int jj = 0; jj < m; ++jj) {
                    double acc = 0.0;
                    for (int64_t e = s.op->B.ptr[jj]; e < s.op->B.ptr[jj + 1]; ++e) acc += s.op->B.val[e] * x[s.op->B.row[e]];
                    y[jj] = acc;
                }
                const double *Bb = s.Bbar->data();
                for (int64_t i = 0; i < s.op->n(); ++i) {
                    double acc = 0.0;
                    for (int jj = 0; jj < m; ++jj) acc += Bb[(size_t)i * m + jj] * y[jj];
                    x[i] -= acc;
                }
            }
        }
    }
    void smooth(int level, bool pre, const double *b, double *x) {
        const int ns = pre ? p.npresmooth : p.npostsmooth;
        if (p.smoother == 1) {  // SSORSmoother (ssor_smoother.cc:9-16)
            for (int k = 0; k < ns; ++k) {
                fwd[level]->apply(b, x);
                bwd[level]->apply(b, x);
            }
        } else {  // SOR: forward before, backward after the coarse correction
            sor_smooth(pre ? *fwd[level] : *bwd[level], ns, b, x);
        }
    }
    void solve(int level) {  // multigrid_preconditioner.cc:73-100
        std::fill(x_ell[level].begin(), x_ell[level].end(), 0.0);
        if (level == p.nlevel - 1) {
            if (woodbury) {
                coarse_w->apply(b_ell[level].data(), x_ell[level].data());
            } else {
                zeros.pos = 0;
                coarse_d->apply(b_ell[level].data(), x_ell[level].data());
            }
            return;
        }
        int cyc = (level > 0) ? p.cycle : 1;
        for (int j = 0; j < cyc; ++j) {
            smooth(level, true, b_ell[level].data(), x_ell[level].data());
            ops[level]->apply(x_ell[level].data(), r_ell[level].data());
            int64_t n = ops[level]->n();
            for (int64_t i = 0; i < n; ++i) r_ell[level][i] = b_ell[level][i] - r_ell[level][i];
            ig[level]->restrict_(r_ell[level].data(), b_ell[level + 1].data());
            solve(level + 1);
            ig[level]->prolongate_add(p.coarse_scaling, x_ell[level + 1].data(), x_ell[level].data());
            smooth(level, false, b_ell[level].data(), x_ell[level].data());
        }
    }
    void apply(const double *b, double *x) {  // :103-108
        std::copy(b, b + ops[0]->n(), b_ell[0].begin());
        solve(0);
        std::copy(x_ell[0].begin(), x_ell[0].end(), x);
    }
};

static double vec_norm(const std::vector<double> &v) {
    double s = 0.0;
    for (double a : v) s += a * a;
    return sqrt(s);
}

// LoopSolver::apply (loop_solver.cc:9-53); returns the iteration count at
// convergence, or maxiter.
static int loop_solve(const LinOp &op, MGPreconditioner &P, const double *b, double *x, double rtol, double atol,
                      int maxiter, double *rnorm, int *converged) {
    const int64_t n = op.n();
    double r0_nrm = vec_norm(std::vector<double>(b, b + n));
    std::fill(x, x + n, 0.0);
    std::vector<double> r(n), Pr(n);
    *converged = 0;
    *rnorm = -1.0;
    int k = 0;
    for (k = 0; k < maxiter; ++k) {
        op.apply(x, r.data());
        for (int64_t i = 0; i < n; ++i) r[i] -= b[i];
        const double r_nrm = vec_norm(r);
        *rnorm = r_nrm;
        if ((r_nrm / r0_nrm < rtol) && (r_nrm < atol)) {
            *converged = 1;
            break;
        }
        P.apply(r.data(), Pr.data());
        for (int64_t i = 0; i < n; ++i) x[i] -= Pr[i];
    }
    return k;
}

// ---------------------------------------------------------------------------
// Statistics: statistics.{hh,cc}
// ---------------------------------------------------------------------------
struct Statistics {
    int dim;
    unsigned k_max;
    unsigned n_samples = 0;
    std::vector<double> avg, avg2;
    std::deque<std::vector<double>> Q_k;
    std::vector<std::vector<double>> S_k;
    Statistics(int dim_, unsigned window) : dim(dim_), k_max(window) {}
    static std::vector<double> outer(const std::vector<double> &a, const std::vector<double> &b) {
        int d = (int)a.size();
        std::vector<double> r(d * d);
        for (int i = 0; i < d; ++i)
            for (int j = 0; j < d; ++j) r[i * d + j] = a[i] * b[j];
        return r;
    }
    void record(const std::vector<double> &Q) {  // statistics.cc:4-39
        n_samples++;
        if (n_samples == 1) {
            avg = Q;
            avg2 = outer(Q, Q);
        } else {
            auto QQ = outer(Q, Q);
            for (int i = 0; i < dim; ++i) avg[i] += (Q[i] - avg[i]) / (1.0 * n_samples);
            for (int i = 0; i < dim * dim; ++i) avg2[i] += (QQ[i] - avg2[i]) / (1.0 * n_samples);
        }
        Q_k.push_front(Q);
        if (Q_k.size() > k_max) Q_k.pop_back();
        for (unsigned k = 0; k < Q_k.size(); ++k) {
            unsigned N_k = n_samples - k;
            auto P = outer(Q_k[0], Q_k[k]);
            if (N_k == 1) {
                S_k.push_back(P);
            } else {
                for (int i = 0; i < dim * dim; ++i) S_k[k][i] += (P[i] - S_k[k][i]) / (1.0 * N_k);
            }
        }
    }
    std::vector<double> covariance() const {  // statistics.cc:42-45
        std::vector<double> c(dim * dim);
        for (int i = 0; i < dim; ++i)
            for (int j = 0; j < dim; ++j)
                c[i * dim + j] = 1.0 * n_samples / (n_samples - 1.0) * (avg2[i * dim + j] - avg[i] * avg[j]);
        return c;
    }
    std::vector<std::vector<double>> auto_covariance() const {  // :54-62
        std::vector<std::vector<double>> r;
        for (auto &S : S_k) {
            std::vector<double> c(dim * dim);
            for (int i = 0; i < dim; ++i)
                for (int j = 0; j < dim; ++j) c[i * dim + j] = S[i * dim + j] - avg[i] * avg[j];
            r.push_back(c);
        }
        return r;
    }
    double vCv(const std::vector<double> &C, const double *v) const {
        double s = 0.0;
        for (int i = 0; i < dim; ++i) {
            double t = 0.0;
            for (int j = 0; j < dim; ++j) t += C[i * dim + j] * v[j];
            s += v[i] * t;
        }
        return s;
    }
    double tau_int(const double *v) const {  // statistics.cc:65-79
        auto C = auto_covariance();
        double variance = vCv(C[0], v);
        double t = 1.0;
        unsigned kmax = (unsigned)C.size();
        for (unsigned k = 1; k < kmax; ++k) t += 2 * (1. - k / (1.0 * kmax)) * vCv(C[k], v) / variance;
        return t;
    }
};

}  // namespace orc

// ===========================================================================
// C interface used by the tests through ctypes.
// ===========================================================================
using namespace orc;

struct orc_op {
    std::shared_ptr<LinOp> op;
};
struct orc_sampler {
    std::unique_ptr<Sampler> s;
};
struct orc_stats {
    Statistics st;
};

extern "C" {

// ---- lattice known-answer helpers (lattice{1,2,3}d.hh) ----
int64_t orc_lattice_nvertex(int dim, int nx, int ny, int nz) { return Lattice(dim, nx, ny, nz).nvertex(); }
void orc_lattice_vertex_euclid(int dim, int nx, int ny, int nz, int64_t ell, int *idx) {
    int v[3];
    Lattice(dim, nx, ny, nz).vertex_euclid(ell, v);
    for (int d = 0; d < dim; ++d) idx[d] = v[d];
}
int64_t orc_lattice_vertex_linear(int dim, int nx, int ny, int nz, const int *idx) {
    int v[3] = {1, 1, 1};
    for (int d = 0; d < dim; ++d) v[d] = idx[d];
    return Lattice(dim, nx, ny, nz).vertex_linear(v);
}
// shift_vertexidx (lattice3d.hh:164-179): the linear index of the shifted
// Euclidean index; like the reference's release build it does not check
// that the shifted vertex is interior (its asserts are debug-only)
int64_t orc_lattice_shift_vertex(int dim, int nx, int ny, int nz, int64_t ell, const int *shift) {
    Lattice lat(dim, nx, ny, nz);
    int v[3];
    lat.vertex_euclid(ell, v);
    for (int d = 0; d < dim; ++d) v[d] += shift[d];
    return lat.vertex_linear(v);
}
void orc_lattice_cell_euclid(int dim, int nx, int ny, int nz, int64_t ell, int *idx) {
    int v[3];
    Lattice(dim, nx, ny, nz).cell_euclid(ell, v);
    for (int d = 0; d < dim; ++d) idx[d] = v[d];
}
int64_t orc_lattice_cell_linear(int dim, int nx, int ny, int nz, const int *idx) {
    Lattice lat(dim, nx, ny, nz);
    int64_t r = 0, s = 1;
    for (int d = 0; d < dim; ++d) {
        r += idx[d] * s;
        s *= lat.n[d];
    }
    return r;
}
int64_t orc_lattice_fine_vertex_idx(int dim, int nx, int ny, int nz, int64_t ell) {
    return Lattice(dim, nx, ny, nz).fine_vertex_idx(ell);
}
void orc_lattice_vertex_coordinates(int dim, int nx, int ny, int nz, int64_t ell, double *x) {
    double v[3];
    Lattice(dim, nx, ny, nz).vertex_coordinates(ell, v);
    for (int d = 0; d < dim; ++d) x[d] = v[d];
}

// ---- quadrature ----
int orc_quadrature(int dim, int order, double *weights, double *points) {
    Quadrature q(dim, order);
    for (size_t j = 0; j < q.weights.size(); ++j) {
        weights[j] = q.weights[j];
        for (int d = 0; d < dim; ++d) points[j * dim + d] = q.points[j][d];
    }
    return (int)q.weights.size();
}

// ---- operators ----
void orc_fd_stencil(int dim, int nx, int ny, int nz, double kappa_sq, double *st) {
    fd_stencil(Lattice(dim, nx, ny, nz), kappa_sq, st);
}
orc_op *orc_stencil_operator(int dim, int nx, int ny, int nz, const double *st) {
    return new orc_op{stencil_operator(Lattice(dim, nx, ny, nz), st)};
}
orc_op *orc_fem_operator(int dim, int nx, int ny, int nz, int model, double p0, double p1) {
    return new orc_op{fem_operator(Lattice(dim, nx, ny, nz), model, p0, p1)};
}
orc_op *orc_fd_operator(int dim, int nx, int ny, int nz, double kappa_sq) {
    Lattice lat(dim, nx, ny, nz);
    double st[27];
    fd_stencil(lat, kappa_sq, st);
    return new orc_op{stencil_operator(lat, st)};
}
void orc_op_destroy(orc_op *o) { delete o; }
int64_t orc_op_n(orc_op *o) { return o->op->n(); }
int orc_op_m(orc_op *o) { return o->op->m(); }
int64_t orc_op_nnz(orc_op *o) { return o->op->A.ptr[o->op->n()]; }
void orc_op_get_csr(orc_op *o, int64_t *ptr, int64_t *col, double *val) {
    const Csr &A = o->op->A;
    std::copy(A.ptr.begin(), A.ptr.end(), ptr);
    std::copy(A.col.begin(), A.col.end(), col);
    std::copy(A.val.begin(), A.val.end(), val);
}
int64_t orc_op_B_nnz(orc_op *o) { return o->op->B.ptr[o->op->m()]; }
void orc_op_get_B(orc_op *o, int64_t *ptr, int64_t *row, double *val, double *Sigma) {
    const Csc &B = o->op->B;
    std::copy(B.ptr.begin(), B.ptr.end(), ptr);
    std::copy(B.row.begin(), B.row.end(), row);
    std::copy(B.val.begin(), B.val.end(), val);
    std::copy(o->op->Sigma.begin(), o->op->Sigma.end(), Sigma);
}
// Attach an explicit low-rank term B (CSC, rows ascending) and Sigma.
void orc_op_set_lowrank(orc_op *o, int m, const int64_t *ptr, const int64_t *row, const double *val, const double *Sigma) {
    Csc &B = o->op->B;
    B.nrow = o->op->n();
    B.m = m;
    B.ptr.assign(ptr, ptr + m + 1);
    B.row.assign(row, row + ptr[m]);
    B.val.assign(val, val + ptr[m]);
    o->op->Sigma.assign(Sigma, Sigma + m);
}
// Per-vertex diagonal (the FD prior with a variable correlation length,
// shiftedlaplace_fd_operator.cc:33-52): the diagonal entry of every row of
// A_0 is replaced by diag[row].
void orc_op_set_diagonal(orc_op *o, const double *diag) {
    Csr &A = o->op->A;
    for (int64_t i = 0; i < A.n; ++i)
        for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k)
            if (A.col[k] == i) A.val[k] = diag[i];
    A.finish_diag();
}
// MeasuredOperator (measured_operator.cc:9-47): locations[k*dim+d],
// Sigma_kk = variance_scaling * variance[k]; optional global mean column.
void orc_op_add_measurements(orc_op *o, int n_meas, const double *locations, const double *variance,
                             double variance_scaling, double radius, int measure_global, double variance_global) {
    LinOp &op = *o->op;
    int dim = op.lat.dim;
    int m = n_meas + (measure_global ? 1 : 0);
    Csc &B = op.B;
    B.nrow = op.n();
    B.m = m;
    B.ptr.assign(1, 0);
    B.row.clear();
    B.val.clear();
    op.Sigma.assign(m, 0.0);
    for (int k = 0; k < n_meas; ++k) {
        auto r = measurement_vector(op.lat, locations + k * dim, radius);
        for (auto &e : r) {
            B.row.push_back(e.first);
            B.val.push_back(e.second);
        }
        B.ptr.push_back((int64_t)B.row.size());
        op.Sigma[k] = variance_scaling * variance[k];
    }
    if (measure_global) {
        double cv = 1.0;
        for (int d = 0; d < dim; ++d) cv /= double(op.lat.n[d]);
        for (int64_t ell = 0; ell < op.n(); ++ell) {
            B.row.push_back(ell);
            B.val.push_back(cv);
        }
        B.ptr.push_back((int64_t)B.row.size());
        op.Sigma[n_meas] = variance_global;
    }
}
int64_t orc_measurement_vector(int dim, int nx, int ny, int nz, const double *x0, double radius, int64_t *idx,
                               double *val, int64_t cap) {
    auto r = measurement_vector(Lattice(dim, nx, ny, nz), x0, radius);
    int64_t k = 0;
    for (auto &e : r) {
        if (k < cap) {
            idx[k] = e.first;
            val[k] = e.second;
        }
        ++k;
    }
    return k;
}
void orc_op_apply(orc_op *o, const double *x, double *y) { o->op->apply(x, y); }
void orc_op_precision(orc_op *o, double *Q) {
    auto P = o->op->precision_dense();
    std::copy(P.begin(), P.end(), Q);
}
orc_op *orc_op_coarsen(orc_op *o) {
    Intergrid ig(o->op->lat);
    return new orc_op{coarsen(*o->op, ig)};
}
int orc_op_coarsenable(orc_op *o) { return o->op->lat.coarsenable() ? 1 : 0; }

// ---- intergrid ----
void orc_restrict(int dim, int nx, int ny, int nz, const double *x, double *xc) {
    Intergrid(Lattice(dim, nx, ny, nz)).restrict_(x, xc);
}
void orc_prolongate_add(int dim, int nx, int ny, int nz, double alpha, const double *xc, double *x) {
    Intergrid(Lattice(dim, nx, ny, nz)).prolongate_add(alpha, xc, x);
}

// ---- random numbers ----
CLCG *orc_rng_create(int n_threads, int thread_id) { return new CLCG(n_threads, thread_id); }
void orc_rng_destroy(CLCG *r) { delete r; }
void orc_rng_draw_int(CLCG *r, int64_t n, int32_t *out) {
    for (int64_t i = 0; i < n; ++i) out[i] = r->draw_int();
}
void orc_rng_draw_uniform(CLCG *r, int64_t n, double *out) {
    for (int64_t i = 0; i < n; ++i) out[i] = r->draw_uniform_real();
}
void orc_rng_draw_normal(CLCG *r, int64_t n, double *out) {
    for (int64_t i = 0; i < n; ++i) out[i] = r->draw_normal();
}
// noise sources: kind 0 = CLCG (seed fixed at 1 as in the reference),
// kind 1 = injected buffer
NormalSource *orc_source_clcg() { return new CLCG(1, 0); }
NormalSource *orc_source_buffer(const double *data, int64_t n) {
    auto *b = new BufferSource();
    b->data.assign(data, data + n);
    return b;
}
int64_t orc_source_position(NormalSource *s) {
    auto *b = dynamic_cast<BufferSource *>(s);
    return b ? (int64_t)b->pos : -1;
}
void orc_source_destroy(NormalSource *s) { delete s; }

// ---- samplers ----
orc_sampler *orc_sor_sampler(orc_op *o, NormalSource *src, double omega, int nsmooth, int forward, int ordering) {
    return new orc_sampler{std::unique_ptr<Sampler>(new SORSampler(o->op, src, omega, nsmooth, forward != 0, ordering))};
}
orc_sampler *orc_ssor_sampler(orc_op *o, NormalSource *src, double omega, int nsmooth, int ordering) {
    return new orc_sampler{std::unique_ptr<Sampler>(new SSORSampler(o->op, src, omega, nsmooth, ordering))};
}
orc_sampler *orc_cholesky_sampler(orc_op *o, NormalSource *src) {
    auto *c = new CholeskySampler(o->op, src);
    if (!c->ok) {
        delete c;
        return nullptr;
    }
    return new orc_sampler{std::unique_ptr<Sampler>(c)};
}
orc_sampler *orc_lowrank_cholesky_sampler(orc_op *o, NormalSource *src) {
    auto *c = new LowRankCholeskySampler(o->op, src);
    if (!c->ok) {
        delete c;
        return nullptr;
    }
    return new orc_sampler{std::unique_ptr<Sampler>(c)};
}
orc_sampler *orc_mgmc_sampler(orc_op *o, NormalSource *src, int nlevel, int smoother, int coarse_solver, int npresmooth,
                              int npostsmooth, int ncoarsesmooth, double omega, int cycle, double coarse_scaling,
                              int ordering) {
    MGParams p{nlevel, smoother, coarse_solver, npresmooth, npostsmooth, ncoarsesmooth, omega, cycle, coarse_scaling, ordering};
    try {
        return new orc_sampler{std::unique_ptr<Sampler>(new MGMCSampler(o->op, src, p))};
    } catch (...) {
        return nullptr;
    }
}
void orc_sampler_destroy(orc_sampler *s) { delete s; }
int orc_sampler_apply(orc_sampler *s, const double *f, double *x, int nsteps) {
    try {
        for (int k = 0; k < nsteps; ++k) s->s->apply(f, x);
    } catch (...) {
        return 1;
    }
    return 0;
}
// nsteps applications; after each the observable obs[k] = b^T x (sparse b)
int orc_sampler_observe(orc_sampler *s, const double *f, double *x, int64_t nsteps, int64_t nb, const int64_t *bidx,
                        const double *bval, double *obs) {
    try {
        for (int64_t k = 0; k < nsteps; ++k) {
            s->s->apply(f, x);
            double z = 0.0;
            for (int64_t e = 0; e < nb; ++e) z += bval[e] * x[bidx[e]];
            obs[k] = z;
        }
    } catch (...) {
        return 1;
    }
    return 0;
}
// Mean and (maximum-likelihood) covariance after nwarmup steps, as in
// test_sampler.hh:113-153.
int orc_sampler_mean_cov(orc_sampler *s, int64_t n, const double *f, double *x, int64_t nwarmup, int64_t nsamples,
                         double *Ex, double *Exx) {
    try {
        for (int64_t k = 0; k < nwarmup; ++k) s->s->apply(f, x);
        std::fill(Ex, Ex + n, 0.0);
        std::fill(Exx, Exx + n * n, 0.0);
        for (int64_t k = 0; k < nsamples; ++k) {
            s->s->apply(f, x);
            double w = 1. / double(k + 1);
            for (int64_t i = 0; i < n; ++i) Ex[i] += w * (x[i] - Ex[i]);
            for (int64_t i = 0; i < n; ++i)
                for (int64_t j = 0; j < n; ++j) Exx[i * n + j] += w * (x[i] * x[j] - Exx[i * n + j]);
        }
        for (int64_t i = 0; i < n; ++i)
            for (int64_t j = 0; j < n; ++j) Exx[i * n + j] -= Ex[i] * Ex[j];
    } catch (...) {
        return 1;
    }
    return 0;
}
// deterministic SSOR smoother (ssor_smoother.cc:9-16) with nsmooth passes
void orc_ssor_smoother_apply(orc_op *o, double omega, int nsmooth, int ordering, const double *b, double *x) {
    SORSmoother f(o->op, omega, true, ordering), bw(o->op, omega, false, ordering);
    for (int k = 0; k < nsmooth; ++k) {
        f.apply(b, x);
        bw.apply(b, x);
    }
}
// dense natural-order Cholesky; returns 0 on success, 1 if not SPD
int orc_dense_cholesky(double *A, int64_t n) {
    std::vector<double> M(A, A + n * n);
    if (!dense_cholesky(M, n)) return 1;
    std::copy(M.begin(), M.end(), A);
    return 0;
}

// ---- deterministic solvers ----
struct orc_mg {
    std::unique_ptr<MGPreconditioner> P;
    std::shared_ptr<LinOp> op;
};
orc_mg *orc_mg_create(orc_op *o, int nlevel, int smoother, int npresmooth, int npostsmooth, double omega, int cycle,
                      double coarse_scaling, int ordering, int woodbury) {
    MGParams p{nlevel, smoother, 0, npresmooth, npostsmooth, 1, omega, cycle, coarse_scaling, ordering};
    try {
        auto *h = new orc_mg{std::unique_ptr<MGPreconditioner>(new MGPreconditioner(o->op, p, woodbury != 0)), o->op};
        if (!h->P->ok) {
            delete h;
            return nullptr;
        }
        return h;
    } catch (...) {
        return nullptr;
    }
}
void orc_mg_destroy(orc_mg *h) { delete h; }
void orc_mg_apply(orc_mg *h, const double *b, double *x) { h->P->apply(b, x); }
int orc_loop_solve(orc_mg *h, const double *b, double *x, double rtol, double atol, int maxiter, double *rnorm,
                   int *converged) {
    return loop_solve(*h->op, *h->P, b, x, rtol, atol, maxiter, rnorm, converged);
}
// CholeskySolver::apply (Woodbury); returns 1 if A_0 is not SPD
int orc_cholesky_solve(orc_op *o, const double *b, double *x) {
    CholeskySolver s(o->op);
    if (!s.ok) return 1;
    s.apply(b, x);
    return 0;
}

// ---- statistics ----
orc_stats *orc_stats_create(int dim, unsigned window) { return new orc_stats{Statistics(dim, window)}; }
void orc_stats_destroy(orc_stats *s) { delete s; }
void orc_stats_record(orc_stats *s, const double *Q, int64_t nsamples) {
    int d = s->st.dim;
    for (int64_t k = 0; k < nsamples; ++k) s->st.record(std::vector<double>(Q + k * d, Q + (k + 1) * d));
}
void orc_stats_average(orc_stats *s, double *out) { std::copy(s->st.avg.begin(), s->st.avg.end(), out); }
void orc_stats_covariance(orc_stats *s, double *out) {
    auto c = s->st.covariance();
    std::copy(c.begin(), c.end(), out);
}
int orc_stats_autocov(orc_stats *s, double *out) {
    auto c = s->st.auto_covariance();
    int d = s->st.dim;
    for (size_t k = 0; k < c.size(); ++k) std::copy(c[k].begin(), c[k].end(), out + k * d * d);
    return (int)c.size();
}
double orc_stats_tau_int(orc_stats *s, const double *v) { return s->st.tau_int(v); }

}  // extern "C"
