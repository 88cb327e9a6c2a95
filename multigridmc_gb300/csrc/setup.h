// setup.h -- host-side set-up of the multigrid hierarchy (no CUDA).
//
// Everything here runs once per sampler: the fine stencil, the Galerkin
// coarse stencils, the measurement matrix B on every level, and the dense
// FP64 factor of the coarse precision matrix.  The per-step work lives in
// kernels.cu.
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <vector>

namespace mgmc {

// Lattice geometry of one level plus its padded device layout.
//
// Interior vertices (i, j, k), 1 <= i <= c[0]-1 etc., are stored at
//   p = k * sz + j * sy + i,   sy = c[0], sz = c[0] * c[1].
// Index 0 of every row is a ghost that is also the right-hand ghost of the
// previous row, row 0 of every plane is a ghost that is also the top ghost
// row of the previous plane, and planes 0 and c[2] are ghost planes; one
// extra ghost plane absorbs the diagonal offsets of the last interior
// plane.  Ghosts hold zero (homogeneous Dirichlet) and are never written.
// Inactive directions of 1d/2d lattices have c = 2, i.e. one interior layer.
struct Geometry {
    int dim = 3;
    int c[3] = {2, 2, 2};  // cells per direction
    int N[3] = {1, 1, 1};  // interior vertices per direction
    int64_t n = 0;         // interior vertices
    int64_t sy = 0, sz = 0, nalloc = 0;

    Geometry() = default;
    Geometry(int dim_, int nx, int ny, int nz);
    bool coarsenable() const;
    Geometry coarse() const;
    // compact (reference) index -> padded index
    int64_t pad(int64_t ell) const {
        int64_t nxy = (int64_t)N[0] * N[1];
        int64_t i = (ell % nxy) % N[0] + 1, j = (ell % nxy) / N[0] + 1, k = ell / nxy + 1;
        return k * sz + j * sy + i;
    }
    double cell_volume() const;
};

// Column-compressed n x m matrix (row indices ascending in each column).
struct SparseCols {
    int m = 0;
    std::vector<int64_t> ptr{0};
    std::vector<int64_t> row;
    std::vector<double> val;
};

void fd_stencil(const Geometry &g, double kappa_sq, double st[27]);
void galerkin_stencil(int dim, const double fine[27], double coarse[27]);
// 2 if the stencil couples axis neighbours only, otherwise 2^dim
int colour_count(int dim, const double st[27]);
std::map<int64_t, double> measurement_vector(const Geometry &g, const double *x0, double radius);
// B_c = R B with the linear restriction (weights prod {1/2, 1, 1/2})
SparseCols restrict_columns(const Geometry &fine, const SparseCols &B);
// dense row-major precision matrix A_0 + B Sigma^{-1} B^T of one level
std::vector<double> dense_precision(const Geometry &g, const double st[27], const SparseCols &B,
                                    const std::vector<double> &Sigma);
// Galerkin product R A R^T (linear_operator.cc:10-23) of a per-point stencil
// field: A's weight k at fine point f (compact index) is full[k * n + f] when
// `full` is given, else the constant stencil[k] with the centre replaced by
// centre[f].  Returns the coarse field, weight-major (k * n_c + p_c);
// neighbours outside the lattice are omitted (Dirichlet), as in the sparse
// triple product.
std::vector<double> galerkin_field(const Geometry &fine, const double stencil[27], const double *centre,
                                   const double *full);
// ShiftedLaplaceFEMOperator (shiftedlaplace_fem_operator.cc:9-152): Q1
// elements, the 2-point Gauss-Legendre rule per direction, local entries
// (kappa^2(x_q) phi_a phi_b + sum_d h_d^{-2} dphi_a dphi_b) w_q times the
// cell volume, between interior vertices only.  kappa^2 is constant
// (model 0, p0 = kappa^2) or periodic (model 1, correlationlength_model.hh:
// 83-112, p0 = Lambda_min, p1 = Lambda_max).  Returns the weight-major
// per-point field (27 x n; inactive directions keep zero weights).
std::vector<double> fem_field(const Geometry &g, int model, double p0, double p1);
// dense row-major A_0 + B Sigma^{-1} B^T of a level with a weight-major
// per-point stencil field (27 x n)
std::vector<double> dense_precision_field(const Geometry &g, const std::vector<double> &field, const SparseCols &B,
                                          const std::vector<double> &Sigma);
// natural-order Cholesky Q = L L^T in place (lower triangle, zeros above);
// false if a pivot is not positive
bool dense_cholesky(std::vector<double> &Q, int64_t n);
// L^{-1} of a lower-triangular row-major factor; returns (L^{-1})^T row-major
std::vector<double> inverse_factor_transposed(const std::vector<double> &L, int64_t n);
// Phi(L^{-1} E L^{-T}) for the constant-stencil matrix E on geometry g
// (Dirichlet: neighbours outside omitted), from T = (L^{-1})^T row-major:
// the strict lower part and half the diagonal, row-major n x n, zeros
// above the diagonal (the derivative of the Cholesky factor in direction E
// is L Phi(L^{-1} E L^{-T}))
std::vector<double> cholesky_phi_sandwich(const std::vector<double> &T, const Geometry &g, const double E[27]);
// L^{-1} B from T = (L^{-1})^T: column k (n values) stored at k * n
std::vector<double> inverse_factor_times(const std::vector<double> &T, int64_t n, const SparseCols &B);
// inverse of a small dense matrix by LU with partial pivoting
std::vector<double> small_inverse(const std::vector<double> &S, int m);

// LowRankCholeskySampler (cholesky_sampler.cc:41-96) set-up.  A_0 (constant
// stencil, Dirichlet) is block tridiagonal in the vertex order, with blocks
// of p = n / nb vertices along the last lattice direction (planes in 3D, rows
// in 2D, single vertices in 1D), so its Cholesky factor L has diagonal
// blocks L_kk and sub-diagonal blocks L_{k,k-1}:
//   S_0 = A_00,  L_kk L_kk^T = S_k,  L_{k+1,k} = A_{k+1,k} L_kk^{-T},
//   S_{k+1} = A_{k+1,k+1} - L_{k+1,k} L_{k+1,k}^T.
// D holds the blocks L_kk^{-1} and O the blocks L_{k,k-1} (block 0 zero),
// row-major p x p each.  With measurements, V = L^{-1} B has the thin QR
// V = Q R (R with a positive diagonal), W is the lower Cholesky factor of
// Id - R (Sigma + V^T V)^{-1} R^T, and QW = Q (W^T - Id), QWT = Q (W - Id),
// n x m row-major.
struct LowRankCholeskyFactors {
    int nb = 0, m = 0;
    int64_t p = 0;
    std::vector<double> D, O, Q, QW, QWT;
};
// false if A_0 or Id - Lambda is not positive definite
bool lowrank_cholesky_factors(const Geometry &g, const double st[27], const SparseCols &B,
                              const std::vector<double> &Sigma, LowRankCholeskyFactors &F);

}  // namespace mgmc
