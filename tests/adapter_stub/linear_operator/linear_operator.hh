// Stand-in for LinearOperator (src/linear_operator/linear_operator.hh): the
// accessors the adapter reads (lattice, B, Sigma).
#pragma once
#include <memory>
#include <Eigen/Dense>
#include <Eigen/Sparse>
#include "lattice/lattice.hh"
class LinearOperator {
public:
    typedef Eigen::SparseMatrix<double> SparseMatrixType;
    LinearOperator(std::shared_ptr<Lattice> lattice, SparseMatrixType B, Eigen::VectorXd Sigma)
        : lattice_(lattice), B_(std::move(B)), Sigma_(Sigma) {}
    std::shared_ptr<Lattice> get_lattice() const { return lattice_; }
    const SparseMatrixType &get_B() const { return B_; }
    const Eigen::DiagonalMatrix<double, Eigen::Dynamic> get_Sigma() const {
        return Eigen::DiagonalMatrix<double, Eigen::Dynamic>(Sigma_);
    }

private:
    std::shared_ptr<Lattice> lattice_;
    SparseMatrixType B_;
    Eigen::VectorXd Sigma_;
};
