// Stand-in for Lattice (src/lattice/lattice.hh): shape() only.
#pragma once
#include <Eigen/Dense>
class Lattice {
public:
    explicit Lattice(Eigen::VectorXi shape) : shape_(shape) {}
    virtual ~Lattice() = default;
    virtual Eigen::VectorXi shape() const { return shape_; }

private:
    Eigen::VectorXi shape_;
};
