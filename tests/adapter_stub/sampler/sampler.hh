// Stand-in for Sampler (src/sampler/sampler.hh:23-78): the same virtual
// interface and protected members.
#pragma once
#include <memory>
#include <Eigen/Dense>
#include "auxilliary/parallel_random.hh"
#include "linear_operator/linear_operator.hh"
class Sampler {
public:
    Sampler(const std::shared_ptr<LinearOperator> linear_operator_, std::shared_ptr<RandomGenerator> rng_)
        : linear_operator(linear_operator_), rng(rng_) {}
    virtual ~Sampler() = default;
    virtual std::shared_ptr<Sampler> deep_copy(std::shared_ptr<RandomGenerator> rng) = 0;
    virtual void apply(const Eigen::VectorXd &f, Eigen::VectorXd &x) const = 0;
    std::shared_ptr<LinearOperator> get_linear_operator() const { return linear_operator; }
    virtual void fix_rhs(const Eigen::VectorXd &f) {}
    virtual void unfix_rhs() {}

protected:
    const std::shared_ptr<LinearOperator> linear_operator;
    std::shared_ptr<RandomGenerator> rng;
};
