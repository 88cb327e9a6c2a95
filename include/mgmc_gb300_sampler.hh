// mgmc_gb300_sampler.hh -- drop-in GPU MultigridMCSampler for the reference's
// driver (C++ side of the boundary; header-only over include/mgmc_gb300.h).
//
// Include it from the reference's source tree (it uses the reference's
// Sampler, LinearOperator, RandomGenerator and MultigridParameters headers
// and Eigen) and link libmgmc_gb300.so.  In driver_mgmc.cc:165-168 replace
//   std::make_shared<MultigridMCSampler>(linear_operator, rng, multigrid_params, cholesky_params)
// by
//   std::make_shared<GpuMultigridMCSampler>(linear_operator, rng, multigrid_params, stencil)
// with `stencil` from mgmc_fd_stencil (FD prior) or the FEM stencil.
//
// Surface kept from the reference (src/sampler/sampler.hh:23-78):
//   apply(f, x)      Sampler::apply -- one MGMC step; after fix_rhs only x
//                    crosses the host link (mgmc_sampler_apply with f = NULL)
//   fix_rhs(f)       Sampler::fix_rhs -- f uploaded once
//   unfix_rhs()      Sampler::unfix_rhs -- apply sends its f again
//   deep_copy(rng)   Sampler::deep_copy -- own device state, key from rng
// and, beyond it, the device-resident loop of measure_sampling_time
// (src/measurements/sampling_time.cc:28-41): set_observable(b, capacity),
// step(n) and read_observations() keep x on the GPU and return b^T x per step.
#ifndef MGMC_GB300_SAMPLER_HH
#define MGMC_GB300_SAMPLER_HH

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "mgmc_gb300.h"

#include <Eigen/Dense>
#include <Eigen/Sparse>
#include "auxilliary/parallel_random.hh"
#include "auxilliary/parameters.hh"
#include "linear_operator/linear_operator.hh"
#include "sampler/sampler.hh"

class GpuMultigridMCSampler : public Sampler {
public:
    GpuMultigridMCSampler(std::shared_ptr<LinearOperator> op, std::shared_ptr<RandomGenerator> rng,
                          const MultigridParameters &p, const std::vector<double> &stencil27,
                          int precision = MGMC_FP32_MIXED)
        : Sampler(op, rng), params(p), stencil(stencil27), precision(precision) {
        const LinearOperator::SparseMatrixType &B = op->get_B();  // column-major CSC
        std::vector<int64_t> colptr(B.outerIndexPtr(), B.outerIndexPtr() + B.cols() + 1);
        std::vector<int64_t> rowidx(B.innerIndexPtr(), B.innerIndexPtr() + B.nonZeros());
        Eigen::VectorXd sigma = op->get_Sigma().diagonal();
        Eigen::VectorXi shape = op->get_lattice()->shape();
        if (stencil.size() != 27) throw std::invalid_argument("GpuMultigridMCSampler: stencil needs 27 weights");
        mgmc_operator_desc d{};
        d.dim = (int)shape.size();
        d.nx = shape[0];
        d.ny = d.dim > 1 ? shape[1] : 2;
        d.nz = d.dim > 2 ? shape[2] : 2;
        for (int k = 0; k < 27; ++k) d.stencil[k] = stencil[k];
        d.m = (int)B.cols();
        d.B_colptr = colptr.data();
        d.B_rowidx = rowidx.data();
        d.B_val = B.valuePtr();
        d.Sigma = sigma.data();
        mgmc_sampler_params q{};
        q.nlevel = (int)p.nlevel;
        q.smoother = p.smoother == "SSOR" ? MGMC_SMOOTHER_SSOR : MGMC_SMOOTHER_SOR;
        q.coarse_solver = p.coarse_solver == "Cholesky" ? MGMC_COARSE_CHOLESKY : MGMC_COARSE_SSOR;
        q.npresmooth = (int)p.npresmooth;
        q.npostsmooth = (int)p.npostsmooth;
        q.ncoarsesmooth = (int)p.ncoarsesmooth;
        q.omega = p.omega;
        q.cycle = (int)p.cycle;
        q.coarse_scaling = p.coarse_scaling;
        q.ordering = MGMC_ORDER_MULTICOLOUR;
        q.precision = precision;
        q.noise = MGMC_NOISE_PHILOX;
        // the Philox key: 53 random bits of the caller's generator, so that
        // deep copies with their own generators draw independent streams
        q.seed = (uint64_t)(rng->draw_uniform_real() * 9007199254740992.0);
        q.device = 0;
        check(mgmc_sampler_create(&d, &q, &h));
    }
    ~GpuMultigridMCSampler() override { mgmc_sampler_destroy(h); }
    GpuMultigridMCSampler(const GpuMultigridMCSampler &) = delete;
    GpuMultigridMCSampler &operator=(const GpuMultigridMCSampler &) = delete;

    std::shared_ptr<Sampler> deep_copy(std::shared_ptr<RandomGenerator> rng) override {
        return std::make_shared<GpuMultigridMCSampler>(linear_operator, rng, params, stencil, precision);
    }

    // x <- one MGMC step; with the right hand side fixed only x travels
    void apply(const Eigen::VectorXd &f, Eigen::VectorXd &x) const override {
        check(mgmc_sampler_apply(h, rhs_fixed ? nullptr : f.data(), x.data(), 0));
    }

    void fix_rhs(const Eigen::VectorXd &f) override {
        check(mgmc_sampler_fix_rhs(h, f.data(), 0));
        rhs_fixed = true;
    }

    void unfix_rhs() override { rhs_fixed = false; }

    // ---- device-resident sampling loop (no counterpart in the reference)
    // observable z = b^T x recorded after every step, up to `capacity` values
    void set_observable(const Eigen::SparseVector<double> &b, int64_t capacity) {
        std::vector<int64_t> idx(b.innerIndexPtr(), b.innerIndexPtr() + b.nonZeros());
        check(mgmc_sampler_set_observable(h, (int64_t)idx.size(), idx.data(), b.valuePtr(), capacity));
    }
    void set_state(const Eigen::VectorXd &x) { check(mgmc_sampler_set_state(h, x.data(), 0)); }
    void get_state(Eigen::VectorXd &x) const { check(mgmc_sampler_get_state(h, x.data(), 0)); }
    // n steps with the fixed right hand side, x staying on the GPU
    void step(int64_t n) { check(mgmc_sampler_step(h, n)); }
    // the observations recorded since the last read
    std::vector<double> read_observations(int64_t capacity) const {
        std::vector<double> z((size_t)capacity);
        int64_t count = 0;
        check(mgmc_sampler_read_observations(h, z.data(), capacity, &count));
        z.resize((size_t)(count < capacity ? count : capacity));
        return z;
    }

private:
    static void check(mgmc_status s) {
        if (s != MGMC_OK) throw std::runtime_error(std::string("libmgmc_gb300: ") + mgmc_last_error());
    }
    MultigridParameters params;
    std::vector<double> stencil;
    int precision;
    bool rhs_fixed = false;
    mgmc_sampler *h = nullptr;
};

#endif  // MGMC_GB300_SAMPLER_HH
