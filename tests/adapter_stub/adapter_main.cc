// Drives include/mgmc_gb300_sampler.hh (the reference-side adapter) the way
// measure_sampling_time does (sampling_time.cc:28-41): fix_rhs, then
// apply(f, x) per step; then one apply after unfix_rhs, the device-resident
// observable loop and a deep copy.  Writes every result to argv[1] (raw
// doubles) for tests/test_adapter.py, which replays the same calls through
// the Python binding.  Exit status: 0 ok, 2 usage, 3 library error.
#include <cstdio>
#include <exception>
#include <vector>

#include "mgmc_gb300_sampler.hh"

namespace {

struct FixedRandom : RandomGenerator {
    explicit FixedRandom(double u) : u(u) {}
    double draw_uniform_real() override { return u; }
    double u;
};

}  // namespace

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    try {
        const int N = 16, m = 4;
        const int64_t n = (int64_t)(N - 1) * (N - 1) * (N - 1);
        double st[27];
        if (mgmc_fd_stencil(3, N, N, N, 10.0, st) != MGMC_OK) return 3;
        const double centres[m][3] = {{0.3, 0.3, 0.3}, {0.6, 0.4, 0.5}, {0.4, 0.7, 0.6}, {0.7, 0.6, 0.3}};
        std::vector<int> outer{0}, inner;
        std::vector<double> val;
        for (int k = 0; k < m; ++k) {
            int64_t nnz = 0;
            if (mgmc_measurement_vector(3, N, N, N, centres[k], 0.1, nullptr, nullptr, 0, &nnz) != MGMC_OK) return 3;
            std::vector<int64_t> idx((size_t)nnz);
            std::vector<double> v((size_t)nnz);
            if (mgmc_measurement_vector(3, N, N, N, centres[k], 0.1, idx.data(), v.data(), nnz, &nnz) != MGMC_OK)
                return 3;
            for (int64_t e = 0; e < nnz; ++e) {
                inner.push_back((int)idx[(size_t)e]);
                val.push_back(v[(size_t)e]);
            }
            outer.push_back((int)inner.size());
        }
        Eigen::VectorXd Sigma(m);
        for (int k = 0; k < m; ++k) Sigma[k] = 1e-4;
        LinearOperator::SparseMatrixType B(n, m, outer, inner, val);
        auto op = std::make_shared<LinearOperator>(std::make_shared<Lattice>(Eigen::VectorXi{N, N, N}), B, Sigma);
        // f = B Sigma^-1 y
        const double y[m] = {1.0, -0.5, 0.25, 2.0};
        Eigen::VectorXd f(n), x(n);
        f.setZero();
        x.setZero();
        for (int k = 0; k < m; ++k)
            for (int e = outer[k]; e < outer[k + 1]; ++e) f[inner[e]] += val[e] * (y[k] / Sigma[k]);
        MultigridParameters p;
        p.nlevel = 3;
        std::vector<double> stencil(st, st + 27);
        GpuMultigridMCSampler s(op, std::make_shared<FixedRandom>(0.25), p, stencil, MGMC_FP64);
        FILE *out = std::fopen(argv[1], "wb");
        if (!out) return 2;
        s.fix_rhs(f);
        for (int k = 0; k < 5; ++k) s.apply(f, x);
        std::fwrite(x.data(), sizeof(double), (size_t)n, out);
        s.unfix_rhs();
        s.apply(f, x);
        std::fwrite(x.data(), sizeof(double), (size_t)n, out);
        // device-resident loop: observable b = column 0 of B
        Eigen::SparseVector<double> b(std::vector<int>(inner.begin(), inner.begin() + outer[1]),
                                      std::vector<double>(val.begin(), val.begin() + outer[1]));
        s.fix_rhs(f);
        s.set_observable(b, 8);
        s.step(3);
        std::vector<double> z = s.read_observations(8);
        const double nz = (double)z.size();
        std::fwrite(&nz, sizeof(double), 1, out);
        std::fwrite(z.data(), sizeof(double), z.size(), out);
        // Sampler::deep_copy with another generator
        auto c = s.deep_copy(std::make_shared<FixedRandom>(0.5));
        Eigen::VectorXd x2(n);
        x2.setZero();
        c->fix_rhs(f);
        c->apply(f, x2);
        std::fwrite(x2.data(), sizeof(double), (size_t)n, out);
        std::fclose(out);
    } catch (const std::exception &e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 3;
    }
    return 0;
}
