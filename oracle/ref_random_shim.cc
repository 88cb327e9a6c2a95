// Test infrastructure only: a C ABI over the reference's own random number
// generator (CLCGenerator of src/auxilliary/parallel_random.{hh,cc},
// compiled from the reference sources by oracle/build_ref.py into
// oracle/_ref/), so that the oracle's restatement of it can be compared draw
// by draw.  Nothing in the product links this.
#include <cstdint>
#include <omp.h>

#include "parallel_random.hh"

extern "C" {

void *ref_clcg_create() { return new CLCGenerator(); }

void ref_clcg_destroy(void *g) { delete static_cast<CLCGenerator *>(g); }

void ref_clcg_draw_int(void *g, int64_t n, int32_t *out) {
    CLCGenerator *r = static_cast<CLCGenerator *>(g);
    for (int64_t i = 0; i < n; ++i) out[i] = r->draw_int();
}

void ref_clcg_draw_uniform(void *g, int64_t n, double *out) {
    CLCGenerator *r = static_cast<CLCGenerator *>(g);
    for (int64_t i = 0; i < n; ++i) out[i] = r->draw_uniform_real();
}

void ref_clcg_draw_normal(void *g, int64_t n, double *out) {
    CLCGenerator *r = static_cast<CLCGenerator *>(g);
    for (int64_t i = 0; i < n; ++i) out[i] = r->draw_normal();
}

// Leapfrog streams: the generator constructed inside an OpenMP team of
// nthreads threads; thread t writes its n integer draws to out[t * n ...].
// Returns the team size actually obtained.
int ref_clcg_leapfrog_ints(int nthreads, int64_t n, int32_t *out) {
    int got = 0;
#pragma omp parallel num_threads(nthreads)
    {
        CLCGenerator r;
        const int t = omp_get_thread_num();
        if (t == 0) got = omp_get_num_threads();
        for (int64_t i = 0; i < n; ++i) out[t * n + i] = r.draw_int();
    }
    return got;
}
}
