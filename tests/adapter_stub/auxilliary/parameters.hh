// Stand-in for MultigridParameters (src/auxilliary/parameters.hh:150-179):
// the fields, without the libconfig parser.
#pragma once
#include <string>
struct MultigridParameters {
    unsigned int nlevel = 3;
    std::string smoother = "SSOR";
    std::string coarse_solver = "Cholesky";
    unsigned int npresmooth = 1;
    unsigned int npostsmooth = 1;
    unsigned int ncoarsesmooth = 1;
    double omega = 1.0;
    unsigned int cycle = 1;
    double coarse_scaling = 1.0;
    int verbose = 0;
};
