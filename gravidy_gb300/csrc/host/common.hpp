// Constants and plain data types of the host side, with the reference's
// names and values (src/include/common.hpp:82-129, :171-329).
#ifndef GRAVIDY_GB300_HOST_COMMON_HPP
#define GRAVIDY_GB300_HOST_COMMON_HPP

#include <string>

#include "gravidy_gb300.h"

namespace gb300 {

const int G = 1;                                  // common.hpp:82
const double E = 1e-4;                            // default softening, common.hpp:107
const float ETA_S = 0.01f;                        // initial timestep eta, common.hpp:114
const float ETA_N = 0.01f;                        // default -e, common.hpp:119
const double D_TIME_MIN = 1.1920928955078125e-07; // 2^-23, common.hpp:122
const double D_TIME_MAX = 0.125;                  // 2^-3, common.hpp:129
// Flops per interaction of the log's GFLOPS column (common.hpp:331).
const double KERNEL_GFLOP = 48e-9;

typedef h4_double4 double4;
typedef h4_double3 double3;
typedef h4_forces Forces;

// Energy bookkeeping of the log (common.hpp:171-178).
struct Energy {
    double ini, end, tmp, kinetic, potential;
};

// Printing options (common.hpp:196-201).
struct options {
    bool print_screen;
    bool print_all;
    bool print_lagrange;
};

// One line of the input file (common.hpp:322-329): the mass is a float.
struct file_data {
    int id;
    float m;
    double r[3];
    double v[3];
};

// Wall-clock phase accumulators (common.hpp:287-310).
struct Gtime {
    double integration_ini, integration_end;
    double update_ini, update_end;
    double gflops;
};

}  // namespace gb300
#endif
