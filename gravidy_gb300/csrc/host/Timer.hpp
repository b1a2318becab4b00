// Wall clock for the log's ElapsedTime and GFLOPS columns (the reference uses
// omp_get_wtime, src/include/utils/Logger.cpp:331).
#ifndef GRAVIDY_GB300_HOST_TIMER_HPP
#define GRAVIDY_GB300_HOST_TIMER_HPP
#include <chrono>
namespace gb300 {
inline double wall_seconds() {
    using namespace std::chrono;
    return duration_cast<duration<double>>(steady_clock::now().time_since_epoch()).count();
}
}  // namespace gb300
#endif
