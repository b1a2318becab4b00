// Output of the run: the energy log (src/include/utils/Logger.cpp:324-391,
// same columns and number formats), snapshots in the reference's format
// (Logger.cpp:77-111), the .info file (Logger.cpp:113-217), the per-particle
// dump of -a (Logger.cpp:270-322) and the coloured messages
// (Logger.cpp:393-460).
#ifndef GRAVIDY_GB300_HOST_LOGGER_HPP
#define GRAVIDY_GB300_HOST_LOGGER_HPP

#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "NbodySystem.hpp"

namespace gb300 {

class Logger {
  public:
    explicit Logger(NbodySystem *ns);

    NbodySystem *ns;
    bool print_screen;
    std::string ofname;
    std::string ofname_info;

    std::string get_timestamp() const;
    void print_info();
    void add_info(const std::string &key, const std::string &value);
    void write_info();
    void write_snapshot(unsigned int snapshot_number, double ITIME);
    void print_all(double ITIME, unsigned int snapshot_number);
    void print_energy_log(double ITIME, unsigned int iterations, long long interactions, unsigned int nsteps,
                          double new_energy);
    // Logger::print_lagrange_radii (Logger.cpp:239-268): "01 t r1 .. r6" to
    // <out>.radii (appended) or the screen.
    void print_lagrange_radii(double ITIME, const std::vector<double> &radii);
    void log_error(const std::string &msg);
    void log_warning(const std::string &msg);
    void log_success(const std::string &msg);
    void log_info(const std::string &msg);

  private:
    void log(int type, const std::string &msg);
};

}  // namespace gb300
#endif
