// Command-line options of the reference program (src/include/utils/
// OptionsParser.hpp:50-79, flags and defaults of OptionsParser.cpp:41-81 and
// :329-421), parsed without boost.  Added flags: --mode fp64|exact|mixed
// selects the force arithmetic, --host-steps drives the block steps one by
// one from the host instead of the device-resident loop.  -r takes either
// this program's exact checkpoint (<out>.chk) or, as the reference does, an
// <out>.info file (OptionsParser.cpp:122-323): the run restarts from the
// snapshot that file names.
#ifndef GRAVIDY_GB300_HOST_OPTIONSPARSER_HPP
#define GRAVIDY_GB300_HOST_OPTIONSPARSER_HPP

#include <string>

#include "common.hpp"

namespace gb300 {

class OptionsParser {
  public:
    OptionsParser(int argc, char *argv[]);

    std::string input_filename;
    std::string output_filename;
    std::string resume_filename;
    std::string snapshot_filename;
    float integration_time;
    float interval_time;
    int gpus;
    float snapshot_time;
    float softening;
    float eta;
    unsigned int snapshot_number;
    unsigned int length_output_number;
    bool resume;
    bool resume_info;   // resume from the reference's <out>.info and its 4-digit snapshot
    options ops;
    int force_mode;
    bool host_steps;

    bool file_exists(const std::string &filename) const;
    bool check_options();
    std::string usage() const;

  private:
    bool read_info(bool have_time, bool have_softening, bool have_eta, bool have_screen);
    int argc_;
    char **argv_;
};

}  // namespace gb300
#endif
