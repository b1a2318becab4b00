#include "OptionsParser.hpp"

#include <sys/stat.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <map>
#include <sstream>

namespace gb300 {

OptionsParser::OptionsParser(int argc, char *argv[])
    : integration_time(1.0f), interval_time((float)D_TIME_MAX), gpus(0), snapshot_time(0.0f),
      softening((float)E), eta(ETA_N), snapshot_number(0), length_output_number(0), resume(false),
      resume_info(false),
      force_mode(H4_FORCE_FP64), host_steps(false), argc_(argc), argv_(argv) {
    ops.print_screen = false;
    ops.print_all = false;
    ops.print_lagrange = false;
}

bool OptionsParser::file_exists(const std::string &filename) const {
    struct stat buffer;
    return stat(filename.c_str(), &buffer) != -1;
}

std::string OptionsParser::usage() const {
    std::ostringstream s;
    s << "GraviDy (GB300)\n"
      << "  -h [ --help ]                  Display this message\n"
      << "Required options:\n"
      << "  -i [ --input ] <filename>      Input data filename\n"
      << "  -t [ --time ] <value> (=1)     Integration time (In N-body units)\n"
      << "  -r [ --resume ] <file>         Resume a run: <out>.chk (exact checkpoint) or\n"
      << "                                 <out>.info (restart from its last snapshot)\n"
      << "Elective options:\n"
      << "  -o [ --output ] <filename>     Output data filename\n"
      << "  -s [ --softening ] <value>     Softening parameter (default 1e-4)\n"
      << "  -e [ --eta ] <value>           ETA of time-step calculation (default 0.01)\n"
      << "  -p [ --screen ]                Print summary in the screen instead of a file\n"
      << "  -z [ --interval ] <value>      Output time interval (default 0.125)\n"
      << "Extra options:\n"
      << "  -l [ --lagrange ]              Print the Lagrange radii at every output time\n"
      << "  -a [ --all ]                   Print all the information of N-particles\n"
      << "  -g [ --gpu ] <value> (=0)      GPUs to use (one GPU is used)\n"
      << "  --mode fp64|exact|mixed        Force arithmetic (default fp64)\n"
      << "  --host-steps                   Drive every block step from the host\n";
    return s.str();
}

static bool is_opt(const char *a, const char *s, const char *l) {
    return (s && std::strcmp(a, s) == 0) || std::strcmp(a, l) == 0;
}

// The reference's resume from an info file (OptionsParser.cpp:122-323):
// "# Key: value" lines with the keys below; the run restarts at the info
// file's IntegrationTime (which -t must exceed) from the snapshot
// <OutputFilename>.snapshot_<SnapshotNumber, 4 digits>, with the info file's
// softening, eta and screen flag unless given on the command line, and
// writes to <InputFilename>.out.  The reference's resume branch leaves the
// output interval, the snapshot-counter width and the -a/-l flags
// uninitialised (its constructor, OptionsParser.cpp:41-89, sets none of
// them); here they come from the command line and the defaults, as in a
// fresh run.  A resumed run is then a fresh run from the snapshot file (whose
// "# Time:" header sets the start time) under the info file's parameters.
bool OptionsParser::read_info(bool have_time, bool have_softening, bool have_eta, bool have_screen) {
    std::cerr << "Reading resume_filename: " << resume_filename << std::endl;
    static const char *allowed[] = {"NumberParticles", "Softening",     "EtaTimestep",    "IntegrationTime",
                                    "PrintScreen",     "InputFilename", "OutputFilename", "SnapshotNumber"};
    std::map<std::string, std::string> cfg;
    std::ifstream rfile(resume_filename.c_str());
    std::string key, value;
    while (rfile.good() && std::getline(rfile, key, ':')) {
        key.erase(std::remove_if(key.begin(), key.end(), [](char c) { return c == '#' || c == ' '; }), key.end());
        if (std::getline(rfile, value)) {
            value.erase(std::remove(value.begin(), value.end(), ' '), value.end());
            cfg[key] = value;
        }
    }
    for (const auto &kv : cfg) {
        if (std::find_if(std::begin(allowed), std::end(allowed),
                         [&](const char *a) { return kv.first == a; }) == std::end(allowed)) {
            std::cerr << "Invalid param" << std::endl
                      << "gravidy: Invalid option -- " << kv.first << " in the info file" << std::endl
                      << usage() << std::endl;
            return false;
        }
        std::cerr << kv.first << " -> " << kv.second << std::endl;
    }
    if (!have_time) {
        std::cerr << "gravidy: option requires an argument -- 'time'" << std::endl << usage() << std::endl;
        return false;
    }
    const double config_time = std::strtod(cfg["IntegrationTime"].c_str(), nullptr);
    if (config_time >= integration_time) {
        std::cerr << "gravidy: option requires an argument -- 'time' greater than the one specifid in the info file"
                  << std::endl << usage() << std::endl;
        return false;
    }
    snapshot_time = (float)config_time;
    if (!have_softening) softening = (float)std::strtod(cfg["Softening"].c_str(), nullptr);
    if (!have_eta) eta = (float)std::strtod(cfg["EtaTimestep"].c_str(), nullptr);
    if (!have_screen) ops.print_screen = std::atoi(cfg["PrintScreen"].c_str()) != 0;
    input_filename = cfg["InputFilename"];
    output_filename = input_filename + ".out";
    snapshot_number = (unsigned int)std::atoi(cfg["SnapshotNumber"].c_str());
    std::ostringstream snap;
    snap << cfg["OutputFilename"] << ".snapshot_" << std::setw(4) << std::setfill('0') << snapshot_number;
    if (!file_exists(snap.str())) {
        std::cerr << "gravidy: cannot access " << snap.str() << ": No such file or directory\n"
                  << "(Check the OutputFilename and SnapshotNumber)" << std::endl;
        return false;
    }
    snapshot_filename = snap.str();
    return true;
}

bool OptionsParser::check_options() {
    bool have_input = false, have_output = false, have_time = false, have_softening = false, have_eta = false;
    std::string out;
    for (int k = 1; k < argc_; k++) {
        const char *a = argv_[k];
        if (is_opt(a, "-h", "--help")) { std::cerr << usage() << std::endl; return false; }
        if (is_opt(a, "-p", "--screen")) { ops.print_screen = true; continue; }
        if (is_opt(a, "-a", "--all")) { ops.print_all = true; continue; }
        if (is_opt(a, "-l", "--lagrange")) { ops.print_lagrange = true; continue; }
        if (is_opt(a, nullptr, "--host-steps")) { host_steps = true; continue; }
        static const char *with_value[][2] = {{"-i", "--input"}, {"-t", "--time"}, {"-o", "--output"},
                                              {"-s", "--softening"}, {"-e", "--eta"}, {"-z", "--interval"},
                                              {"-g", "--gpu"}, {nullptr, "--mode"}, {"-r", "--resume"}};
        bool known = false;
        for (auto &w : with_value) known = known || is_opt(a, w[0], w[1]);
        if (!known) {
            std::cerr << "gravidy: unknown option " << a << "\n" << usage() << std::endl;
            return false;
        }
        if (k + 1 >= argc_) {
            std::cerr << "gravidy: option requires an argument -- '" << a << "'" << std::endl;
            return false;
        }
        const char *v = argv_[++k];
        if (is_opt(a, "-i", "--input")) { input_filename = v; have_input = true; }
        else if (is_opt(a, "-t", "--time")) { integration_time = (float)std::strtod(v, nullptr); have_time = true; }
        else if (is_opt(a, "-o", "--output")) { out = v; have_output = true; }
        else if (is_opt(a, "-s", "--softening")) { softening = (float)std::strtod(v, nullptr); have_softening = true; }
        else if (is_opt(a, "-e", "--eta")) { eta = (float)std::strtod(v, nullptr); have_eta = true; }
        else if (is_opt(a, "-z", "--interval")) interval_time = (float)std::strtod(v, nullptr);
        else if (is_opt(a, "-g", "--gpu")) gpus = std::atoi(v);
        else if (is_opt(a, nullptr, "--mode")) {
            std::string m = v;
            if (m == "fp64") force_mode = H4_FORCE_FP64;
            else if (m == "exact") force_mode = H4_FORCE_EXACT;
            else if (m == "mixed") force_mode = H4_FORCE_MIXED;
            else { std::cerr << "gravidy: unknown --mode " << m << std::endl; return false; }
        } else if (is_opt(a, "-r", "--resume")) {
            resume_filename = v;
            resume = true;
        } else {
            std::cerr << "gravidy: unknown option " << a << "\n" << usage() << std::endl;
            return false;
        }
    }
    const bool screen_flag = ops.print_screen;
    if (resume) {
        if (!file_exists(resume_filename)) {
            std::cerr << "gravidy: cannot access " << resume_filename << ": No such file or directory" << std::endl;
            return false;
        }
        const std::string ext = ".chk";
        resume_info = !(resume_filename.size() >= ext.size() &&
                        resume_filename.compare(resume_filename.size() - ext.size(), ext.size(), ext) == 0);
        if (resume_info) {
            if (!read_info(have_time, have_softening, have_eta, screen_flag)) return false;
        } else if (!have_input) {
            input_filename = resume_filename;
        }
    } else if (!have_input) {
        std::cerr << "gravidy: option requires an argument -- 'input'" << std::endl << usage() << std::endl;
        return false;
    }
    if (!resume && !file_exists(input_filename)) {
        std::cerr << "gravidy: cannot access " << input_filename << ": No such file or directory" << std::endl;
        return false;
    }
    if (!(integration_time > 0.0f) || !(interval_time > 0.0f) || !(eta > 0.0f) || !(softening >= 0.0f)) {
        std::cerr << "gravidy: time, interval and eta must be > 0, softening >= 0" << std::endl;
        return false;
    }
    // Digits of the snapshot counter (OptionsParser.cpp:392-399).
    length_output_number = 0;
    unsigned int tmp = (unsigned int)(integration_time / interval_time);
    do {
        ++length_output_number;
        tmp /= 10;
    } while (tmp);
    length_output_number += 1;
    if (!resume_info) output_filename = (have_output ? out : input_filename) + ".out";
    return true;
}

}  // namespace gb300
