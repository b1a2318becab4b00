/* Command-line parsing for the oracle build of the reference GraviDy CPU path.
 *
 * This translation unit replaces src/include/utils/OptionsParser.cpp (which
 * needs boost::program_options) and defines the members declared in
 * src/include/utils/OptionsParser.hpp:50-79.  It fills the same fields with
 * the same defaults as OptionsParser.cpp:41-81 and :329-421:
 *   -i/--input  -t/--time (1)  -o/--output  -s/--softening (E = 1e-4)
 *   -e/--eta (ETA_N)  -z/--interval (D_TIME_MAX)  -p/--screen  -a/--all
 *   -l/--lagrange  -g/--gpu (0)
 * Resume (-r) is not supported by the oracle and is rejected.
 *
 * Test infrastructure only: this file is compiled together with the reference
 * sources into oracle/_ref/ and is never part of the product library. */
#include "utils/OptionsParser.hpp"
#include <cstdlib>
#include <cstring>

namespace {
struct Args {
    int argc;
    char **argv;
};
Args g_args;
}  // namespace

OptionsParser::OptionsParser(int argc, char *argv[])
{
    g_args.argc = argc;
    g_args.argv = argv;
    this->argc = argc;
    this->argv = argc > 0 ? argv[0] : 0;
    input_filename = "";
    output_filename = "";
    resume_filename = "";
    snapshot_filename = "";
    integration_time = 1.0f;
    interval_time = (float)D_TIME_MAX;
    gpus = 0;
    snapshot_time = 0.0f;
    softening = (float)E;
    eta = ETA_N;
    snapshot_number = 0;
    length_output_number = 0;
    resume = false;
    ops.print_screen = false;
    ops.print_all = false;
    ops.print_lagrange = false;
}

OptionsParser::~OptionsParser() {}

bool OptionsParser::file_exists(std::string filename)
{
    struct stat buffer;
    return stat(filename.c_str(), &buffer) != -1;
}

static bool is_opt(const char *a, const char *s, const char *l)
{
    return std::strcmp(a, s) == 0 || std::strcmp(a, l) == 0;
}

bool OptionsParser::check_options()
{
    bool have_input = false;
    bool have_output = false;
    std::string out;
    for (int k = 1; k < g_args.argc; k++) {
        const char *a = g_args.argv[k];
        const char *v = (k + 1 < g_args.argc) ? g_args.argv[k + 1] : 0;
        if (is_opt(a, "-p", "--screen")) { ops.print_screen = true; continue; }
        if (is_opt(a, "-a", "--all")) { ops.print_all = true; continue; }
        if (is_opt(a, "-l", "--lagrange")) { ops.print_lagrange = true; continue; }
        if (v == 0) {
            std::cerr << "gravidy(oracle): missing value for " << a << std::endl;
            return false;
        }
        if (is_opt(a, "-i", "--input")) { input_filename = v; have_input = true; }
        else if (is_opt(a, "-t", "--time")) { integration_time = (float)std::strtod(v, 0); }
        else if (is_opt(a, "-o", "--output")) { out = v; have_output = true; }
        else if (is_opt(a, "-s", "--softening")) { softening = (float)std::strtod(v, 0); }
        else if (is_opt(a, "-e", "--eta")) { eta = (float)std::strtod(v, 0); }
        else if (is_opt(a, "-z", "--interval")) { interval_time = (float)std::strtod(v, 0); }
        else if (is_opt(a, "-g", "--gpu")) { gpus = std::atoi(v); }
        else if (is_opt(a, "-r", "--resume")) {
            std::cerr << "gravidy(oracle): resume is not supported" << std::endl;
            return false;
        } else {
            std::cerr << "gravidy(oracle): unknown option " << a << std::endl;
            return false;
        }
        k++;
    }
    if (!have_input) {
        std::cerr << "gravidy: option requires an argument -- 'input'" << std::endl;
        return false;
    }
    if (!file_exists(input_filename)) {
        std::cerr << "gravidy: cannot access " << input_filename
                  << ": No such file or directory" << std::endl;
        return false;
    }
    /* Number of digits of the snapshot counter, as OptionsParser.cpp:392-399. */
    length_output_number = 0;
    unsigned int tmp = (integration_time / interval_time);
    do {
        ++length_output_number;
        tmp /= 10;
    } while (tmp);
    length_output_number += 1;
    output_filename = (have_output ? out : input_filename) + ".out";
    return true;
}
