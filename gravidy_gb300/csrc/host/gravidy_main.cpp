// gravidy-gb300: the reference program's flow (src/gravidy.cpp:54-115) over
// the GB300 Hermite4 path -- parse options, read the input file, build the
// system, integrate with the energy log and snapshots.
#include <iostream>

#include "Hermite4GPU.hpp"
#include "Logger.hpp"
#include "NbodySystem.hpp"
#include "OptionsParser.hpp"

int main(int argc, char *argv[]) {
    using namespace gb300;
    OptionsParser op(argc, argv);
    if (!op.check_options()) return 1;
    NbodySystem ns(op);
    CheckpointScalars chk{};
    const bool exact_resume = op.resume && !op.resume_info;
    if (exact_resume) {
        // exact continuation: state and loop counters from the checkpoint
        if (!read_checkpoint(op.resume_filename, ns, chk)) return 1;
    } else {
        if (!ns.read_input_file()) return 1;
        ns.alloc_base_attributes(0);
        ns.copy_input_data();
    }
    Logger logger(&ns);
    try {
        if (exact_resume) {
            Hermite4GPU h4(&ns, &logger, chk);
            h4.integration();
        } else {
            Hermite4GPU h4(&ns, &logger);
            h4.integration();
        }
    } catch (const H4Failure &e) {
        logger.log_error(e.what());
        return 2;
    }
    logger.log_success("Finishing...");
    return 0;
}
