/* The reference program's main (src/gravidy.cpp:54-115) with the GB300
 * backend class Hermite4GB300 in place of Hermite4GPU -- what the reference's
 * main becomes when its GPU branch constructs Hermite4GB300 instead.  Test
 * infrastructure: it shows the adapter compiles and links against the
 * reference's own classes (make -C oracle adapter); the reference's
 * gravidy.cpp itself is not modified. */
#include "gb300/Hermite4GB300.hpp"

int main(int argc, char *argv[])
{
    OptionsParser op(argc, argv);
    if (!op.check_options()) return 1;
    NbodySystem ns(op);
    ns.read_input_file();
    ns.alloc_base_attributes(0);
    ns.copy_input_data();
    Logger logger(&ns);
    NbodyUtils nu(&ns);
    Hermite4GB300 h4(&ns, &logger, &nu);
    h4.integration();
    logger.log_success(std::string("Finishing..."));
    return 0;
}
