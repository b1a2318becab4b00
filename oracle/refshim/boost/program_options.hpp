/* Minimal stand-in for <boost/program_options.hpp>, used only to compile the
 * reference GraviDy CPU path as a test oracle (boost is not installed here).
 *
 * The reference header src/include/utils/OptionsParser.hpp:39,69-70 needs the
 * namespace and two default-constructible member types; nothing else from
 * boost is used by the sources compiled into the oracle, because
 * utils/OptionsParser.cpp is replaced by oracle/ref_options.cpp. */
#ifndef ORACLE_REFSHIM_BOOST_PROGRAM_OPTIONS_HPP
#define ORACLE_REFSHIM_BOOST_PROGRAM_OPTIONS_HPP
namespace boost {
namespace program_options {
class variables_map {};
class options_description {};
}  // namespace program_options
}  // namespace boost
#endif
