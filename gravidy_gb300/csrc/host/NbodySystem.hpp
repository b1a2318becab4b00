// Particle system and run parameters: the fields of the reference's
// NbodySystem (src/include/NbodySystem.hpp:48-134) that the Hermite4 block
// step uses, with the same names, plus the input reader.  The host arrays are
// mirrors of the device state, refreshed by Hermite4GPU::sync_host() for logs
// and snapshots; the per-GPU d_* arrays of the reference are replaced by the
// device state of an h4_handle.
#ifndef GRAVIDY_GB300_HOST_NBODYSYSTEM_HPP
#define GRAVIDY_GB300_HOST_NBODYSYSTEM_HPP

#include <string>
#include <vector>

#include "OptionsParser.hpp"
#include "common.hpp"

namespace gb300 {

class NbodySystem {
  public:
    explicit NbodySystem(const OptionsParser &op);
    ~NbodySystem();
    NbodySystem(const NbodySystem &) = delete;
    NbodySystem &operator=(const NbodySystem &) = delete;

    Gtime gtime;
    std::vector<file_data> reader;
    options ops;

    int gpus;
    long long int iterations;
    unsigned int n;
    unsigned int snapshot_number;
    unsigned int length_snap;
    int force_mode;
    bool host_steps;

    float eta;
    float total_mass;
    float integration_time;
    float interval_time;

    double e2;
    double snapshot_time;
    bool resume;
    bool resume_info;               // resumed from a reference .info file: read snapshot_filename
    Energy en;
    float max_mass;

    std::string input_filename;
    std::string output_filename;
    std::string resume_filename;
    std::string snapshot_filename;

    // Host mirrors (NbodySystem.hpp:112-128).
    unsigned int *h_id;
    unsigned int *h_move;
    double *h_t;
    double *h_dt;
    double4 *h_r;   // position + mass
    double4 *h_v;   // velocity
    double3 *h_a2;
    double3 *h_a3;
    Forces *h_f;
    Forces *h_old;

    // NbodySystem::read_input_file (NbodySystem.cpp:79-207).  Returns false
    // (with a message) if the file cannot be read; a line with a token count
    // other than 8 ends the reading, as in the reference.
    bool read_input_file();
    // NbodySystem::alloc_base_attributes / copy_input_data
    // (NbodySystem.cpp:212-263), and the host arrays Hermite4 allocates
    // (Hermite4.cpp:158-171).
    void alloc_base_attributes(int rank);
    void copy_input_data();
    void free_base_attributes();
};

}  // namespace gb300
#endif
