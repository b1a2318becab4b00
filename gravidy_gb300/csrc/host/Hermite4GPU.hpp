// Drop-in for the reference's GPU integrator class Hermite4GPU
// (src/include/gpu/Hermite4GPU.cuh:100-144) and the Hermite4 base methods it
// inherits (src/include/Hermite4.hpp:48-88): the same constructor arguments
// and method names, so the flow of the reference's main program
// (src/gravidy.cpp:54-115) is kept.  Every method is a call into the C ABI
// of include/gravidy_gb300.h; the particle state lives on the GPU and the
// NbodySystem arrays are mirrors refreshed by sync_host().  Errors throw
// H4Failure (the reference exits the process, Hermite4GPU.cuh:43-50).
#ifndef GRAVIDY_GB300_HOST_HERMITE4GPU_HPP
#define GRAVIDY_GB300_HOST_HERMITE4GPU_HPP

#include <stdexcept>
#include <string>

#include "Checkpoint.hpp"
#include "Logger.hpp"
#include "NbodySystem.hpp"

namespace gb300 {

class H4Failure : public std::runtime_error {
  public:
    H4Failure(int status, const std::string &what) : std::runtime_error(what), status(status) {}
    int status;
};

class Hermite4GPU {
  public:
    Hermite4GPU(NbodySystem *ns, Logger *logger);
    // Continue a run from a checkpoint already read into ns (read_checkpoint).
    Hermite4GPU(NbodySystem *ns, Logger *logger, const CheckpointScalars &resume_from);
    ~Hermite4GPU();
    Hermite4GPU(const Hermite4GPU &) = delete;
    Hermite4GPU &operator=(const Hermite4GPU &) = delete;

    NbodySystem *ns;
    Logger *logger;

    // Hermite4 base (Hermite4.hpp:60-63)
    void next_integration_time(double &ATIME);
    void save_old_acc_jrk(unsigned int nact);
    unsigned int find_particles_to_move(double ITIME);
    void init_dt(double &ATIME, float ETA, double ITIME);

    // Hermite4GPU (Hermite4GPU.cuh:129-142)
    void init_acc_jrk();
    void update_acc_jrk(int nact);
    void predicted_pos_vel(double ITIME);
    void correction_pos_vel(double ITIME, int nact);
    void integration();
    double get_energy_gpu();

    // Device-resident block steps until ITIME >= t_stop or >= t_log.
    void advance(double t_stop, double t_log, double &ATIME, double &ITIME, unsigned long long &steps,
                 unsigned long long &psteps, unsigned long long &inter, unsigned int &last_nact);
    // Copy the device state into the NbodySystem arrays.
    void sync_host();

    h4_handle handle() const { return h_; }

  private:
    bool resumed_ = false;
    CheckpointScalars chk_{};
    void check(int status, const char *what);
    h4_handle h_;
};

}  // namespace gb300
#endif
