// Hermite4GB300 -- the GB300 path as a backend class of the reference program.
//
// A maintainer adds this header and Hermite4GB300.cpp next to the reference's
// backends (src/include/gb300/), compiles the reference sources with -DGB300
// and links libgravidy_gb300.so.  The class derives from the reference's
// Hermite4 (src/include/Hermite4.hpp:48-88) and has the constructor and
// methods of Hermite4GPU (src/include/gpu/Hermite4GPU.cuh:100-144); the
// reference's main (src/gravidy.cpp:89-95) then needs one more branch:
//
//     #elif defined(GB300)
//     Hermite4GB300 h4(&ns, &logger, &nu);
//
// The particle state lives on the GPU behind an h4_handle; the NbodySystem
// arrays (h_r, h_v, h_f, h_t, h_dt, ...) are refreshed from it whenever the
// reference's logger or utilities read them (energy log times, snapshots,
// Lagrange radii).
#ifndef HERMITE4GB300_HPP
#define HERMITE4GB300_HPP

#include "../Hermite4.hpp"
#include "gravidy_gb300.h"

class Hermite4GB300 : public Hermite4 {
  public:
    Hermite4GB300(NbodySystem *ns, Logger *logger, NbodyUtils *nu);
    ~Hermite4GB300();

    // Hermite4GPU's methods (Hermite4GPU.cuh:129-142)
    void init_acc_jrk();
    void update_acc_jrk(int nact);
    void predicted_pos_vel(double ITIME);
    void correction_pos_vel(double ITIME, int nact);
    void integration();
    double get_energy_gpu();

    // Hermite4's host methods (Hermite4.hpp:60-63), here on the device
    unsigned int find_particles_to_move(double ITIME);
    void next_integration_time(double &ATIME);
    void init_dt(double &ATIME, float ETA, double ITIME);
    void save_old_acc_jrk(unsigned int nact);

    // Copy the device state into ns->h_* (and h_p, the predictors).
    void sync_host();

  private:
    void check(int status, const char *what);
    h4_handle h_;
};

#endif
