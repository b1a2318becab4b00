#include "Hermite4GPU.hpp"

#include <sstream>

#include "NbodyUtils.hpp"
#include "Timer.hpp"

namespace gb300 {

void Hermite4GPU::check(int status, const char *what) {
    if (status != H4_OK) {
        std::ostringstream s;
        s << what << ": " << h4_last_error() << " (" << h4_status_string(status) << ")";
        throw H4Failure(status, s.str());
    }
}

Hermite4GPU::Hermite4GPU(NbodySystem *ns_, Logger *logger_) : ns(ns_), logger(logger_), h_(nullptr) {
    check(h4_create(&h_, ns->n, ns->e2, ns->eta, ns->h_r, ns->h_v, ns->force_mode), "h4_create");
    if (ns->gpus > 1)
        logger->log_warning("this build runs one system on one GPU; --gpu " + std::to_string(ns->gpus) +
                            " is ignored");
    logger->log_info("GPUs: 1");
}

Hermite4GPU::Hermite4GPU(NbodySystem *ns_, Logger *logger_, const CheckpointScalars &resume_from)
    : ns(ns_), logger(logger_), h_(nullptr) {
    check(h4_create(&h_, ns->n, ns->e2, ns->eta, ns->h_r, ns->h_v, ns->force_mode), "h4_create");
    check(h4_set_dt_limits(h_, resume_from.dt_min > 0 ? resume_from.dt_min : D_TIME_MIN,
                           resume_from.dt_max > 0 ? resume_from.dt_max : D_TIME_MAX),
          "h4_set_dt_limits");
    check(h4_restore(h_, ns->h_r, ns->h_v, ns->h_f, ns->h_t, ns->h_dt, resume_from.atime), "h4_restore");
    resumed_ = true;
    chk_ = resume_from;
    logger->log_info("resuming at t = " + std::to_string(resume_from.itime));
}

Hermite4GPU::~Hermite4GPU() { h4_destroy(h_); }

void Hermite4GPU::next_integration_time(double &ATIME) {
    check(h4_next_integration_time(h_, &ATIME), "next_integration_time");
}

void Hermite4GPU::save_old_acc_jrk(unsigned int nact) { check(h4_save_old_acc_jrk(h_, nact), "save_old_acc_jrk"); }

unsigned int Hermite4GPU::find_particles_to_move(double ITIME) {
    unsigned int nact = 0;
    check(h4_find_particles_to_move(h_, ITIME, &nact), "find_particles_to_move");
    return nact;
}

void Hermite4GPU::init_dt(double &ATIME, float ETA, double ITIME) { check(h4_init_dt(h_, &ATIME, ETA, ITIME), "init_dt"); }

void Hermite4GPU::init_acc_jrk() { check(h4_init_acc_jrk(h_), "init_acc_jrk"); }

void Hermite4GPU::update_acc_jrk(int nact) {
    const double t0 = wall_seconds();
    check(h4_update_acc_jrk(h_, (unsigned)nact), "update_acc_jrk");
    float ms = 0.f;
    check(h4_last_timings(h_, &ms, nullptr), "update_acc_jrk timing");
    (void)t0;
    ns->gtime.update_end += ms * 1e-3;
}

void Hermite4GPU::predicted_pos_vel(double ITIME) { check(h4_predicted_pos_vel(h_, ITIME), "predicted_pos_vel"); }

void Hermite4GPU::correction_pos_vel(double ITIME, int nact) {
    check(h4_correction_pos_vel(h_, ITIME, (unsigned)nact), "correction_pos_vel");
}

double Hermite4GPU::get_energy_gpu() {
    double k = 0, p = 0, e = 0;
    check(h4_get_energy(h_, &k, &p, &e), "get_energy_gpu");
    ns->en.kinetic = k;
    ns->en.potential = p;
    return e;
}

void Hermite4GPU::advance(double t_stop, double t_log, double &ATIME, double &ITIME, unsigned long long &steps,
                          unsigned long long &psteps, unsigned long long &inter, unsigned int &last_nact) {
    double st[5] = {0, 0, 0, 0, 0};
    check(h4_advance(h_, t_stop, t_log, &ATIME, &ITIME, st), "advance");
    float adv_ms = 0.f;
    check(h4_last_timings(h_, nullptr, &adv_ms), "advance timing");
    ns->gtime.update_end += adv_ms * 1e-3;
    steps = (unsigned long long)st[0];
    psteps = (unsigned long long)st[1];
    inter = (unsigned long long)st[2];
    last_nact = (unsigned int)st[4];
}

void Hermite4GPU::sync_host() {
    check(h4_download(h_, ns->h_r, ns->h_v, ns->h_f, ns->h_old, ns->h_a2, ns->h_a3, ns->h_t, ns->h_dt, ns->h_move),
          "download");
}

// Hermite4GPU::integration (src/include/gpu/Hermite4GPU_integration.cpp:38-124):
// the same outputs at the same times.  The block steps between two outputs run
// on the device (h4_advance) unless --host-steps asks for the reference's
// call-per-method loop.  nbody_attributes (diagnostics only) is not computed.
void Hermite4GPU::integration() {
    ns->gtime.integration_ini = wall_seconds();
    double ATIME = 1.0e+10;
    double ITIME = ns->snapshot_time;
    unsigned int nact = 0;
    unsigned int nsteps = 0;
    long long interactions = 0;
    unsigned int output_factor = 1;
    unsigned int snap_number = ns->snapshot_number;
    const std::string chk_path = ns->output_filename + ".chk";

    if (resumed_) {
        ITIME = chk_.itime;
        ATIME = chk_.atime;
        nsteps = (unsigned int)chk_.nsteps;
        interactions = (long long)chk_.interactions;
        output_factor = (unsigned int)chk_.output_factor;
        snap_number = (unsigned int)chk_.snapshot_number;
        ns->iterations = (long long)chk_.iterations;
        ns->en.ini = chk_.e_ini;
        ns->en.tmp = chk_.e_tmp;
        logger->write_info();   // the energy log is appended to, not restarted
    } else {
        init_acc_jrk();
        init_dt(ATIME, ETA_S, ITIME);
        ns->en.ini = get_energy_gpu();
        ns->en.tmp = ns->en.ini;
        logger->print_info();
        logger->write_info();
        logger->print_energy_log(ITIME, (unsigned int)ns->iterations, interactions, nsteps, ns->en.ini);
        sync_host();
        logger->write_snapshot(snap_number, ITIME);
        snap_number++;
        if (ns->ops.print_all) logger->print_all(ITIME, snap_number);
    }
    NbodyUtils nu(ns, h_);
    if (!resumed_ && nu.nbody_attributes(ns->en.ini)) {
        std::ostringstream a;
        a << "r_virial " << nu.r_virial << ", t_cr " << nu.t_cr << ", r_core " << nu.r_core << ", r_hm "
          << nu.r_hm << ", t_rlx " << nu.t_rlx;
        logger->log_info(a.str());
    }
    if (!resumed_ && ns->ops.print_lagrange && nu.lagrange_radii()) logger->print_lagrange_radii(ITIME, nu.layers_radii);
    auto checkpoint = [&]() {
        CheckpointScalars sc{};
        sc.e2 = ns->e2;
        sc.eta = ns->eta;
        sc.dt_min = D_TIME_MIN;
        sc.dt_max = D_TIME_MAX;
        sc.itime = ITIME;
        sc.atime = ATIME;
        sc.iterations = (double)ns->iterations;
        sc.nsteps = nsteps;
        sc.interactions = (double)interactions;
        sc.e_ini = ns->en.ini;
        sc.e_tmp = ns->en.tmp;
        sc.output_factor = output_factor;
        sc.snapshot_number = snap_number;
        sc.t_end = ns->integration_time;
        write_checkpoint(chk_path, *ns, sc);
    };

    while (ITIME < ns->integration_time) {
        const float t_log_f = ns->interval_time * (float)output_factor;
        if (ns->host_steps) {
            ITIME = ATIME;
            nact = find_particles_to_move(ITIME);
            save_old_acc_jrk(nact);
            predicted_pos_vel(ITIME);
            update_acc_jrk(nact);
            correction_pos_vel(ITIME, nact);
            interactions += (long long)nact * ns->n;
            next_integration_time(ATIME);
            ns->iterations++;
            nsteps += nact;
        } else {
            unsigned long long steps = 0, psteps = 0, inter = 0;
            advance((double)ns->integration_time, (double)t_log_f, ATIME, ITIME, steps, psteps, inter, nact);
            interactions += (long long)inter;
            ns->iterations += (long long)steps;
            nsteps += (unsigned int)psteps;
        }
        if (ITIME >= t_log_f) {
            // values as the reference prints them: before the step is counted
            const double e = get_energy_gpu();
            logger->print_energy_log(ITIME, (unsigned int)(ns->iterations - 1), interactions,
                                     nsteps - nact, e);
            sync_host();
            if (ns->ops.print_all) logger->print_all(ITIME, snap_number);
            if (ns->ops.print_lagrange && nu.lagrange_radii()) logger->print_lagrange_radii(ITIME, nu.layers_radii);
            logger->write_snapshot(snap_number, ITIME);
            snap_number++;
            output_factor += 1;
            checkpoint();
        }
    }
    ns->gtime.integration_end = wall_seconds() - ns->gtime.integration_ini;
    sync_host();
    checkpoint();
    logger->write_snapshot(snap_number, ITIME);
    logger->add_info("SnapshotNumber:", std::to_string(snap_number));
}

}  // namespace gb300
