// Hermite4GB300: see Hermite4GB300.hpp.  Written against the reference's
// classes: NbodySystem (src/include/NbodySystem.hpp:48-134), Logger
// (src/include/utils/Logger.hpp), NbodyUtils (src/include/utils/NbodyUtils.hpp)
// and the loop of src/include/gpu/Hermite4GPU_integration.cpp:38-124.
#include "Hermite4GB300.hpp"

#include <cstdlib>
#include <vector>

static const char *gb300_mode_env() {
    const char *m = std::getenv("GRAVIDY_GB300_MODE");
    return m ? m : "fp64";
}

static int gb300_mode() {
    const std::string m = gb300_mode_env();
    if (m == "exact") return H4_FORCE_EXACT;
    if (m == "mixed") return H4_FORCE_MIXED;
    return H4_FORCE_FP64;
}

void Hermite4GB300::check(int status, const char *what) {
    if (status != H4_OK) {
        logger->log_error(std::string(what) + ": " + h4_last_error());
        std::exit(EXIT_FAILURE);   // the reference's CSC behaviour (Hermite4GPU.cuh:43-50)
    }
}

Hermite4GB300::Hermite4GB300(NbodySystem *ns, Logger *logger, NbodyUtils *nu)
    : Hermite4(ns, logger, nu), h_(0) {
    // ns->h_r / h_v have the layout of h4_double4 (x, y, z, w)
    check(h4_create(&h_, ns->n, ns->e2, ns->eta, (const h4_double4 *)ns->h_r, (const h4_double4 *)ns->h_v,
                    gb300_mode()),
          "h4_create");
    logger->log_info(std::string("GPUs: 1 (GB300, ") + gb300_mode_env() + " forces)");
}

Hermite4GB300::~Hermite4GB300() { h4_destroy(h_); }

void Hermite4GB300::init_acc_jrk() { check(h4_init_acc_jrk(h_), "init_acc_jrk"); }

void Hermite4GB300::update_acc_jrk(int nact) {
    // the log's GFLOPS column divides by the accumulated update time
    // (Logger.cpp:333-335); here the force kernel's device time
    check(h4_update_acc_jrk(h_, (unsigned)nact), "update_acc_jrk");
    float ms = 0.f;
    check(h4_last_timings(h_, &ms, 0), "update_acc_jrk");
    ns->gtime.update_end += ms * 1e-3f;
}

void Hermite4GB300::predicted_pos_vel(double ITIME) { check(h4_predicted_pos_vel(h_, ITIME), "predicted_pos_vel"); }

void Hermite4GB300::correction_pos_vel(double ITIME, int nact) {
    check(h4_correction_pos_vel(h_, ITIME, (unsigned)nact), "correction_pos_vel");
}

double Hermite4GB300::get_energy_gpu() {
    double k = 0, p = 0, e = 0;
    check(h4_get_energy(h_, &k, &p, &e), "get_energy_gpu");
    ns->en.kinetic = k;
    ns->en.potential = p;
    return e;
}

unsigned int Hermite4GB300::find_particles_to_move(double ITIME) {
    unsigned int nact = 0;
    check(h4_find_particles_to_move(h_, ITIME, &nact), "find_particles_to_move");
    return nact;
}

void Hermite4GB300::next_integration_time(double &ATIME) {
    check(h4_next_integration_time(h_, &ATIME), "next_integration_time");
}

void Hermite4GB300::init_dt(double &ATIME, float ETA, double ITIME) { check(h4_init_dt(h_, &ATIME, ETA, ITIME), "init_dt"); }

void Hermite4GB300::save_old_acc_jrk(unsigned int nact) { check(h4_save_old_acc_jrk(h_, nact), "save_old_acc_jrk"); }

void Hermite4GB300::sync_host() {
    check(h4_download(h_, (h4_double4 *)ns->h_r, (h4_double4 *)ns->h_v, (h4_forces *)ns->h_f,
                      (h4_forces *)ns->h_old, (h4_double3 *)ns->h_a2, (h4_double3 *)ns->h_a3, ns->h_t, ns->h_dt,
                      ns->h_move),
          "download");
    std::vector<h4_double4> pr(ns->n), pv(ns->n);
    check(h4_download_predicted(h_, &pr[0], &pv[0]), "download predicted");
    for (unsigned int i = 0; i < ns->n; i++) {
        ns->h_p[i].r[0] = pr[i].x; ns->h_p[i].r[1] = pr[i].y; ns->h_p[i].r[2] = pr[i].z;
        ns->h_p[i].v[0] = pv[i].x; ns->h_p[i].v[1] = pv[i].y; ns->h_p[i].v[2] = pv[i].z;
        ns->h_p[i].m = (float)pr[i].w;
    }
}

// The loop of Hermite4GPU_integration.cpp:38-124, the block steps between two
// outputs on the device (h4_advance).
void Hermite4GB300::integration() {
    ns->gtime.integration_ini = omp_get_wtime();
    double ATIME = 1.0e+10;
    double ITIME = ns->snapshot_time;
    unsigned int nsteps = 0;
    long long interactions = 0;
    unsigned int output_factor = 1;

    init_acc_jrk();
    init_dt(ATIME, ETA_S, ITIME);
    ns->en.ini = get_energy_gpu();
    ns->en.tmp = ns->en.ini;
    sync_host();
    nu->nbody_attributes();
    logger->print_info();
    logger->write_info();
    logger->print_energy_log(ITIME, ns->iterations, interactions, nsteps, ns->en.ini);
    unsigned int snap_number = ns->snapshot_number;
    logger->write_snapshot(snap_number, ITIME);
    snap_number++;
    if (ns->ops.print_all) logger->print_all(ITIME, snap_number);
    if (ns->ops.print_lagrange) {
        nu->lagrange_radii();
        logger->print_lagrange_radii(ITIME, nu->layers_radii);
    }
    while (ITIME < ns->integration_time) {
        const float t_log = ns->interval_time * output_factor;
        double st[5] = {0, 0, 0, 0, 0};
        const double t0 = omp_get_wtime();
        check(h4_advance(h_, ns->integration_time, t_log, &ATIME, &ITIME, st), "advance");
        ns->gtime.update_end += (float)(omp_get_wtime() - t0);
        interactions += (long long)st[2];
        ns->iterations += (long long)st[0];
        nsteps += (unsigned int)st[1];
        if (ITIME >= t_log) {
            const unsigned int last = (unsigned int)st[4];
            const double e = get_energy_gpu();
            sync_host();
            logger->print_energy_log(ITIME, (unsigned int)(ns->iterations - 1), interactions, nsteps - last, e);
            if (ns->ops.print_all) logger->print_all(ITIME, snap_number);
            if (ns->ops.print_lagrange) {
                nu->lagrange_radii();
                logger->print_lagrange_radii(ITIME, nu->layers_radii);
            }
            logger->write_snapshot(snap_number, ITIME);
            snap_number++;
            output_factor += 1;
        }
    }
    ns->gtime.integration_end = omp_get_wtime() - ns->gtime.integration_ini;
    sync_host();
    logger->write_snapshot(snap_number, ITIME);
    logger->add_info(std::string("SnapshotNumber:"), std::string(SSTR(snap_number)));
}
