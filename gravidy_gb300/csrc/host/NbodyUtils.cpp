#include "NbodyUtils.hpp"

#include <cmath>

namespace gb300 {

NbodyUtils::NbodyUtils(NbodySystem *ns_, h4_handle h)
    : ns(ns_), layers_radii(6, 0.0), r_virial(0), t_cr(0), r_cl(0), dt_cl(0), r_core(0), t_rlx(0), r_hm(0), h_(h) {
    cod.x = cod.y = cod.z = 0.0;
}

bool NbodyUtils::nbody_attributes(double e_ini) {
    if (ns->n < 8) return false;   // the 6th-neighbour density needs n >= 8
    const float M = ns->total_mass;
    const unsigned int n = ns->n;
    // get_virial_radius (:81-86), kept as the float NbodySystem::r_virial
    const float rv = (-G * M * M) / (4 * e_ini);
    r_virial = rv;
    // get_crossing_time (:88-97)
    const float Rv3 = (double)rv * (double)rv * (double)rv;
    const float Ut = std::sqrt((double)(Rv3 / (G * M)));
    t_cr = (float)(2 * std::sqrt(2.0) * Ut);
    // get_close_encounter_radius / _timestep (:99-110)
    r_cl = (4.0 * (double)rv) / n;
    const float r_cl3 = r_cl * r_cl * r_cl;
    dt_cl = 0.04 * std::sqrt((double)(r_cl3 * n));
    // get_core_radius (:108-143) about the current cod
    const double c0[3] = {cod.x, cod.y, cod.z};
    if (h4_mass_radii(h_, c0, M, &r_core, nullptr, nullptr) != H4_OK) return false;
    // get_half_mass_relaxation_time (:145-160)
    double c[3];
    if (h4_center_of_density(h_, c) != H4_OK) return false;
    cod.x = c[0]; cod.y = c[1]; cod.z = c[2];
    double half = 0.0;
    if (h4_mass_radii(h_, c, M, nullptr, &half, nullptr) != H4_OK) return false;
    const float r_h = half;
    r_hm = r_h;
    const float a = std::sqrt((double)((n * r_h * r_h * r_h) / (G * (M / (n)))));
    const float b = 1 / std::log(0.11 * n);
    t_rlx = (float)(0.138 * a * b);
    return true;
}

bool NbodyUtils::lagrange_radii() {
    if (ns->n < 8) return false;
    double c[3];
    if (h4_center_of_density(h_, c) != H4_OK) return false;
    cod.x = c[0]; cod.y = c[1]; cod.z = c[2];
    return h4_mass_radii(h_, c, ns->total_mass, nullptr, nullptr, layers_radii.data()) == H4_OK;
}

}  // namespace gb300
