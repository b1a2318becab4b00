// Cluster diagnostics of the reference's NbodyUtils
// (src/include/utils/NbodyUtils.hpp:48-88, NbodyUtils.cpp:59-328) over the
// device state: center of density and mass radii come from the C ABI
// (h4_center_of_density, h4_mass_radii), the scalar formulas are evaluated
// here with the reference's float/double types.
#ifndef GRAVIDY_GB300_HOST_NBODYUTILS_HPP
#define GRAVIDY_GB300_HOST_NBODYUTILS_HPP

#include <vector>

#include "NbodySystem.hpp"

namespace gb300 {

class NbodyUtils {
  public:
    NbodyUtils(NbodySystem *ns, h4_handle h);

    NbodySystem *ns;
    double3 cod;                        // NbodyUtils::cod (starts at 0)
    std::vector<double> layers_radii;   // 6 Lagrange radii
    double r_virial, t_cr, r_cl, dt_cl, r_core, t_rlx, r_hm;

    // NbodyUtils::nbody_attributes (:59-78), e_ini = the initial energy.
    bool nbody_attributes(double e_ini);
    // NbodyUtils::lagrange_radii (:246-263).
    bool lagrange_radii();

  private:
    h4_handle h_;
};

}  // namespace gb300
#endif
