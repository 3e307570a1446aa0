// Stand-in for the reference's RungeKuttaLevelIntegrator class (SAMRAI hierarchy integrator):
// the flow models only register their conservative variables with it, which one patch does not
// need.  Shadows include/algs/integrator/RungeKuttaLevelIntegrator.hpp, whose SAMRAI algorithm
// dependencies this build does not provide.
#ifndef RUNGE_KUTTA_LEVEL_INTEGRATOR_HPP
#define RUNGE_KUTTA_LEVEL_INTEGRATOR_HPP

#include "HAMeRS_config.hpp"
#include "HAMeRS_memory.hpp"

#include "SAMRAI/shim_core.h"

#include <string>

using namespace SAMRAI;

class RungeKuttaLevelIntegrator {
public:
    enum RK_VAR_TYPE { TIME_DEP = 0, INPUT = 1, NO_FILL = 2, FLUX = 3, TEMPORARY = 4 };

    void registerVariable(const HAMERS_SHARED_PTR<hier::Variable>&, const hier::IntVector&,
                          const hier::IntVector&, const RK_VAR_TYPE&,
                          const HAMERS_SHARED_PTR<geom::CartesianGridGeometry>&,
                          const std::string& = "", const std::string& = "") {}
};

#endif
