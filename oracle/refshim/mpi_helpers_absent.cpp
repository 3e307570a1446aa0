// The monitoring-statistics utilities of the three flow models (compiled unmodified) refer to
// the reference's MPI reduction helpers, which walk a SAMRAI patch hierarchy this build does not
// have.  Monitoring statistics are not on the convective path; these definitions only satisfy
// the linker and refuse to run.
#include "flow/flow_models/MPI_helpers/FlowModelMPIHelperAverage.hpp"
#include "flow/flow_models/MPI_helpers/FlowModelMPIHelperMaxMin.hpp"

#include <stdexcept>

MPIHelper::MPIHelper(const std::string& name, const tbox::Dimension& dim,
                     const HAMERS_SHARED_PTR<geom::CartesianGridGeometry>& grid_geometry,
                     const HAMERS_SHARED_PTR<hier::PatchHierarchy>& hierarchy)
    : d_object_name(name), d_dim(dim), d_grid_geometry(grid_geometry), d_patch_hierarchy(hierarchy), d_mpi(tbox::SAMRAI_MPI::getSAMRAIWorld()),
      d_ratio_finest_level_to_coarsest_level(dim), d_coarsest_level_dims(dim), d_finest_level_dims(dim) {
    throw std::runtime_error("MPI helpers are not part of this build");
}

double FlowModelMPIHelperAverage::getAveragedQuantity(const std::vector<std::string>&, const std::vector<int>&,
                                                      const HAMERS_SHARED_PTR<hier::VariableContext>&) {
    throw std::runtime_error("MPI helpers are not part of this build");
}

double FlowModelMPIHelperMaxMin::getMaxQuantity(const std::vector<std::string>&, const std::vector<int>&,
                                                const std::vector<bool>&,
                                                const HAMERS_SHARED_PTR<hier::VariableContext>&) {
    throw std::runtime_error("MPI helpers are not part of this build");
}
