// C entry point over the reference's own translation units (test infrastructure only).
//
// hmrref_conv_flux_source builds, for one patch, exactly the objects a HAMeRS run builds --
// the flow model (FlowModelSingleSpecies / FlowModelFourEqnConservative /
// FlowModelFiveEqnAllaire, with their ideal-gas mixing rules, basic utilities and Riemann
// solvers) and the WCNS56 convective flux reconstructor (ConvectiveFluxReconstructorWCNS5_JS,
// _WCNS6_LD, _WCNS5_Z or _WCNS6_CU_M2, all _HLLC_HLL) -- from the reference's unmodified
// sources, compiled against the SAMRAI stand-in in include/SAMRAI/shim_core.h, and calls
// ConvectiveFluxReconstructorWCNS56::computeConvectiveFluxAndSourceOnPatch
// (src/flow/convective_flux_reconstructors/WCNS56/ConvectiveFluxReconstructorWCNS56-HLLC-HLL.cpp:40).
// The objects are made the way ConvectiveFluxReconstructorManager.cpp:40-91 and
// FlowModelManager.cpp make them, from the same input-database keys.
//
// Arguments and array layout are those of hmro_conv_flux_source (oracle/hmr_oracle.cpp), so a
// test calls both with the same buffers:
//   Q      : ncomp arrays over the ghost box (ghost width 4, x fastest)
//   flux   : for axis a = 0..dim-1, neq arrays over n grown by one along a (overwritten, dt-scaled)
//   source : neq arrays over the interior (accumulated, as the reference does)
// Returns 0, or -1 with the reference's error text available from hmrref_last_error().
#include "flow/convective_flux_reconstructors/WCNS56/ConvectiveFluxReconstructorWCNS5-JS-HLLC-HLL.hpp"
#include "flow/convective_flux_reconstructors/WCNS56/ConvectiveFluxReconstructorWCNS5-Z-HLLC-HLL.hpp"
#include "flow/convective_flux_reconstructors/WCNS56/ConvectiveFluxReconstructorWCNS6-CU-M2-HLLC-HLL.hpp"
#include "flow/convective_flux_reconstructors/WCNS56/ConvectiveFluxReconstructorWCNS6-LD-HLLC-HLL.hpp"
#include "flow/flow_models/FlowModels.hpp"

#include <cstring>
#include <exception>
#include <string>
#include <vector>

namespace {

std::string g_last_error;

const int kGhosts = 4;   // ConvectiveFluxReconstructorWCNS56-HLLC-HLL.cpp:22

}  // namespace

extern "C" {

// Same field order as hmro_config (oracle/hmr_oracle.hpp).
struct hmrref_config {
    int model;   // 0 single species, 1 four-equation conservative, 2 five-equation Allaire
    int dim;
    int num_species;
    int scheme;  // 0 WCNS5-JS, 1 WCNS6-LD, 2 WCNS5-Z, 3 WCNS6-CU-M2
    double gamma[8];
    double R[8];
    int p;
    int q;
    double C;
    double alpha_tau;
    double Chi;
    double epsilon;
    double grid_dx[3];
};

const char* hmrref_last_error() { return g_last_error.c_str(); }
void hmrref_set_error(const char* what) { g_last_error = what; }

int hmrref_conv_flux_source(const hmrref_config* cfg, const int* n, const double* dx, double dt, const double* Q,
                            double* flux, double* source) {
    try {
        const tbox::Dimension dim((unsigned short)cfg->dim);
        const int D = cfg->dim;
        const int nsp = cfg->num_species;

        // Input databases with the keys of a HAMeRS input file.
        auto fm_db = HAMERS_MAKE_SHARED<tbox::Database>("Flow_model");
        fm_db->putString("equation_of_state", "IDEAL_GAS");
        auto eos_db = fm_db->putDatabase("Equation_of_state_mixing_rules");
        eos_db->putDoubleVector("species_gamma", std::vector<double>(cfg->gamma, cfg->gamma + nsp));
        eos_db->putDoubleVector("species_R", std::vector<double>(cfg->R, cfg->R + nsp));

        double gdx[3];
        for (int d = 0; d < 3; d++) gdx[d] = (cfg->grid_dx[d] > 0.0) ? cfg->grid_dx[d] : dx[d];
        auto grid_geometry = HAMERS_MAKE_SHARED<geom::CartesianGridGeometry>(dim, gdx, nullptr);

        HAMERS_SHARED_PTR<FlowModel> flow_model;
        FLOW_MODEL::TYPE type;
        if (cfg->model == 0) {
            type = FLOW_MODEL::SINGLE_SPECIES;
            flow_model = HAMERS_MAKE_SHARED<FlowModelSingleSpecies>("flow_model", "project", dim, grid_geometry,
                                                                    nsp, fm_db);
        } else if (cfg->model == 1) {
            type = FLOW_MODEL::FOUR_EQN_CONSERVATIVE;
            flow_model = HAMERS_MAKE_SHARED<FlowModelFourEqnConservative>("flow_model", "project", dim,
                                                                          grid_geometry, nsp, fm_db);
        } else if (cfg->model == 2) {
            type = FLOW_MODEL::FIVE_EQN_ALLAIRE;
            flow_model = HAMERS_MAKE_SHARED<FlowModelFiveEqnAllaire>("flow_model", "project", dim, grid_geometry,
                                                                     nsp, fm_db);
        } else {
            throw std::runtime_error("unknown flow model");
        }
        const int neq = flow_model->getNumberOfEquations();

        auto rec_db = HAMERS_MAKE_SHARED<tbox::Database>("Convective_flux_reconstructor");
        rec_db->putInteger("constant_p", cfg->p);
        rec_db->putInteger("constant_q", cfg->q);
        rec_db->putDouble("constant_C", cfg->C);
        rec_db->putDouble("constant_alpha_tau", cfg->alpha_tau);
        rec_db->putDouble("constant_Chi", cfg->Chi);
        rec_db->putDouble("constant_epsilon", cfg->epsilon);
        std::unique_ptr<ConvectiveFluxReconstructor> rec;
        if (cfg->scheme == 0)
            rec.reset(new ConvectiveFluxReconstructorWCNS5_JS_HLLC_HLL("rec", dim, grid_geometry, neq, type,
                                                                       flow_model, rec_db));
        else if (cfg->scheme == 1)
            rec.reset(new ConvectiveFluxReconstructorWCNS6_LD_HLLC_HLL("rec", dim, grid_geometry, neq, type,
                                                                       flow_model, rec_db));
        else if (cfg->scheme == 2)
            rec.reset(new ConvectiveFluxReconstructorWCNS5_Z_HLLC_HLL("rec", dim, grid_geometry, neq, type,
                                                                      flow_model, rec_db));
        else if (cfg->scheme == 3)
            rec.reset(new ConvectiveFluxReconstructorWCNS6_CU_M2_HLLC_HLL("rec", dim, grid_geometry, neq, type,
                                                                          flow_model, rec_db));
        else
            throw std::runtime_error("unknown scheme");

        // The patch: interior box [0, n-1], cell width dx, conservative variables on ghost width 4.
        hier::IntVector lo(dim, 0), hi(dim, 0);
        for (int d = 0; d < D; d++) hi[d] = n[d] - 1;
        const hier::Box box(lo, hi, hier::BlockId(0));
        double pdx[3] = {dx[0], D > 1 ? dx[1] : 1.0, D > 2 ? dx[2] : 1.0};
        auto patch_geom = HAMERS_MAKE_SHARED<geom::CartesianPatchGeometry>(pdx, nullptr);
        hier::Patch patch(box, patch_geom);
        auto ctx = HAMERS_MAKE_SHARED<hier::VariableContext>("CURRENT");

        const hier::IntVector ghosts(dim, kGhosts);
        const double* q = Q;
        for (auto& var : flow_model->getConservativeVariables()) {
            auto data = HAMERS_MAKE_SHARED<pdat::CellData<double>>(box, var->getDepth(), ghosts);
            const long nc = data->getGhostBox().size();
            for (int di = 0; di < var->getDepth(); di++) {
                std::memcpy(data->getPointer(di), q, sizeof(double) * (size_t)nc);
                q += nc;
            }
            patch.setPatchData(var, ctx, data);
        }

        auto flux_var = HAMERS_MAKE_SHARED<pdat::SideVariable<double>>(dim, "convective flux", neq);
        auto source_var = HAMERS_MAKE_SHARED<pdat::CellVariable<double>>(dim, "source", neq);
        auto flux_data = HAMERS_MAKE_SHARED<pdat::SideData<double>>(box, neq, hier::IntVector::getZero(dim));
        auto source_data = HAMERS_MAKE_SHARED<pdat::CellData<double>>(box, neq, hier::IntVector::getZero(dim));
        flux_data->fillAll(0.0);
        const long nint = box.size();
        for (int e = 0; e < neq; e++)
            std::memcpy(source_data->getPointer(e), source + (size_t)e * nint, sizeof(double) * (size_t)nint);
        patch.setPatchData(flux_var, ctx, flux_data);
        patch.setPatchData(source_var, ctx, source_data);

        rec->computeConvectiveFluxAndSourceOnPatch(patch, flux_var, source_var, ctx, 0.0, dt, 0);

        double* f = flux;
        for (int a = 0; a < D; a++) {
            const long nf = flux_data->getSideBox(a).size();
            for (int e = 0; e < neq; e++) {
                std::memcpy(f, flux_data->getPointer(a, e), sizeof(double) * (size_t)nf);
                f += nf;
            }
        }
        for (int e = 0; e < neq; e++)
            std::memcpy(source + (size_t)e * nint, source_data->getPointer(e), sizeof(double) * (size_t)nint);
        return 0;
    } catch (const std::exception& ex) {
        g_last_error = ex.what();
        return -1;
    }
}

}  // extern "C"
