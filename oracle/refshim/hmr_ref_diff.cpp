// C entry point over the reference's own diffusive-flux translation units (test infrastructure only).
//
// hmrref_diff_flux builds, for one single-species patch, the objects a HAMeRS NavierStokes run
// builds for its diffusive flux -- FlowModelSingleSpecies with CONSTANT shear and bulk viscosity
// and the PRANDTL thermal conductivity (FlowModelSingleSpecies.cpp:160-380 reads exactly these
// keys), and DiffusiveFluxReconstructorMidpointSecondOrder / _FourthOrder / _SixthOrder, made as
// DiffusiveFluxReconstructorManager.cpp:14-50 makes them -- from the reference's unmodified
// sources compiled against the SAMRAI stand-in, and calls
// DiffusiveFluxReconstructorMidpoint::computeDiffusiveFluxOnPatch
// (src/flow/diffusive_flux_reconstructors/midpoint/DiffusiveFluxReconstructorMidpoint.cpp:38).
//
// Layout as hmro_diff_flux (oracle/hmr_oracle.cpp):
//   Q    : ncomp arrays over the ghost box of width `ghosts` (x fastest); the reconstructor needs
//          1, 3 or 5 ghosts for orders 2, 4, 6
//   flux : for axis a = 0..dim-1, neq arrays over n grown by one along a (overwritten, dt-scaled)
// Returns 0, or -1 with the reference's error text available from hmrref_last_error().
#include "flow/diffusive_flux_reconstructors/DiffusiveFluxReconstructors.hpp"
#include "flow/flow_models/FlowModels.hpp"

#include <cstring>
#include <exception>
#include <string>
#include <vector>

extern "C" {

struct hmrref_config;   // hmr_ref.cpp; only the fields below are read here
void hmrref_set_error(const char* what);

// The leading fields of hmrref_config (same order as hmro_config).
struct hmrref_config_head {
    int model;
    int dim;
    int num_species;
    int scheme;
    double gamma[8];
    double R[8];
};

// Same field order as hmro_transport (oracle/hmr_oracle.hpp).
struct hmrref_transport {
    int order;        // 2, 4 or 6: MIDPOINT_SECOND_ORDER / _FOURTH_ORDER / _SIXTH_ORDER
    double mu;        // Equation_of_shear_viscosity_mixing_rules.species_mu
    double mu_v;      // Equation_of_bulk_viscosity_mixing_rules.species_mu_v
    double c_p, Pr;   // Equation_of_thermal_conductivity_mixing_rules.species_c_p, species_Pr
    double mu_kappa;  // ... and that model's own species_mu
};

int hmrref_diff_flux(const hmrref_config* cfg_opaque, const hmrref_transport* tr, const int* n, int ghosts,
                     const double* dx, double dt, const double* Q, double* flux) {
    try {
        const hmrref_config_head* cfg = reinterpret_cast<const hmrref_config_head*>(cfg_opaque);
        if (cfg->model != 0) throw std::runtime_error("diffusive flux: single-species model only");
        const tbox::Dimension dim((unsigned short)cfg->dim);
        const int D = cfg->dim;

        auto fm_db = HAMERS_MAKE_SHARED<tbox::Database>("Flow_model");
        fm_db->putString("equation_of_state", "IDEAL_GAS");
        auto eos_db = fm_db->putDatabase("Equation_of_state_mixing_rules");
        eos_db->putDoubleVector("species_gamma", std::vector<double>(1, cfg->gamma[0]));
        eos_db->putDoubleVector("species_R", std::vector<double>(1, cfg->R[0]));
        fm_db->putString("equation_of_shear_viscosity", "CONSTANT");
        auto mu_db = fm_db->putDatabase("Equation_of_shear_viscosity_mixing_rules");
        mu_db->putDoubleVector("species_mu", std::vector<double>(1, tr->mu));
        mu_db->putDoubleVector("species_M", std::vector<double>(1, 1.0));
        fm_db->putString("equation_of_bulk_viscosity", "CONSTANT");
        auto mv_db = fm_db->putDatabase("Equation_of_bulk_viscosity_mixing_rules");
        mv_db->putDoubleVector("species_mu_v", std::vector<double>(1, tr->mu_v));
        mv_db->putDoubleVector("species_M", std::vector<double>(1, 1.0));
        fm_db->putString("equation_of_thermal_conductivity", "PRANDTL");
        auto k_db = fm_db->putDatabase("Equation_of_thermal_conductivity_mixing_rules");
        k_db->putDoubleVector("species_c_p", std::vector<double>(1, tr->c_p));
        k_db->putDoubleVector("species_Pr", std::vector<double>(1, tr->Pr));
        k_db->putDoubleVector("species_M", std::vector<double>(1, 1.0));
        k_db->putString("equation_of_shear_viscosity", "CONSTANT");
        k_db->putDoubleVector("species_mu", std::vector<double>(1, tr->mu_kappa));

        double gdx[3] = {dx[0], D > 1 ? dx[1] : 1.0, D > 2 ? dx[2] : 1.0};
        auto grid_geometry = HAMERS_MAKE_SHARED<geom::CartesianGridGeometry>(dim, gdx, nullptr);
        HAMERS_SHARED_PTR<FlowModel> flow_model =
            HAMERS_MAKE_SHARED<FlowModelSingleSpecies>("flow_model", "project", dim, grid_geometry, 1, fm_db);
        const int neq = flow_model->getNumberOfEquations();

        auto rec_db = HAMERS_MAKE_SHARED<tbox::Database>("Diffusive_flux_reconstructor");
        std::unique_ptr<DiffusiveFluxReconstructor> rec;
        if (tr->order == 2)
            rec.reset(new DiffusiveFluxReconstructorMidpointSecondOrder("rec", dim, grid_geometry, neq, flow_model,
                                                                        rec_db));
        else if (tr->order == 4)
            rec.reset(new DiffusiveFluxReconstructorMidpointFourthOrder("rec", dim, grid_geometry, neq, flow_model,
                                                                        rec_db));
        else if (tr->order == 6)
            rec.reset(new DiffusiveFluxReconstructorMidpointSixthOrder("rec", dim, grid_geometry, neq, flow_model,
                                                                       rec_db));
        else
            throw std::runtime_error("diffusive flux: order must be 2, 4 or 6");

        hier::IntVector lo(dim, 0), hi(dim, 0);
        for (int d = 0; d < D; d++) hi[d] = n[d] - 1;
        const hier::Box box(lo, hi, hier::BlockId(0));
        auto patch_geom = HAMERS_MAKE_SHARED<geom::CartesianPatchGeometry>(gdx, nullptr);
        hier::Patch patch(box, patch_geom);
        auto ctx = HAMERS_MAKE_SHARED<hier::VariableContext>("CURRENT");

        const hier::IntVector gw(dim, ghosts);
        const double* q = Q;
        for (auto& var : flow_model->getConservativeVariables()) {
            auto data = HAMERS_MAKE_SHARED<pdat::CellData<double>>(box, var->getDepth(), gw);
            const long nc = data->getGhostBox().size();
            for (int di = 0; di < var->getDepth(); di++) {
                std::memcpy(data->getPointer(di), q, sizeof(double) * (size_t)nc);
                q += nc;
            }
            patch.setPatchData(var, ctx, data);
        }

        auto flux_var = HAMERS_MAKE_SHARED<pdat::SideVariable<double>>(dim, "diffusive flux", neq);
        auto flux_data = HAMERS_MAKE_SHARED<pdat::SideData<double>>(box, neq, hier::IntVector::getZero(dim));
        flux_data->fillAll(0.0);
        patch.setPatchData(flux_var, ctx, flux_data);

        rec->computeDiffusiveFluxOnPatch(patch, flux_var, ctx, 0.0, dt, 0);

        double* f = flux;
        for (int a = 0; a < D; a++) {
            const long nf = flux_data->getSideBox(a).size();
            for (int e = 0; e < neq; e++) {
                std::memcpy(f, flux_data->getPointer(a, e), sizeof(double) * (size_t)nf);
                f += nf;
            }
        }
        return 0;
    } catch (const std::exception& ex) {
        hmrref_set_error(ex.what());
        return -1;
    }
}

}  // extern "C"
