// C entry point over the reference's own physical-boundary fills (test infrastructure only).
//
// hmrref_fill_boundaries fills the ghost cells of one patch that covers the whole domain, with a
// FLOW (extrapolation) or REFLECT (slip wall) condition on both sides of every axis, the way
// EulerBoundaryConditions::setPhysicalBoundaryConditions (src/apps/Euler/EulerBoundaryConditions.cpp:
// 836-1100) does it: the flow model's conservative variables of type SCALAR take SYMMETRY where
// the master condition is REFLECT and the VECTOR one (the momentum) REFLECT (:205-297); the
// reference's BasicCartesianBoundaryUtilities2 / 3 (compiled unmodified from
// src/util/basic_boundary_conditions/) fill the edges and then the nodes in 2D, the faces, the
// edges and then the nodes in 3D.  A corner (2D node, 3D edge or node) needs one condition of the
// X/Y/Z-prefixed kind naming one of its axes; corner_axis picks which of its walls (the lowest
// axis index >= corner_axis among them, else the lowest).
//
// hmrref_fill_boundaries_bv also takes DIRICHLET sides (mode 4) with their conservative values
// bvals[(2 axis + high) ncomp + e], handed to the reference's routines per variable as
// EulerBoundaryConditions holds them (d_bdry_edge/face_conservative_var, :638-723); a corner with a
// Dirichlet side takes the condition naming the lowest such axis (XDIRICHLET before YDIRICHLET).
//
// Layout as hmro_fill_ghosts (oracle/hmr_oracle.cpp): ncomp arrays over the ghost box of width
// 4, x fastest, filled in place.  mode per axis: 0 FLOW, 3 REFLECT, 5 SYMMETRY (every variable
// mirrored as it is) (4 DIRICHLET with values).
// Returns 0, or -1 with the reference's error text available from hmrref_last_error().
#include "flow/flow_models/FlowModels.hpp"
#include "util/basic_boundary_conditions/BasicBoundaryConditions.hpp"
#include "util/basic_boundary_conditions/BasicCartesianBoundaryUtilities2.hpp"
#include "util/basic_boundary_conditions/BasicCartesianBoundaryUtilities3.hpp"

#include <cstring>
#include <exception>
#include <string>
#include <vector>

extern "C" {

struct hmrref_config;
void hmrref_set_error(const char* what);

struct hmrref_config_head {
    int model;
    int dim;
    int num_species;
    int scheme;
    double gamma[8];
    double R[8];
};

}  // extern "C"

namespace {

using namespace BDRY_COND::BASIC;

int axis_cond(int axis, int mode) {
    static const int flow[3] = {XFLOW, YFLOW, ZFLOW};
    static const int refl[3] = {XREFLECT, YREFLECT, ZREFLECT};
    static const int diri[3] = {XDIRICHLET, YDIRICHLET, ZDIRICHLET};
    static const int symm[3] = {XSYMMETRY, YSYMMETRY, ZSYMMETRY};
    if (mode == 5) return symm[axis];
    return mode == 4 ? diri[axis] : (mode == 3 ? refl[axis] : flow[axis]);
}

// X/Y/Z-prefixed condition of a corner whose outward axes are `axes`.
int corner_cond(const std::vector<int>& axes, const int* mode, int corner_axis) {
    for (int a : axes)
        if (mode[a] == 4) return axis_cond(a, 4);
    int pick = axes[0];
    for (int a : axes)
        if (a >= corner_axis) { pick = a; break; }
    return axis_cond(pick, mode[pick]);
}

int scalar_of(int c) {
    if (c == REFLECT) return SYMMETRY;
    if (c == XREFLECT) return XSYMMETRY;
    if (c == YREFLECT) return YSYMMETRY;
    if (c == ZREFLECT) return ZSYMMETRY;
    return c;
}

}  // namespace

extern "C" int hmrref_fill_boundaries_bv(const hmrref_config* cfg_opaque, const int* n, const int* mode,
                                         int corner_axis, const double* bvals, double* Q) {
    try {
        const hmrref_config_head* cfg = reinterpret_cast<const hmrref_config_head*>(cfg_opaque);
        const int D = cfg->dim;
        const tbox::Dimension dim((unsigned short)D);
        const int nsp = cfg->num_species;
        for (int a = 0; a < D; a++) {
            if (mode[a] != 0 && mode[a] != 3 && mode[a] != 4 && mode[a] != 5)
                throw std::runtime_error("boundary mode must be 0 (FLOW), 3 (REFLECT), 4 (DIRICHLET) or 5 (SYMMETRY)");
            if (mode[a] == 4 && !bvals) throw std::runtime_error("DIRICHLET sides need values");
        }

        auto fm_db = HAMERS_MAKE_SHARED<tbox::Database>("Flow_model");
        fm_db->putString("equation_of_state", "IDEAL_GAS");
        auto eos_db = fm_db->putDatabase("Equation_of_state_mixing_rules");
        eos_db->putDoubleVector("species_gamma", std::vector<double>(cfg->gamma, cfg->gamma + nsp));
        eos_db->putDoubleVector("species_R", std::vector<double>(cfg->R, cfg->R + nsp));
        double dx[3] = {1.0, 1.0, 1.0};
        auto grid_geometry = HAMERS_MAKE_SHARED<geom::CartesianGridGeometry>(dim, dx, nullptr);
        HAMERS_SHARED_PTR<FlowModel> flow_model;
        if (cfg->model == 0)
            flow_model = HAMERS_MAKE_SHARED<FlowModelSingleSpecies>("fm", "project", dim, grid_geometry, nsp, fm_db);
        else if (cfg->model == 1)
            flow_model = HAMERS_MAKE_SHARED<FlowModelFourEqnConservative>("fm", "project", dim, grid_geometry, nsp, fm_db);
        else if (cfg->model == 2)
            flow_model = HAMERS_MAKE_SHARED<FlowModelFiveEqnAllaire>("fm", "project", dim, grid_geometry, nsp, fm_db);
        else
            throw std::runtime_error("unknown flow model");

        // The patch covers the domain [0, n-1]; its boundary boxes by codimension.
        hier::IntVector lo(dim, 0), hi(dim, 0);
        for (int d = 0; d < D; d++) hi[d] = n[d] - 1;
        const hier::Box box(lo, hi, hier::BlockId(0));
        auto patch_geom = HAMERS_MAKE_SHARED<geom::CartesianPatchGeometry>(dx, nullptr);
        std::vector<hier::BoundaryBox> bb[4];
        std::vector<std::vector<int>> outward[4];   // per box: its outward axes
        const int ncorner = D == 2 ? 9 : 27;
        for (int code = 0; code < ncorner; code++) {
            int side[3] = {0, 0, 0};   // -1 low, 0 inside, 1 high
            int c = code;
            for (int d = 0; d < D; d++) { side[d] = c % 3 - 1; c /= 3; }
            std::vector<int> axes;
            hier::IntVector blo(dim, 0), bhi(dim, 0);
            for (int d = 0; d < D; d++) {
                if (side[d] == 0) { blo[d] = 0; bhi[d] = n[d] - 1; continue; }
                axes.push_back(d);
                blo[d] = bhi[d] = side[d] < 0 ? -1 : n[d];
            }
            const int codim = (int)axes.size();
            if (codim == 0) continue;
            int loc;
            if (codim == 1) {
                loc = 2 * axes[0] + (side[axes[0]] > 0);
            } else if (D == 2 || codim == 3) {
                loc = (side[0] > 0) + 2 * (side[1] > 0) + (D == 3 ? 4 * (side[2] > 0) : 0);
            } else {   // 3D edges: parallel to z, then y, then x
                const int s0 = side[axes[0]] > 0, s1 = side[axes[1]] > 0;
                if (axes[0] == 0 && axes[1] == 1) loc = s0 + 2 * s1;
                else if (axes[0] == 0 && axes[1] == 2) loc = 4 + s0 + 2 * s1;
                else loc = 8 + s0 + 2 * s1;
            }
            bb[codim].emplace_back(hier::Box(blo, bhi, hier::BlockId(0)), codim, loc);
            outward[codim].push_back(axes);
        }
        for (int k = 1; k <= D; k++) patch_geom->setCodimensionBoundaries(k, bb[k]);
        hier::Patch patch(box, patch_geom);
        auto ctx = HAMERS_MAKE_SHARED<hier::VariableContext>("CURRENT");

        // Conditions by location, as EulerBoundaryConditions holds them.
        const int nside = 2 * D;
        std::vector<int> side_conds(nside);
        for (int l = 0; l < nside; l++)
            side_conds[l] = mode[l / 2] == 5 ? SYMMETRY : (mode[l / 2] == 4 ? DIRICHLET : (mode[l / 2] == 3 ? REFLECT : FLOW));
        std::vector<int> edge_conds(D == 3 ? 12 : 4, FLOW), node_conds(D == 3 ? 8 : 4, FLOW);
        std::vector<int>& c2 = D == 2 ? node_conds : edge_conds;
        for (size_t i = 0; i < bb[2].size(); i++) c2[bb[2][i].getLocationIndex()] = corner_cond(outward[2][i], mode, corner_axis);
        if (D == 3)
            for (size_t i = 0; i < bb[3].size(); i++)
                node_conds[bb[3][i].getLocationIndex()] = corner_cond(outward[3][i], mode, corner_axis);
        auto scalarise = [](std::vector<int> v) {
            for (int& c : v) c = scalar_of(c);
            return v;
        };

        const hier::IntVector ghosts(dim, 4);
        std::vector<HAMERS_SHARED_PTR<pdat::CellData<double>>> data;
        double* q = Q;
        for (auto& var : flow_model->getConservativeVariables()) {
            auto d = HAMERS_MAKE_SHARED<pdat::CellData<double>>(box, var->getDepth(), ghosts);
            const long nc = d->getGhostBox().size();
            for (int di = 0; di < var->getDepth(); di++) {
                std::memcpy(d->getPointer(di), q, sizeof(double) * (size_t)nc);
                q += nc;
            }
            data.push_back(d);
        }
        const std::vector<std::string> types = flow_model->getVariableTypesOfConservativeVariables();
        const std::vector<std::string> names = flow_model->getNamesOfConservativeVariables();
        const hier::IntVector gcw = -hier::IntVector::getOne(dim);
        std::vector<int> all_sides, all_edges, all_nodes;
        for (int l = 0; l < nside; l++) all_sides.push_back(l);
        for (int l = 0; l < (D == 3 ? 12 : 4); l++) all_edges.push_back(l);
        for (int l = 0; l < (D == 3 ? 8 : 4); l++) all_nodes.push_back(l);
        int ncomp = 0;
        for (auto& d : data) ncomp += d->getDepth();
        int off = 0;   // first component of variable vi
        for (size_t vi = 0; vi < data.size(); vi++) {
            const bool vec = types[vi] == "VECTOR";
            const std::vector<int> sc = vec ? side_conds : scalarise(side_conds);
            const std::vector<int> ec = vec ? edge_conds : scalarise(edge_conds);
            const std::vector<int> nc = vec ? node_conds : scalarise(node_conds);
            // this variable's boundary values by side location, as d_bdry_edge/face_conservative_var
            const int depth = data[vi]->getDepth();
            std::vector<double> vals((size_t)nside * depth, 0.0);
            if (bvals)
                for (int l = 0; l < nside; l++)
                    for (int di = 0; di < depth; di++) vals[(size_t)l * depth + di] = bvals[l * ncomp + off + di];
            if (D == 2) {
                BasicCartesianBoundaryUtilities2::fillEdgeBoundaryData(names[vi], data[vi], patch, all_sides, sc, vals, gcw);
                BasicCartesianBoundaryUtilities2::fillNodeBoundaryData(names[vi], data[vi], patch, all_nodes, nc, vals, gcw);
            } else {
                BasicCartesianBoundaryUtilities3::fillFaceBoundaryData(names[vi], data[vi], patch, all_sides, sc, vals, gcw);
                BasicCartesianBoundaryUtilities3::fillEdgeBoundaryData(names[vi], data[vi], patch, all_edges, ec, vals, gcw);
                BasicCartesianBoundaryUtilities3::fillNodeBoundaryData(names[vi], data[vi], patch, all_nodes, nc, vals, gcw);
            }
            off += depth;
        }
        q = Q;
        for (auto& d : data) {
            const long ncell = d->getGhostBox().size();
            for (int di = 0; di < d->getDepth(); di++) {
                std::memcpy(q, d->getPointer(di), sizeof(double) * (size_t)ncell);
                q += ncell;
            }
        }
        return 0;
    } catch (const std::exception& ex) {
        hmrref_set_error(ex.what());
        return -1;
    }
}

extern "C" int hmrref_fill_boundaries(const hmrref_config* cfg, const int* n, const int* mode, int corner_axis,
                                      double* Q) {
    return hmrref_fill_boundaries_bv(cfg, n, mode, corner_axis, nullptr, Q);
}
