// Host-side launch interface between the C ABI (hmr_abi.cu) and the kernel
// translation units.  hmr_faces.cu is compiled twice: once in the exact form
// (namespace hmr_exact, --fmad=false) and once in the fast form (namespace
// hmr_fast).  hmr_cells.cu (cell data, sensor, ghost fill, elementwise RK
// stage) is always exact so both forms see identical sensor inputs.
#pragma once

#include <cuda_runtime.h>

#include "hmr.h"
#include "hmr_kernels.cuh"
#include "hmr_vjp_items.cuh"

namespace hmr {

// Species constants of Params from species_gamma / species_R, as the
// ideal-gas mixing rules derive them (EquationOfStateMixingRulesIdealGas.cpp:107-120).
inline void species_params(const double* gamma, const double* R, int nsp, Params& P) {
    for (int s = 0; s < MAX_SPECIES; s++) {
        P.gamma[s] = s < nsp ? gamma[s] : 1.4;
        const double Rs = s < nsp ? R[s] : 1.0;
        P.inv_gm1[s] = double(1)/(P.gamma[s] - double(1));
        P.cp[s] = P.gamma[s]/(P.gamma[s] - double(1))*Rs;
        P.cv[s] = double(1)/(P.gamma[s] - double(1))*Rs;
    }
}

inline bool reconstructor_known(int r) {
    return r == HMR_WCNS5_JS_HLLC_HLL || r == HMR_WCNS6_LD_HLLC_HLL || r == HMR_WCNS5_Z_HLLC_HLL ||
           r == HMR_WCNS6_CU_M2_HLLC_HLL;
}

// Node-to-midpoint interpolation of a cell value (…MidpointSecondOrder.cpp, …FourthOrder.cpp
// interpolateDataFromNodeToMidpoint), in the reference's operation order; host code is built
// with -ffp-contract=off so that the products are not fused into the sums.
inline double host_mid_value(int order, double LL, double L, double R, double RR) {
    if (order == 2) return double(1)/double(2)*(R + L);
    return double(9)/double(16)*(R + L) + -double(1)/double(16)*(RR + LL);
}
// The sixth-order node -> midpoint value of a constant (…MidpointSixthOrder.cpp:962-1000).
inline double host_mid_value6(double v) {
    return (double(75)/double(128)*(v + v) + -double(25)/double(256)*(v + v) + double(3)/double(256)*(v + v));
}

// Navier-Stokes constants of Params (single species): the side values of the constant
// transport properties, interpolated from cells as every side variable is, and the
// combinations D0, D1 of FlowModelDiffusiveFluxUtilitiesSingleSpecies.cpp:2471-2799 use.
inline int diffusive_params(const hmr_config* cfg, Params& P) {
    const int order = cfg->diffusive_flux_reconstructor;
    P.dorder = 0;
    P.dS43 = P.dS23 = P.dmu = P.dkappa = P.dTc = 0.0;
    P.cmu = P.cmu_v = P.ckappa = 0.0;
    if (order == HMR_DIFFUSIVE_NONE) return HMR_OK;
    if (order != HMR_MIDPOINT_SECOND_ORDER && order != HMR_MIDPOINT_FOURTH_ORDER &&
        order != HMR_MIDPOINT_SIXTH_ORDER)
        return HMR_ERR_UNSUPPORTED;
    if (cfg->flow_model != HMR_SINGLE_SPECIES) return HMR_ERR_UNSUPPORTED;
    if (!(cfg->species_mu >= 0.0) || !(cfg->species_mu_v >= 0.0) || !(cfg->species_c_p >= 0.0) ||
        !(cfg->species_Pr > 0.0) || !(cfg->species_mu_kappa >= 0.0) || !(cfg->species_gamma[0] > 1.0))
        return HMR_ERR_ARGUMENT;
    const double mu = cfg->species_mu, mu_v = cfg->species_mu_v;
    const double kappa = cfg->species_c_p*cfg->species_mu_kappa/cfg->species_Pr;   // Prandtl.cpp:63
    auto side = [order](double v) { return order == 6 ? host_mid_value6(v) : host_mid_value(order, v, v, v, v); };
    const double mu_s = side(mu);
    const double mu_v_s = side(mu_v);
    P.dorder = order;
    P.cmu = mu;
    P.cmu_v = mu_v;
    P.ckappa = kappa;
    P.dmu = mu_s;
    P.dkappa = side(kappa);
    P.dS43 = double(4)/double(3)*mu_s + mu_v_s;
    P.dS23 = double(2)/double(3)*mu_s - mu_v_s;
    const double gamma = cfg->species_gamma[0];
    const double c_v = double(1)/(gamma - double(1))*cfg->species_R[0];   // MixingRulesIdealGas.cpp:116-120
    P.dTc = (gamma - double(1))*c_v;
    return HMR_OK;
}

// Scheme constants of Params from a configuration whose reconstructor is known:
// p, q, C, alpha_tau, and WCNS6-CU-M2's epsilon dx^2 and Chi dx^2 per axis, each
// evaluated as the reference writes it (epsilon*dx*dx, left to right) from the
// grid geometry's spacing, and the Navier-Stokes constants.  Returns HMR_ERR_ARGUMENT for
// constants out of range, HMR_ERR_UNSUPPORTED for a diffusive flux the context cannot compute.
inline int scheme_params(const hmr_config* cfg, Params& P) {
    if (cfg->constant_p < 1 || cfg->constant_p > 8 || cfg->constant_q < 1 || cfg->constant_q > 8)
        return HMR_ERR_ARGUMENT;
    P.p = cfg->constant_p;
    P.q = cfg->constant_q;
    P.C = cfg->constant_C;
    P.alpha_tau = cfg->constant_alpha_tau;
    for (int d = 0; d < 3; d++) P.cu_e[d] = P.cu_x[d] = 0.0;
    if (cfg->convective_flux_reconstructor == HMR_WCNS6_CU_M2_HLLC_HLL) {
        if (!(cfg->constant_Chi >= 0.0) || !(cfg->constant_epsilon >= 0.0)) return HMR_ERR_ARGUMENT;
        for (int d = 0; d < cfg->dim && d < 3; d++) {
            const double dx = cfg->grid_dx[d];
            if (!(dx > 0.0)) return HMR_ERR_ARGUMENT;
            P.cu_e[d] = cfg->constant_epsilon*dx*dx;
            P.cu_x[d] = cfg->constant_Chi*dx*dx;
        }
    }
    return diffusive_params(cfg, P);
}

// A fine patch over a coarse patch of the next coarser level: geometries, first interior
// cells in the level index spaces, ratio, and the covered coarse cells [lo, hi) (local).
struct CoarsenArgs {
    Geom gc, gf;
    int clo[3], flo[3], r[3];
    int lo[3], hi[3];
};

struct Variant {
    int dim;
    int model;
    int nsp;
    int scheme;
    int dorder = 0;   // NavierStokes midpoint diffusive flux order (0: Euler)
};

inline int variant_neq(const Variant& v) {
    if (v.model == SINGLE_SPECIES) return v.dim + 2;
    if (v.model == FOUR_EQN_CONSERVATIVE) return v.nsp + v.dim + 1;
    return v.dim + 2 * v.nsp;
}

// Items of each phase of one patch's substep VJP (VjpWork phases; face phases per axis).
inline void vjp_item_counts(const Variant& v, const Geom& g, long* n) {
    for (int k = 0; k < VJP_NPH * 3; k++) n[k] = 0;
    const int neq = variant_neq(v);
    for (int a = 0; a < v.dim; a++) {
        const long nf = nface_of(g, a);
        n[VJP_PH_PROJ * 3 + a] = n[VJP_PH_RIEM * 3 + a] = n[VJP_PH_CHAR * 3 + a] = nf;
        n[VJP_PH_FWD * 3 + a] = n[VJP_PH_BWDW * 3 + a] = nf * neq;
        if (v.dorder) n[VJP_PH_DMID * 3 + a] = nface_w(g, a, v.dorder == 6 ? 2 : 1);
    }
    if (v.dorder) n[VJP_PH_DGD * 3] = n[VJP_PH_DCELL * 3] = ncell_of(g);
    n[VJP_PH_CELLB * 3] = ncell_of(g);
}

// One entry of the batched worklist: a patch with its stage states.
struct PatchWork {
    Geom g;
    Scratch S;
    Comp Q[3];        // stage states (ghost box)
    Comp Qout;        // output of the substep
    int periodic[3];  // own ghost fill per axis (hmr_fill_mode) when the level has no layout
    int lo[3];        // first interior cell in the level's index space (layout set)
    long off_fill;    // prefix offsets of the item counts, per phase
    long off_cells;
    long off_sensor;
    long off_face[3];
    long off_dface[3];   // diffusive midpoints (faces -W .. n + W; W = 2 at sixth order, else 1)
    long off_update;
};

// One box of ghost cells of patch dst copied from the interior of patch src (possibly a
// periodic image): dst-local start dlo, src-local start slo, extent ext; off = prefix
// offset of its cells in the flat copy index space.
struct GhostCopy {
    int dst, src;
    int dlo[3], slo[3], ext[3];
    long off;
};

struct LevelArgs {
    const PatchWork* work;   // device array
    int npatch;
    int ncomp;
    long total_fill, total_cells, total_sensor, total_face[3], total_update;
    long total_dface[3];
    double alpha[3];
    int nst;
    double beta;
    double dt;
    unsigned int* barrier;   // device counter for the grid barrier (zeroed before launch)
    int* status;             // device error flag (barrier give-up)
    unsigned long long timeout_ns;   // bound of every barrier wait
    unsigned int barrier_extra;      // diagnostic: arrivals that never come (0 in normal use)
    Redo redo;                       // faces handed from the fast to the exact form (count zeroed per launch)
    unsigned int* chunk;             // counters of the chunks each phase has handed out (zeroed per launch)
    const double* dt_dev;            // when set, the time step is read from this device value instead of dt
    // ghost exchange between the patches of the level (hmr_level_set_layout): copies from
    // neighbours and periodic images, then zero-gradient at the domain's non-periodic faces
    int exchange;
    const GhostCopy* copies;         // device array
    int ncopy;
    long total_copy;
    int dom[3];                      // domain extent in cells
    int dom_periodic[3];             // per axis: 1 periodic, 0 zero-gradient, 3 reflecting wall or 4 Dirichlet faces
    int mom0;                        // first momentum component (the normal one flips at a reflecting wall)
    const double* bvals;             // device [6][ncomp]: the Dirichlet values per side (2 axis + high)
    // work splitting (autotuned; results do not depend on it): phase chunks of chunk_mult
    // block widths; split_mode bit 0 hands the cell-wise phases out by a fixed grid stride,
    // bit 1 (fast form) sorts the faces by their sensor before the face phase
    int chunk_mult;
    int split_mode;
    // sorted faces: per axis a the level's face items taking HLLC at sorted + sort_off[a]
    // (sort_count[a] of them); sort_count[3] HLLC-HLL faces at the head of the redo queue
    unsigned long long* sorted;
    long sort_off[3];
    unsigned int* sort_count;
};

}  // namespace hmr

namespace hmr_cells {
int launch_cells(const hmr::Variant& v, const hmr::Params& P, const hmr::Geom& g, const hmr::Comp& Q,
                 const hmr::Scratch& S, cudaStream_t st);
int launch_sensor(const hmr::Variant& v, const hmr::Geom& g, const hmr::Scratch& S, cudaStream_t st);
// Ghost fill of one patch per axis (hmr_fill_mode); mom0: the first momentum component, whose
// normal one a reflecting wall negates; bv: device [6][ncomp] values of Dirichlet sides.
int launch_fill(int dim, const hmr::Geom& g, const hmr::Comp& Q, int ncomp, const int* periodic, int mom0,
                const double* bv, cudaStream_t st);
int launch_fill_vjp(int dim, const hmr::Geom& g, const hmr::Comp& Qb, int ncomp, const int* periodic, int mom0,
                    cudaStream_t st);
// Adjoint of the level's ghost fill with a layout (the exchange between patches, then the domain's
// physical faces): the physical ghost cells first add their adjoints to the in-domain cells they
// were copied from (negated normal momentum at reflecting walls; Dirichlet ghost cells copy no
// cell and are only zeroed), then the exchanged ghost cells
// to the patch interiors they were copied from; both are zeroed.  Ghost cells no copy wrote keep
// theirs.  Sums of several ghost cells into one source cell are atomic.
struct LevelFillVjpPatch {
    hmr::Geom g;
    hmr::Comp Qb;   // adjoint arrays of the patch (ghost box)
    int lo[3];      // first interior cell in the level's index space
    long off;       // prefix offset of its ghost-box cells
};
int launch_level_fill_vjp(int dim, const LevelFillVjpPatch* d_patches, int npatch, long total_cells,
                          const hmr::GhostCopy* d_copies, int ncopy, long total_copy, int ncomp, const int* dom,
                          const int* dom_periodic, int mom0, cudaStream_t st);
// Stable time step (Euler::computeSpectralRadiusesAndStableDtOnPatch): running max over the
// ghost-box cells of sum_d (|u_d| + c)/dx_d (NavierStokes: and of the diffusive radius) into
// *d_max (bits of a non-negative double), per patch or over a level's worklist (slot-0 states),
// and dt = (1/max)*cfl (NavierStokes: (1/(max + eps))*cfl).
int launch_spectral_patch(const hmr::Variant& v, const hmr::Params& P, const hmr::Geom& g, const hmr::Comp& Q,
                          unsigned long long* d_max, cudaStream_t st);
int launch_spectral_level(const hmr::Variant& v, const hmr::Params& P, const hmr::PatchWork* work, int npatch,
                          long total_interior, unsigned long long* d_max, cudaStream_t st);
// Cell data (from each patch's stage-`slot` state) and sensor of every patch of a worklist, one
// launch each over the flat cell / sensor item spaces (PatchWork offsets).
int launch_cells_level(const hmr::Variant& v, const hmr::Params& P, const hmr::PatchWork* work, int npatch,
                       long total_cells, int slot, cudaStream_t st);
int launch_sensor_level(const hmr::Variant& v, const hmr::PatchWork* work, int npatch, long total_sensor,
                        cudaStream_t st);
// Temperature and node velocity gradient of the stage of every patch of a level (NavierStokes;
// after launch_cells_level).
int launch_diff_grad_level(const hmr::Variant& v, const hmr::Params& P, const hmr::PatchWork* work, int npatch,
                           long total, cudaStream_t st);
int launch_stable_dt(const unsigned long long* d_max, double cfl, double* d_dt, cudaStream_t st, bool ns = false);
// Euler / NavierStokes advanceSingleStepOnPatch; with Fdint (ncoef diffusive flux sets) the
// NavierStokes form, and Fdacc (optional) accumulates them with gamma.
int launch_rk_stage(const hmr::Variant& v, const hmr::Geom& g, int ncoef, const double* alpha,
                    const double* beta, const double* gamma, const hmr::Comp* Qint, const hmr::FluxComp* Fint,
                    const hmr::Comp* Sint, const hmr::Comp& Qout, const hmr::FluxComp& Facc, const hmr::Comp& Sacc,
                    cudaStream_t st, const hmr::FluxComp* Fdint = nullptr, const hmr::FluxComp* Fdacc = nullptr);
// Refluxing: synchronizeFluxes on a coarse patch (Fd for NavierStokes), and the coarsening
// of a fine patch's interior / outer-side flux sums onto a coarse patch.
int launch_sync(const hmr::Variant& v, const hmr::Geom& g, const hmr::Comp& Q, const hmr::FluxComp& F,
                const hmr::FluxComp* Fd, const hmr::Comp& S, cudaStream_t st);
int launch_coarsen_cells(int dim, const hmr::CoarsenArgs& C, const hmr::Comp& Qf, const hmr::Comp& Qc, int ncomp,
                         cudaStream_t st);
int launch_coarsen_fluxsum(int dim, const hmr::CoarsenArgs& C, const hmr::FluxComp& Ff, const hmr::FluxComp& Fc,
                           int neq, cudaStream_t st);
// Coarse-fine ghost cells of a fine patch from a coarse patch (time fraction theta).
int launch_refine_ghosts(int dim, const hmr::CoarsenArgs& C, const hmr::Comp& Qo, const hmr::Comp& Qn, double theta,
                         const hmr::Comp& Qf, int ncomp, cudaStream_t st);
// Navier-Stokes cell phase: temperature and node velocity gradient into S.Td, S.Gd.
int launch_diff_grad(const hmr::Variant& v, const hmr::Params& P, const hmr::Geom& g, const hmr::Scratch& S,
                     cudaStream_t st);
}

// hmr_diffusive.cu, built once per arithmetic form (namespaces hmr_diff_exact, hmr_diff_fast):
// midpoint diffusive fluxes into S.Fd, and the dt-scaled face fluxes in SAMRAI side layout.
#define HMR_DECLARE_DIFF_LAUNCHERS(NS)                                                                         \
    namespace NS {                                                                                             \
    int launch_diff_mid(const hmr::Variant& v, const hmr::Params& P, const hmr::Geom& g, const hmr::Scratch& S, \
                        cudaStream_t st);                                                                      \
    int launch_diff_faces_out(const hmr::Variant& v, const hmr::Params& P, const hmr::Geom& g,                 \
                              const hmr::Scratch& S, double dt, const hmr::FluxComp& F, cudaStream_t st);      \
    }
HMR_DECLARE_DIFF_LAUNCHERS(hmr_diff_exact)
HMR_DECLARE_DIFF_LAUNCHERS(hmr_diff_fast)

// hmr_faces.cu is built once per arithmetic form, flow model and scheme set
// (twelve translation units compiled in parallel); each defines these launchers
// in namespace <form>_m<model> (WCNS5-JS, WCNS6-LD) or <form>_zc_m<model>
// (WCNS5-Z, WCNS6-CU-M2).
#define HMR_DECLARE_FACE_LAUNCHERS(NS)                                                                       \
    namespace NS {                                                                                           \
    int launch_faces(const hmr::Variant& v, const hmr::Params& P, const hmr::Geom& g, const hmr::Scratch& S, \
                     hmr::Counters* cnt, const hmr::Redo& R, cudaStream_t st);                               \
    int launch_update(const hmr::Variant& v, const hmr::Geom& g, const hmr::Scratch& S,                      \
                      const hmr::UpdateArgs& U, cudaStream_t st);                                            \
    int launch_level(const hmr::Variant& v, const hmr::Params& P, const hmr::LevelArgs& L, int blocks,       \
                     int threads, cudaStream_t st);                                                          \
    int level_max_blocks(const hmr::Variant& v, int threads, int* blocks);                                   \
    }

HMR_DECLARE_FACE_LAUNCHERS(hmr_exact_m0)
HMR_DECLARE_FACE_LAUNCHERS(hmr_exact_m1)
HMR_DECLARE_FACE_LAUNCHERS(hmr_exact_m2)
HMR_DECLARE_FACE_LAUNCHERS(hmr_fast_m0)
HMR_DECLARE_FACE_LAUNCHERS(hmr_fast_m1)
HMR_DECLARE_FACE_LAUNCHERS(hmr_fast_m2)
HMR_DECLARE_FACE_LAUNCHERS(hmr_exact_zc_m0)
HMR_DECLARE_FACE_LAUNCHERS(hmr_exact_zc_m1)
HMR_DECLARE_FACE_LAUNCHERS(hmr_exact_zc_m2)
HMR_DECLARE_FACE_LAUNCHERS(hmr_fast_zc_m0)
HMR_DECLARE_FACE_LAUNCHERS(hmr_fast_zc_m1)
HMR_DECLARE_FACE_LAUNCHERS(hmr_fast_zc_m2)

// Per-form entry points: route to the translation unit of the variant's model.
#define HMR_ROUTE(NS, FN, ...)                                            \
    switch (v.model) {                                                    \
    case hmr::SINGLE_SPECIES: return NS##_m0::FN(__VA_ARGS__);            \
    case hmr::FOUR_EQN_CONSERVATIVE: return NS##_m1::FN(__VA_ARGS__);     \
    case hmr::FIVE_EQN_ALLAIRE: return NS##_m2::FN(__VA_ARGS__);          \
    default: return -2;                                                   \
    }

// ... and to the translation unit of its scheme set.
#define HMR_ROUTE_SCHEME(NS, FN, ...)                                     \
    if (v.scheme == hmr::WCNS5_Z || v.scheme == hmr::WCNS6_CU_M2) {       \
        HMR_ROUTE(NS##_zc, FN, __VA_ARGS__)                               \
    } else {                                                              \
        HMR_ROUTE(NS, FN, __VA_ARGS__)                                    \
    }

#define HMR_DEFINE_FACE_ROUTER(NS)                                                                             \
    namespace NS {                                                                                             \
    inline int launch_faces(const hmr::Variant& v, const hmr::Params& P, const hmr::Geom& g,                   \
                            const hmr::Scratch& S, hmr::Counters* cnt, const hmr::Redo& R, cudaStream_t st) {  \
        HMR_ROUTE_SCHEME(NS, launch_faces, v, P, g, S, cnt, R, st)                                                    \
    }                                                                                                          \
    inline int launch_update(const hmr::Variant& v, const hmr::Geom& g, const hmr::Scratch& S,                 \
                             const hmr::UpdateArgs& U, cudaStream_t st) {                                      \
        HMR_ROUTE_SCHEME(NS, launch_update, v, g, S, U, st)                                                           \
    }                                                                                                          \
    inline int launch_level(const hmr::Variant& v, const hmr::Params& P, const hmr::LevelArgs& L, int blocks,  \
                            int threads, cudaStream_t st) {                                                    \
        HMR_ROUTE_SCHEME(NS, launch_level, v, P, L, blocks, threads, st)                                              \
    }                                                                                                          \
    inline int level_max_blocks(const hmr::Variant& v, int threads, int* blocks) {                             \
        HMR_ROUTE_SCHEME(NS, level_max_blocks, v, threads, blocks)                                                    \
    }                                                                                                          \
    }

HMR_DEFINE_FACE_ROUTER(hmr_exact)
HMR_DEFINE_FACE_ROUTER(hmr_fast)

// Substep adjoint, one translation unit per flow model (hmr_vjp.cu).
#define HMR_DECLARE_VJP_LAUNCHER(NS)                                                                           \
    namespace NS {                                                                                             \
    int launch_vjp(const hmr::Variant& v, const hmr::Params& P, const hmr::Geom& g, const hmr::Scratch& S,     \
                   const hmr::VjpArgs& A, hmr::VjpWork* d_rec, cudaStream_t st);                               \
    int launch_vjp_level(const hmr::Variant& v, const hmr::Params& P, const hmr::VjpWork* W, int np,           \
                         const long* totals, bool flux_terms, cudaStream_t st);                                \
    }
HMR_DECLARE_VJP_LAUNCHER(hmr_vjp_m0)
HMR_DECLARE_VJP_LAUNCHER(hmr_vjp_m1)
HMR_DECLARE_VJP_LAUNCHER(hmr_vjp_m2)

namespace hmr_vjp {
// d_rec: device space for one VjpWork record (the per-patch form is a group of one patch).
inline int launch_vjp(const hmr::Variant& v, const hmr::Params& P, const hmr::Geom& g, const hmr::Scratch& S,
                      const hmr::VjpArgs& A, hmr::VjpWork* d_rec, cudaStream_t st) {
    HMR_ROUTE(hmr_vjp, launch_vjp, v, P, g, S, A, d_rec, st)
}
// The substep VJP of a group of patches (device array W of np records; totals[PH * 3 + axis]
// items per phase); flux_terms false (beta == 0) runs only the cell gather.
inline int launch_vjp_level(const hmr::Variant& v, const hmr::Params& P, const hmr::VjpWork* W, int np,
                            const long* totals, bool flux_terms, cudaStream_t st) {
    HMR_ROUTE(hmr_vjp, launch_vjp_level, v, P, W, np, totals, flux_terms, st)
}
}
