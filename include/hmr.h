/*
 * hmr.h -- C ABI of the GB300 (sm_103a) FP64 convective hot path of HAMeRS.
 *
 * The entry points replace the per-patch calls that HAMeRS makes from its
 * Runge-Kutta level integrator (src/algs/integrator/RungeKuttaLevelIntegrator.cpp:1717-1743):
 *
 *   ConvectiveFluxReconstructor::computeConvectiveFluxAndSourceOnPatch
 *       include/flow/convective_flux_reconstructors/ConvectiveFluxReconstructor.hpp:73-81
 *       (WCNS56 implementation: src/flow/convective_flux_reconstructors/WCNS56/
 *        ConvectiveFluxReconstructorWCNS56-HLLC-HLL.cpp:40-2656)
 *   RungeKuttaPatchStrategy::advanceSingleStepOnPatch
 *       include/algs/patch_strategy/RungeKuttaPatchStrategy.hpp (implemented by
 *       src/apps/Euler/Euler.cpp:1003-1680)
 *   the per-patch stage loop of RungeKuttaLevelIntegrator::advanceLevel
 *       src/algs/integrator/RungeKuttaLevelIntegrator.cpp:1672-1748 (batched form)
 *
 * Conventions (identical to SAMRAI's pdat layout used by the reference):
 *   - every array is FP64 in device memory, x fastest, then y, then z;
 *   - a patch's conserved variables are CellData on the ghost box (interior
 *     grown by hmr_num_patch_ghosts() = 4 cells, 5 with the sixth-order diffusive
 *     flux), one array per component, in the
 *     flow model's order:
 *       single species          : rho, rho*u_k (dim), E
 *       five-equation (Allaire) : Z_i*rho_i (N), rho*u_k (dim), E, Z_i (N; the
 *                                 last volume fraction is stored as the
 *                                 reference's depth-N CellData stores it)
 *   - face fluxes are SideData with zero ghosts: for axis a the array spans
 *     the interior grown by one cell along a; arrays are ordered axis-major,
 *     flux[a*neq + e];
 *   - sources are CellData with zero ghosts (neq arrays).
 * Pointer arrays (double* const*) live in host memory; the arrays they point
 * to live in device memory.  All work is enqueued on the given CUDA stream
 * (cudaStream_t passed as void*, NULL for the legacy default stream).
 *
 * Errors: every function returns an hmr_status.  0 is success; negative
 * values reject arguments before any work is queued; positive values report
 * a CUDA error code (the context stays usable unless the CUDA error is sticky).
 * Nothing is thrown across the ABI.  A context is not thread-safe; use one
 * context per host thread / stream.
 */
#ifndef HMR_H
#define HMR_H

#ifdef __cplusplus
extern "C" {
#endif

#define HMR_MAX_SPECIES 4
#define HMR_MAX_COMPONENTS 12

typedef enum {
    HMR_OK = 0,
    HMR_ERR_ARGUMENT = -1,
    HMR_ERR_UNSUPPORTED = -2,
    HMR_ERR_NO_DEVICE = -3,
    HMR_ERR_STATE = -4,
    HMR_ERR_BARRIER = -5,
    HMR_ERR_CAPACITY = -6     /* patch too large for hmr_rk_substep_patch_noalloc's fixed scratch */
} hmr_status;

/* FlowModelManager model names (src/flow/flow_models/FlowModelManager.cpp). */
typedef enum {
    HMR_SINGLE_SPECIES = 0,
    HMR_FOUR_EQN_CONSERVATIVE = 1,
    HMR_FIVE_EQN_ALLAIRE = 2
} hmr_flow_model;

/* ConvectiveFluxReconstructorManager names
 * (src/flow/convective_flux_reconstructors/ConvectiveFluxReconstructorManager.cpp:40-91). */
typedef enum {
    HMR_WCNS5_JS_HLLC_HLL = 0,
    HMR_WCNS6_LD_HLLC_HLL = 1,
    HMR_WCNS5_Z_HLLC_HLL = 2,
    HMR_WCNS6_CU_M2_HLLC_HLL = 3
} hmr_reconstructor;

/* NavierStokes diffusive_flux_reconstructor (DiffusiveFluxReconstructorManager.cpp):
 * none (the Euler equations) or the midpoint reconstructors of the given order
 * (DiffusiveFluxReconstructorMidpointSecondOrder / ...FourthOrder / ...SixthOrder).  Single
 * species only.  The sixth order reads 5 ghost cells, so a context with it takes patch arrays
 * of ghost width 5 everywhere (hmr_num_patch_ghosts, the level's bound states included). */
typedef enum {
    HMR_DIFFUSIVE_NONE = 0,
    HMR_MIDPOINT_SECOND_ORDER = 2,
    HMR_MIDPOINT_FOURTH_ORDER = 4,
    HMR_MIDPOINT_SIXTH_ORDER = 6
} hmr_diffusive;

typedef enum {
    HMR_PRECISION_FAST = 0,   /* regrouped FP64 with FMA; <= 1e-12 relative to the reference per flux
                                 component (<= 2e-15 c/|u_n| for the components proportional to a
                                 normal velocity u_n below 1e-3 of the sound speed c) */
    HMR_PRECISION_EXACT = 1   /* the reference's operation order, no FMA: bitwise equal to it */
} hmr_precision;

typedef struct {
    int flow_model;                            /* hmr_flow_model */
    int dim;                                   /* 2 or 3 */
    int num_species;
    double species_gamma[HMR_MAX_SPECIES];     /* Equation_of_state_mixing_rules.species_gamma */
    double species_R[HMR_MAX_SPECIES];         /* Equation_of_state_mixing_rules.species_R */
    int convective_flux_reconstructor;         /* hmr_reconstructor */
    int constant_p;                            /* WCNS5-JS / WCNS5-Z / WCNS6-LD constant p (default 2) */
    int constant_q;                            /* WCNS6-LD / WCNS6-CU-M2 constant q (default 4) */
    double constant_C;                         /* WCNS6-LD constant C (default 1e9); WCNS6-CU-M2 C (default 1000) */
    double constant_alpha_tau;                 /* WCNS6-LD constant alpha_tau (default 35) */
    int precision;                             /* hmr_precision */
    double constant_Chi;                       /* WCNS6-CU-M2 constant Chi (default 1e8) */
    double constant_epsilon;                   /* WCNS6-CU-M2 constant epsilon (default 1e-8) */
    double grid_dx[3];                         /* CartesianGridGeometry::getDx(), the coarsest level's spacing:
                                                  WCNS6-CU-M2 scales its weights by it on every level
                                                  (WCNS6-CU-M2-HLLC-HLL.cpp:367-368).  Required (> 0 on the
                                                  used axes) for WCNS6-CU-M2, ignored by the other schemes. */
    int diffusive_flux_reconstructor;          /* hmr_diffusive; HMR_DIFFUSIVE_NONE by default */
    double species_mu;                         /* Equation_of_shear_viscosity_mixing_rules (CONSTANT) */
    double species_mu_v;                       /* Equation_of_bulk_viscosity_mixing_rules (CONSTANT) */
    double species_c_p;                        /* Equation_of_thermal_conductivity_mixing_rules (PRANDTL): */
    double species_Pr;                         /*   kappa = c_p*mu/Pr with that model's own constant */
    double species_mu_kappa;                   /*   shear viscosity species_mu */
} hmr_config;

typedef struct {
    int n[3];          /* interior cells per axis (n[2] ignored in 2D) */
    double dx[3];      /* grid spacing (CartesianPatchGeometry::getDx) */
} hmr_patch_geometry;

typedef struct hmr_ctx hmr_ctx;
typedef struct hmr_level hmr_level;

/* Fills cfg with the reference's defaults for the given model, scheme and dimension. */
int hmr_config_default(hmr_config* cfg, int flow_model, int reconstructor, int dim, int num_species);

/* Context: FlowModel + ConvectiveFluxReconstructor of one configuration.
 * Replaces the construction in FlowModelManager / ConvectiveFluxReconstructorManager
 * (ConvectiveFluxReconstructorManager.cpp:14-152).  Owns scratch memory. */
int hmr_ctx_create(const hmr_config* cfg, hmr_ctx** out);
int hmr_ctx_destroy(hmr_ctx* ctx);
/* FlowModel::getNumberOfEquations (include/flow/flow_models/FlowModel.hpp). */
int hmr_num_equations(const hmr_ctx* ctx);
/* Number of stored conserved components (neq, plus the last volume fraction of the five-equation model). */
int hmr_num_components(const hmr_ctx* ctx);
/* ConvectiveFluxReconstructor::getConvectiveFluxNumberOfGhostCells (ConvectiveFluxReconstructor.hpp:46-50). */
int hmr_num_ghosts(const hmr_ctx* ctx);
/* Ghost width of the patch arrays every entry point of this context reads and writes: the larger
 * of the convective and diffusive widths (NavierStokes.cpp:317-349), 4, or 5 with
 * HMR_MIDPOINT_SIXTH_ORDER. */
int hmr_num_patch_ghosts(const hmr_ctx* ctx);
/* Pre-sizes the context's scratch for patches up to this geometry (needed before stream capture). */
int hmr_ctx_reserve(hmr_ctx* ctx, const hmr_patch_geometry* geom);
/* Face counters accumulated by the flux entry points since the last reset:
 * out[0] = faces reverted to first order by the bounds check,
 * out[1] = faces where the shock sensor selected HLLC-HLL.  Synchronises the device. */
int hmr_read_counters(hmr_ctx* ctx, unsigned long long out[2], int reset);

/* ConvectiveFluxReconstructorWCNS56::computeConvectiveFluxAndSourceOnPatch
 * (ConvectiveFluxReconstructorWCNS56-HLLC-HLL.cpp:40-2656): dt-scaled convective face
 * fluxes (overwritten) and the advective source (accumulated, +=) of one patch whose
 * ghost cells are filled. */
int hmr_conv_flux_source_patch(hmr_ctx* ctx, const hmr_patch_geometry* geom, const double* const* Q,
                               double dt, double* const* flux, double* const* source, void* stream);

/* Euler::advanceSingleStepOnPatch (src/apps/Euler/Euler.cpp:1003-1680) for one stage:
 *   Q = sum_n alpha[n] Q_int[n] + beta[n] * (-div F_int[n] + S_int[n]),
 *   flux_acc += gamma[n] F_int[n], source_acc += gamma[n] S_int[n] (both optional, NULL to skip),
 * followed by updateCellDataOfConservativeVariables.  num_coeffs <= 4.  Q's interior is written. */
int hmr_rk_stage_patch(hmr_ctx* ctx, const hmr_patch_geometry* geom, int num_coeffs,
                       const double* alpha, const double* beta, const double* gamma,
                       const double* const* const* Q_int, const double* const* const* F_int,
                       const double* const* const* S_int, double* const* Q,
                       double* const* flux_acc, double* const* source_acc, void* stream);

/* DiffusiveFluxReconstructorMidpoint::computeDiffusiveFluxOnPatch
 * (src/flow/diffusive_flux_reconstructors/midpoint/DiffusiveFluxReconstructorMidpoint.cpp:38-2312):
 * dt-scaled diffusive face fluxes (overwritten; same layout as the convective flux) of one
 * single-species patch whose ghost cells are filled.  Needs a context created with a
 * diffusive_flux_reconstructor; HMR_ERR_UNSUPPORTED otherwise. */
int hmr_diff_flux_patch(hmr_ctx* ctx, const hmr_patch_geometry* geom, const double* const* Q, double dt,
                        double* const* flux, void* stream);

/* NavierStokes::advanceSingleStepOnPatch (src/apps/Navier-Stokes/NavierStokes.cpp:1249-2330):
 * hmr_rk_stage_patch with the diffusive fluxes Fd_int[n] entering the divergence,
 *   Q = sum_n alpha[n] Q_int[n] + beta[n] * (-div (F_int[n] + Fd_int[n]) + S_int[n]),
 * and diff_flux_acc += gamma[n] Fd_int[n] beside flux_acc and source_acc (all three optional
 * together).  Single-species contexts with a diffusive_flux_reconstructor. */
int hmr_rk_stage_ns_patch(hmr_ctx* ctx, const hmr_patch_geometry* geom, int num_coeffs,
                          const double* alpha, const double* beta, const double* gamma,
                          const double* const* const* Q_int, const double* const* const* F_int,
                          const double* const* const* Fd_int, const double* const* const* S_int,
                          double* const* Q, double* const* flux_acc, double* const* diff_flux_acc,
                          double* const* source_acc, void* stream);

/* Fused flux + stage update of stage `stage` of a Shu-Osher scheme whose flux weight is
 * non-zero only for the current stage (SSPRK3 is): computes the convective flux and source
 * of Q_int[stage] and writes Q_out = sum_n alpha[n] Q_int[n] + beta * (-div F + S) on the
 * interior.  Q_int has stage+1 states; Q_int[stage] must have its ghost cells filled.
 * With a diffusive_flux_reconstructor in the context this is NavierStokes's stage: the
 * diffusive flux of Q_int[stage] enters the divergence too. */
int hmr_rk_substep_patch(hmr_ctx* ctx, const hmr_patch_geometry* geom, int stage, const double* alpha,
                         double beta, const double* const* const* Q_int, double dt, double* const* Q_out,
                         void* stream);

/* Ghost fill modes per axis (the `periodic` arrays below). */
typedef enum {
    HMR_FILL_ZERO_GRADIENT = 0,   /* copy of the nearest interior cell (extrapolation boundary) */
    HMR_FILL_PERIODIC = 1,        /* periodic image within the patch */
    HMR_FILL_PROVIDED = 2,        /* ghost cells supplied by the caller are left untouched */
    HMR_FILL_REFLECT = 3,         /* reflecting (slip) wall: mirror image across the boundary face with the
                                     normal momentum negated -- the reference's REFLECT condition
                                     (BasicCartesianBoundaryUtilities2.cpp:349-440 with the scalar/vector
                                     split of EulerBoundaryConditions.cpp:205-297); needs >= 4 cells along
                                     the axis */
    HMR_FILL_DIRICHLET = 4,       /* the reference's DIRICHLET condition (BasicCartesianBoundaryUtilities2.cpp:
                                     150-165, values from EulerBoundaryConditions::
                                     readDirichletBoundaryDataEntry): every ghost cell beyond the side takes
                                     the side's conservative values (hmr_set_dirichlet_values); a corner
                                     beyond two Dirichlet sides takes the lower axis's, and one beyond a
                                     Dirichlet side and another condition the Dirichlet values -- the corner
                                     conditions XDIRICHLET / YDIRICHLET / ZDIRICHLET naming that axis */
    HMR_FILL_SYMMETRY = 5         /* the reference's SYMMETRY condition as the master condition of every
                                     variable (BasicCartesianBoundaryUtilities2.cpp:397-440): the mirror
                                     image across the boundary face, no component negated; needs >= 4
                                     cells along the axis */
} hmr_fill_mode;

/* Values of the HMR_FILL_DIRICHLET side `side` (0 low, 1 high) of axis `axis`: ncomp conservative
 * values (the reference converts the input's primitive values to these once, with the flow model's
 * basic utilities, EulerBoundaryConditions.cpp:638-723).  Held by the context for every fill that
 * runs on it afterwards, per patch and per level (captured level graphs included: they read the
 * values from the context's device copy); 0.0 until set.  The device copy is written by a
 * synchronous cudaMemcpy: set values between steps, not while a fill of this context is in
 * flight on another stream.  Rejects non-finite values. */
int hmr_set_dirichlet_values(hmr_ctx* ctx, int axis, int side, const double* values);

/* Single-patch ghost fill, mode per axis (hmr_fill_mode; other values are rejected with
 * HMR_ERR_ARGUMENT) -- the one-patch equivalent of the SAMRAI fill schedule,
 * RungeKuttaLevelIntegrator.cpp:1568,1701. */
int hmr_fill_ghosts_patch(hmr_ctx* ctx, const hmr_patch_geometry* geom, double* const* Q,
                          const int* periodic, void* stream);

/* Stable time step of a patch (Euler::computeSpectralRadiusesAndStableDtOnPatch,
 * src/apps/Euler/Euler.cpp:489-900): the maximum over the cells of the ghost box (the
 * reference's loops include the ghost cells) of sum_d (|u_d| + c)/dx_d is max-reduced into
 * *d_max (a device double holding a non-negative value: 0.0 to start, or a previous patch's
 * value for a running maximum over a level).  The level's time step is then (1/max)*CFL
 * (RungeKuttaLevelIntegrator.cpp:1846-1916).  With a diffusive_flux_reconstructor this is
 * NavierStokes's (NavierStokes.cpp:595-1100): the maximum also covers the diffusive radius
 * 2 max_d(D/dx_d^2), D = max(mu/rho, mu_v/rho, kappa/(rho c_p)), and the time step is
 * (1/(max + 1e-15))*CFL. */
int hmr_spectral_radius_patch(hmr_ctx* ctx, const hmr_patch_geometry* geom, const double* const* Q,
                              double* d_max, void* stream);

/* Refluxing (RungeKuttaLevelIntegrator.cpp:2120-2230, synchronising a coarse level with the
 * finer one after its step).  Fluxes are the time-integrated ones that hmr_rk_stage_patch /
 * hmr_rk_stage_ns_patch accumulate with gamma (keep accumulating the fine patch's over its
 * time-refined steps).  A patch's placement is the level index of its first interior cell (lo)
 * and its size; the fine box must be aligned with the refinement ratio.
 *
 * hmr_coarsen_fluxsum_patch: on the outer sides of the fine patch, every coarse face of
 * coarse_flux that the side covers takes the mean of the fine faces of fine_flux within it
 * (the flux-sum coarsening, :2140-2160).
 * hmr_sync_fluxes_patch: Euler::synchronizeFluxes (src/apps/Euler/Euler.cpp:1682-1943) /
 * NavierStokes::synchronizeFluxes (diff_flux non-null; NavierStokes.cpp:2425-2700): the coarse
 * patch's step redone from its old state Q (ghost box, interior updated) with those fluxes,
 * Q += -div (flux [+ diff_flux]) + source, then the five-equation last volume fraction.
 * hmr_coarsen_patch: every coarse cell the fine patch covers takes the mean of its fine cells
 * (the coarsening of fine interiors, :2190-2230).
 * The two coarsenings are SAMRAI's CONSERVATIVE_COARSEN (volume / area weighted means). */
int hmr_coarsen_fluxsum_patch(hmr_ctx* ctx, const hmr_patch_geometry* coarse, const int* coarse_lo,
                              const hmr_patch_geometry* fine, const int* fine_lo, const int* ratio,
                              const double* const* fine_flux, double* const* coarse_flux, void* stream);
int hmr_sync_fluxes_patch(hmr_ctx* ctx, const hmr_patch_geometry* geom, double* const* Q,
                          const double* const* flux, const double* const* diff_flux,
                          const double* const* source, void* stream);
int hmr_coarsen_patch(hmr_ctx* ctx, const hmr_patch_geometry* coarse, const int* coarse_lo,
                      const hmr_patch_geometry* fine, const int* fine_lo, const int* ratio,
                      const double* const* Q_fine, double* const* Q_coarse, void* stream);

/* Coarse-fine ghost cells of a fine patch: the part of the fill schedule that interpolates
 * from the next coarser level (RungeKuttaLevelIntegrator.cpp:1568,1701; operators registered at
 * src/flow/flow_models/single-species/FlowModelSingleSpecies.cpp:578-597).  The coarse state at
 * the fine time is (1 - theta) Q_coarse_old + theta Q_coarse_new; every ghost cell of Q_fine
 * whose coarse cell lies in the coarse patch's interior takes the conservative linear
 * refinement of it (monotonised-central slopes per coarse cell: the fine values average back
 * to the coarse value).  The coarse patch's ghost cells must be filled.  Same-level neighbour
 * copies overwrite these values afterwards where a neighbour exists. */
int hmr_refine_ghosts_patch(hmr_ctx* ctx, const hmr_patch_geometry* fine, const int* fine_lo,
                            const hmr_patch_geometry* coarse, const int* coarse_lo, const int* ratio,
                            const double* const* Q_coarse_old, const double* const* Q_coarse_new, double theta,
                            double* const* Q_fine, void* stream);

/* Adjoint (vector-Jacobian product) of hmr_rk_substep_patch.  No counterpart in the reference,
 * which has no derivative code.  For the adjoint Qbar_out of the substep's output (ghost-box
 * arrays; interior read) it accumulates into Qbar_int[n] (n = 0..stage, ghost boxes, caller
 * zeroes them) the product of Qbar_out with the Jacobian of the output with respect to Q_int[n]:
 * alpha[n] Qbar_out on the interior, plus, for n = stage, beta times the transposed Jacobian of
 * the flux divergence and source, which also reaches the ghost cells of Qbar_int[stage] (fold it
 * into the interior with hmr_fill_ghosts_vjp_patch when the ghosts were filled from it).
 * The forward values are recomputed in the reference's operation order, so every discrete choice
 * (bounds fallback, shock sensor, HLLC side, WCNS6-LD switch, min/max) is the forward substep's;
 * derivatives follow that branch (|x|, min, max and sqrt(0) take the one-sided conventions of the
 * oracle's tangent).  Same arguments as hmr_rk_substep_patch otherwise; uses the context's
 * scratch plus (6 neq + 2) doubles per midpoint face of its own. */
int hmr_rk_substep_vjp_patch(hmr_ctx* ctx, const hmr_patch_geometry* geom, int stage, const double* alpha,
                             double beta, const double* const* const* Q_int, double dt,
                             const double* const* Qbar_out, double* const* const* Qbar_int, void* stream);

/* Adjoint of hmr_fill_ghosts_patch: adds the adjoint of every filled ghost cell to the interior
 * cell it is copied from (negated for the normal momentum at a reflecting wall) and zeroes it;
 * Dirichlet ghost cells copy no cell (their adjoints are zeroed); ghost cells along
 * HMR_FILL_PROVIDED axes keep their adjoints (they belong to whatever supplied the values).  No
 * counterpart in the reference. */
int hmr_fill_ghosts_vjp_patch(hmr_ctx* ctx, const hmr_patch_geometry* geom, double* const* Qbar,
                              const int* periodic, void* stream);

/* Batched form: every patch of a level advanced by one persistent kernel per RK substep over a
 * device-resident worklist (replaces the patch loop of RungeKuttaLevelIntegrator.cpp:1717-1743).
 * The caller owns each patch's state (slot 0, bound with hmr_level_bind_state); the level owns
 * the intermediate stage buffers (slots 1, 2), the scratch and the captured step graph. */
int hmr_level_create(hmr_ctx* ctx, int num_patches, const hmr_patch_geometry* geoms, hmr_level** out);
int hmr_level_destroy(hmr_level* level);
/* Places the level's patches in its index space and enables the device-resident ghost exchange
 * (the same-level part of SAMRAI's fill schedule, RungeKuttaLevelIntegrator.cpp:1568,1701):
 * before every substep the ghost cells of each patch are copied from the interiors of the
 * patches (and of their periodic images) that cover them, then cells outside the domain along
 * non-periodic axes take the nearest in-domain value (zero-gradient, the extrapolation boundary)
 * or, at reflecting walls, the mirror image across the domain face with the normal momentum
 * negated, or at Dirichlet faces the face's values (as hmr_fill_ghosts_patch); ghost cells inside
 * the domain covered by no patch of the level (a coarse-fine boundary) are left as the caller
 * provides them.  lo: 3 ints per patch (first interior cell), domain: cells per axis, periodic
 * per axis: 1 periodic, 0 zero-gradient faces, HMR_FILL_REFLECT reflecting walls,
 * HMR_FILL_DIRICHLET Dirichlet faces, HMR_FILL_SYMMETRY symmetry planes.  Boxes must lie in the
 * domain and not overlap. */
int hmr_level_set_layout(hmr_level* level, const int* lo, const int* domain, const int* periodic);
/* Binds the caller's ghost-box arrays (ncomp device pointers) as slot 0 of a patch. */
int hmr_level_bind_state(hmr_level* level, int patch, double* const* comps);
/* Device pointers of the stage-`slot` state of a patch (slot 0: the bound arrays). */
int hmr_level_state(hmr_level* level, int patch, int slot, double** comps_out);
/* Ghost fill mode per axis of a patch in the batched substeps (hmr_fill_mode; default
 * HMR_FILL_ZERO_GRADIENT): HMR_FILL_PERIODIC for a patch spanning a periodic direction,
 * HMR_FILL_PROVIDED where the caller supplies the ghost cells. */
int hmr_level_set_periodic(hmr_level* level, int patch, const int* periodic);
/* Runs substep `stage` (0..2 of SSPRK3) for all patches as one captured CUDA graph (barrier
 * reset + one persistent kernel: ghost fill, cells, sensor, faces, update).  Reads slots
 * 0..stage, writes slot stage+1 (slot 0 for the last stage).  The graph is captured on the
 * first call for a given dt, so the first call should precede any outer stream capture. */
int hmr_level_substep(hmr_level* level, int stage, double dt, void* stream);
/* One SSPRK3 step: the three substep graphs in order. */
int hmr_level_step(hmr_level* level, double dt, void* stream);
/* Vector-Jacobian product of hmr_level_substep over every patch of the level, batched (no
 * counterpart in the reference: its adjoint form, like hmr_rk_substep_vjp_patch's).  For each
 * patch p it adds to Qbar_int[p][n] (n = 0..stage; ncomp ghost-box arrays each) the product of
 * Qbar_out[p] (ncomp ghost-box arrays; interior read) with the Jacobian of substep `stage` at
 * the level's stage states, as they stand after the forward substep (slot `stage` ghost-filled);
 * the ghost fill's own adjoint is the caller's, as for the per-patch form.  Results are bitwise
 * those of hmr_rk_substep_vjp_patch on each patch.  The patches run together, one launch per
 * phase over the flat item space of a group of patches whose per-face reverse buffers (about
 * 1.2 KB per face) fit a quarter of the device memory free at the first call; the buffers
 * stay with the level.  With a diffusive_flux_reconstructor the diffusive flux's reverse is
 * included, as in the per-patch form.  HMR_ERR_STATE until every patch's slot 0 is bound. */
int hmr_level_substep_vjp(hmr_level* level, int stage, double dt, const double* const* const* Qbar_out,
                          double* const* const* const* Qbar_int, void* stream);
/* Adjoint of the level's ghost fill (the fill at the start of every substep): Qbar[p] (ncomp
 * ghost-box arrays per patch) hold the adjoints of the filled state; every ghost cell the fill
 * wrote adds its adjoint to the cell it was copied from -- for a level with a layout, first the
 * physical faces' ghost cells (zero-gradient or mirror images, the normal momentum negated at
 * reflecting walls) into in-domain cells, then the exchanged ghost cells into the interiors of
 * the patches (and periodic images) they came from; without a layout, each patch's own fill as
 * hmr_fill_ghosts_vjp_patch -- and is zeroed.  Ghost cells no copy wrote keep their adjoints.
 * Several ghost cells summing into one cell add atomically, so the last bits of such sums may
 * vary between runs.  No counterpart in the reference. */
int hmr_level_fill_vjp(hmr_level* level, double* const* const* Qbar, void* stream);
/* Memory budget of hmr_level_substep_vjp's per-face reverse buffers, in bytes (0: a quarter of
 * the device memory free at the next call).  The largest patch always gets its buffers; a
 * smaller budget splits the level into more groups of patches. */
int hmr_level_set_vjp_budget(hmr_level* level, unsigned long long bytes);
/* Synchronises and reports whether a barrier of a persistent kernel gave up
 * (HMR_ERR_BARRIER, flag cleared) since the last check. */
/* One SSPRK3 step whose time step is computed on the device from the slot-0 states (ghost
 * boxes as they stand), dt = (1/max spectral radius)*cfl over every patch of the level
 * (NavierStokes: as hmr_spectral_radius_patch describes), inside the same captured
 * graph as the three substeps: no host synchronisation per step.  The graph is cached for
 * the cfl value. */
int hmr_level_step_cfl(hmr_level* level, double cfl, void* stream);
/* Time step used by the last hmr_level_step_cfl (synchronises). */
int hmr_level_last_dt(hmr_level* level, double* dt);
int hmr_level_check(hmr_level* level);
/* Diagnostic: bound every barrier wait by timeout_ns and, with extra_arrivals = 1, make the
 * first barrier unreachable so that the give-up path can be tested.  Use (0, 2e9) to restore. */
int hmr_level_barrier_diagnostic(hmr_level* level, unsigned int extra_arrivals, unsigned long long timeout_ns);
/* Launch shape of the persistent kernel: 64 or 128 threads per block and 1..(resident
 * maximum) blocks per SM; HMR_ERR_ARGUMENT for a shape that cannot be resident at once. */
int hmr_level_set_launch(hmr_level* level, int threads, int blocks_per_sm);
/* Work splitting of the persistent kernel: every phase's items are handed out in chunks of
 * chunk_blocks (1, 2 or 4) block widths taken from a counter in order; mode bit 0 hands the
 * cell-wise phases (cell data, sensor, update) out by a fixed grid stride instead; bit 1 (fast
 * form) sorts the faces by their sensor first and runs the HLLC faces in the fast form beside the
 * HLLC-HLL faces in the exact form (instead of the exact form in a phase of its own).  Results
 * do not depend on any of them. */
int hmr_level_set_work_split(hmr_level* level, int chunk_blocks, int mode);
int hmr_level_work_split(hmr_level* level, int* chunk_blocks, int* mode);
/* Autotuner: times the persistent kernel of this level at 64 and 128 threads per block and
 * every resident block count per SM, then the work splittings at the fastest shape, and keeps
 * the fastest.  Returns the chosen shape (hmr_level_work_split gives the chosen splitting). */
int hmr_level_autotune(hmr_level* level, double dt, int* threads_out, int* blocks_per_sm_out, void* stream);

/* Fixed device scratch of hmr_rk_substep_patch_noalloc: 32 MiB, held on every GPU that loads
 * the library until the process exits. */
#define HMR_NOALLOC_SCRATCH_BYTES (32u << 20)

/* hmr_rk_substep_patch without any allocation.  No counterpart in the reference: it exists for
 * callers that cannot allocate device memory at the point of the call -- hosts whose device memory
 * is owned by their own pool allocator, code that must not trigger the implicit device
 * synchronisation of cudaMalloc/cudaFree inside a time-step loop, and plugin environments that
 * forbid allocation.  It takes the configuration directly (creating an hmr_ctx allocates) and
 * keeps its scratch in a file-scope device array of HMR_NOALLOC_SCRATCH_BYTES.
 *   - Same arguments and result as hmr_rk_substep_patch (stage < 3, Q_int[stage] ghost-filled).
 *   - Patches whose scratch exceeds the array are rejected with HMR_ERR_CAPACITY before any work
 *     is queued: square/cubic patches fit up to 453^2 (2D single species), 397^2 (2D five-equation),
 *     48^3 (3D single species) and 44^3 (3D five-equation) cells.
 *   - The first call on a device resolves the array's device address (cudaGetSymbolAddress with
 *     that device current) and caches it.  The address belongs to the CUDA context: after cudaDeviceReset, or when another context is
 *     current on the device, the next call resolves it again (and is again a first call).
 *   - Allocates nothing: no cudaMalloc, cudaFree or allocating library call.  The face counters
 *     of hmr_read_counters are not updated.
 *   - Every call shares the one array and leaves its contents behind; calls whose work overlaps
 *     on the GPU (different streams without ordering) race on it.  Serialise them. */
int hmr_rk_substep_patch_noalloc(const hmr_config* cfg, const hmr_patch_geometry* geom, int stage,
                                 const double* alpha, double beta, const double* const* const* Q_int,
                                 double dt, double* const* Q_out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* HMR_H */
