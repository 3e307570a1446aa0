// C ABI of the GB300 convective hot path (declarations and contracts in include/hmr.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <vector>

#include "../../include/hmr.h"
#include "hmr_launch.h"

using namespace hmr;

struct hmr_ctx {
    Variant v;
    Params P;
    int precision;
    int neq, ncomp;
    double* scratch = nullptr;
    size_t scratch_bytes = 0;
    Counters* counters = nullptr;
    unsigned int* redo_count = nullptr;
    double* vjp = nullptr;             // face contributions of the substep adjoint
    size_t vjp_bytes = 0;
    double* d_bvals = nullptr;         // Dirichlet values per side (2 axis + high) x ncomp, on the device
    double h_bvals[6 * MAX_COMP] = {};  // and their host copy
};

// barrier arrivals, redo-queue length, eight phase-chunk counters, four sorted-face counts
constexpr int LEVEL_COUNTERS = 14;

struct hmr_level {
    hmr_ctx* ctx;
    int npatch;
    std::vector<Geom> geoms;
    std::vector<PatchWork> work;       // host copy
    PatchWork* d_work = nullptr;       // 3 x npatch: the worklist of each stage
    double* d_state = nullptr;         // stage slots 1 and 2 of every patch (slot 0 is bound by the caller)
    double* d_scratch = nullptr;
    std::vector<size_t> state_off;     // per patch, in doubles
    LevelArgs L = {};
    unsigned int* d_barrier = nullptr;   // [0] barrier arrivals, [1] redo-queue length, [2..8] phase chunks
    int* d_status = nullptr;
    unsigned long long* d_redo = nullptr;
    unsigned long long* d_sorted = nullptr;   // per-axis lists of sorted faces (redo_cap entries)
    long redo_cap = 0;
    int threads = 128;
    int blocks = 0;
    // one captured graph per substep (barrier reset + persistent kernel)
    cudaGraphExec_t graph[3] = {nullptr, nullptr, nullptr};
    double graph_dt[3] = {0.0, 0.0, 0.0};
    bool graph_ok[3] = {false, false, false};
    bool dirty = true;                 // worklist changed since it was uploaded
    int bound = 0;                     // patches whose slot 0 is bound
    // step with the stable time step computed on the device (spectral radius -> dt -> 3 substeps)
    // ghost exchange between patches (hmr_level_set_layout)
    GhostCopy* d_copies = nullptr;
    int ncopy = 0;
    long total_copy = 0;
    bool exchange = false;
    int dom[3] = {1, 1, 1};
    int dom_periodic[3] = {0, 0, 0};
    unsigned long long* d_srmax = nullptr;
    double* d_dt = nullptr;
    cudaGraphExec_t cfl_graph = nullptr;
    double cfl_graph_cfl = 0.0;
    // batched substep VJP: per-face reverse buffers of one group of patches, and the records
    double* d_vjp = nullptr;
    size_t vjp_bytes = 0;
    size_t vjp_budget = 0;             // 0: a quarter of the free device memory at the first call
    VjpWork* d_vjpwork = nullptr;
    hmr_cells::LevelFillVjpPatch* d_fillvjp = nullptr;   // records of the ghost fill's adjoint
};

static int cuda_status(cudaError_t e) { return e == cudaSuccess ? HMR_OK : (int)e; }

static inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Ghost width of a context's patch arrays: the larger of the convective (4) and diffusive
// widths, as NavierStokes.cpp:317-349 sizes them; the sixth-order midpoint diffusive flux
// needs 5 (DiffusiveFluxReconstructorMidpointSixthOrder.cpp:22), the others at most 3.
static int patch_ghosts(const Variant& v) { return v.dorder == HMR_MIDPOINT_SIXTH_ORDER ? 5 : GHOST; }

// Half-width of the diffusive midpoint set (faces -W .. n + W): 2 at sixth order, else 1.
static int diff_half_width(const Variant& v) { return v.dorder == HMR_MIDPOINT_SIXTH_ORDER ? 2 : 1; }

static Geom make_geom(int dim, const hmr_patch_geometry* pg, int gh) {
    Geom g;
    g.gh = gh;
    for (int d = 0; d < 3; d++) {
        g.n[d] = d < dim ? pg->n[d] : 1;
        g.G[d] = d < dim ? g.n[d] + 2 * gh : 1;
        g.dx[d] = d < dim ? pg->dx[d] : 1.0;
    }
    return g;
}

// First momentum component of the conserved variables: single species (rho, rho u, E) 1;
// four- and five-equation models (partial densities first) the number of species.
static int momentum0(const Variant& v) { return v.model == SINGLE_SPECIES ? 1 : v.nsp; }

// Fill modes of a patch's axes (hmr_fill_mode); a reflecting wall mirrors its gh ghost cells,
// so the patch needs at least that many along the axis.
static bool valid_fill_modes(int dim, const hmr_patch_geometry* pg, const int* mode, int gh) {
    if (!mode) return false;
    for (int a = 0; a < dim; a++) {
        if (mode[a] < HMR_FILL_ZERO_GRADIENT || mode[a] > HMR_FILL_SYMMETRY) return false;
        if ((mode[a] == HMR_FILL_REFLECT || mode[a] == HMR_FILL_SYMMETRY) && pg->n[a] < gh) return false;
    }
    return true;
}

static bool valid_geom(int dim, const hmr_patch_geometry* pg) {
    if (!pg) return false;
    for (int d = 0; d < dim; d++) {
        if (pg->n[d] < 1 || pg->n[d] > (1 << 20)) return false;
        if (!(pg->dx[d] > 0.0)) return false;
    }
    long cells = 1;
    for (int d = 0; d < dim; d++) cells *= (long)pg->n[d] + 2 * GHOST_MAX;
    return cells < (1L << 40);
}

// Scratch size in doubles for one patch (cell data, midpoint fluxes and
// velocities, and the queue of faces handed to the exact form).
static long total_faces_of(int dim, const Geom& g) {
    long t = 0;
    for (int a = 0; a < dim; a++) t += nface_of(g, a);
    return t;
}

static size_t scratch_doubles(const hmr_ctx* c, const Geom& g) {
    const long nc = ncell_of(g);
    size_t s = (size_t)(c->neq + 4) * nc;
    for (int a = 0; a < c->v.dim; a++) s += (size_t)(c->neq + 2) * nface_of(g, a);
    s += (size_t)total_faces_of(c->v.dim, g);   // the fast form's lists of sorted faces
    if (c->P.dorder) {
        // NavierStokes: temperature, node velocity gradient, midpoint diffusive fluxes
        s += (size_t)(1 + c->v.dim * c->v.dim) * nc;
        for (int a = 0; a < c->v.dim; a++) s += (size_t)c->neq * nface_w(g, a, diff_half_width(c->v));
    }
    return s + 64;
}

static long total_faces(const hmr_ctx* c, const Geom& g) {
    long t = 0;
    for (int a = 0; a < c->v.dim; a++) t += nface_of(g, a);
    return t;
}

static Scratch carve_scratch(const hmr_ctx* c, const Geom& g, double* base) {
    Scratch S;
    const long nc = ncell_of(g);
    double* p = base;
    S.V = p; p += (size_t)c->neq * nc;
    S.rho = p; p += nc;
    S.cs = p; p += nc;
    S.theta = p; p += nc;
    S.Omega = p; p += nc;
    for (int a = 0; a < 3; a++) {
        if (a < c->v.dim) {
            const long nf = nface_of(g, a);
            S.Fm[a] = p; p += (size_t)c->neq * nf;
            S.um[a] = p; p += nf;
        } else {
            S.Fm[a] = nullptr;
            S.um[a] = nullptr;
        }
    }
    p += total_faces(c, g);   // queue of faces for the exact pass (face_launch)
    p += total_faces(c, g);   // the fast form's per-axis lists of HLLC faces (face_launch)
    S.Td = S.Gd = nullptr;
    for (int a = 0; a < 3; a++) S.Fd[a] = nullptr;
    if (c->P.dorder) {
        S.Td = p; p += nc;
        S.Gd = p; p += (size_t)c->v.dim * c->v.dim * nc;
        for (int a = 0; a < c->v.dim; a++) { S.Fd[a] = p; p += (size_t)c->neq * nface_w(g, a, diff_half_width(c->v)); }
    }
    return S;
}

static int ensure_scratch(hmr_ctx* c, const Geom& g) {
    const size_t need = scratch_doubles(c, g) * sizeof(double);
    if (need <= c->scratch_bytes) return HMR_OK;
    if (c->scratch) cudaFree(c->scratch);
    c->scratch = nullptr;
    c->scratch_bytes = 0;
    cudaError_t e = cudaMalloc(&c->scratch, need);
    if (e != cudaSuccess) return cuda_status(e);
    c->scratch_bytes = need;
    return HMR_OK;
}

static int face_launch(hmr_ctx* c, const Geom& g, const Scratch& S, cudaStream_t st) {
    Redo R;
    // The queue follows the per-axis arrays carved by carve_scratch.
    R.list = reinterpret_cast<unsigned long long*>(S.um[c->v.dim - 1] + nface_of(g, c->v.dim - 1));
    R.count = c->redo_count;
    R.cap = (unsigned long long)total_faces(c, g);
    // Sorted faces (the fast form's HLLC faces beside the exact HLLC-HLL ones in one launch) pay on
    // patches too small to fill the GPU with either set alone (256^2: 1.51e8 -> 1.67e8 cell-updates
    // per second); on larger ones each set fills it and the sorting pass is a small extra cost.
    if (total_faces(c, g) <= (1L << 20)) {
        R.fast = R.list + total_faces(c, g);
        R.fast_count = c->redo_count + 1;
        for (int a = 1; a < c->v.dim; a++) R.fast_off[a] = R.fast_off[a - 1] + nface_of(g, a - 1);
    }
    if (c->precision == HMR_PRECISION_EXACT) return hmr_exact::launch_faces(c->v, c->P, g, S, c->counters, R, st);
    return hmr_fast::launch_faces(c->v, c->P, g, S, c->counters, R, st);
}

static int update_launch(hmr_ctx* c, const Geom& g, const Scratch& S, const UpdateArgs& U, cudaStream_t st) {
    if (c->precision == HMR_PRECISION_EXACT) return hmr_exact::launch_update(c->v, g, S, U, st);
    return hmr_fast::launch_update(c->v, g, S, U, st);
}

// NavierStokes: temperature and node gradient (always exact), then the midpoint diffusive fluxes.
static int diff_launch(hmr_ctx* c, const Geom& g, const Scratch& S, cudaStream_t st) {
    int r = hmr_cells::launch_diff_grad(c->v, c->P, g, S, st);
    if (r) return r;
    if (c->precision == HMR_PRECISION_EXACT) return hmr_diff_exact::launch_diff_mid(c->v, c->P, g, S, st);
    return hmr_diff_fast::launch_diff_mid(c->v, c->P, g, S, st);
}

template <class C>
static bool load_ptrs(C& out, const double* const* ptrs, int n) {
    constexpr int cap = (int)(sizeof(out.p) / sizeof(out.p[0]));
    for (int e = 0; e < cap; e++) out.p[e] = nullptr;
    if (!ptrs || n < 1 || n > cap) return false;
    for (int e = 0; e < n; e++) {
        if (!ptrs[e]) return false;
        out.p[e] = const_cast<double*>(ptrs[e]);
    }
    return true;
}
static bool load_comp(Comp& C, const double* const* ptrs, int n) { return load_ptrs(C, ptrs, n); }
static bool load_flux(FluxComp& C, const double* const* ptrs, int n) { return load_ptrs(C, ptrs, n); }

extern "C" {

int hmr_config_default(hmr_config* cfg, int flow_model, int reconstructor, int dim, int num_species) {
    if (!cfg) return HMR_ERR_ARGUMENT;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->flow_model = flow_model;
    cfg->dim = dim;
    cfg->num_species = num_species;
    for (int s = 0; s < HMR_MAX_SPECIES; s++) {
        cfg->species_gamma[s] = 1.4;
        cfg->species_R[s] = 1.0;
    }
    cfg->convective_flux_reconstructor = reconstructor;
    cfg->constant_p = 2;
    cfg->constant_q = 4;
    // WCNS6-CU-M2-HLLC-HLL.cpp:252-270; the other schemes' C is WCNS6-LD's
    cfg->constant_C = reconstructor == HMR_WCNS6_CU_M2_HLLC_HLL ? 1000.0 : 1.0e9;
    cfg->constant_alpha_tau = 35.0;
    cfg->constant_Chi = 1.0e8;
    cfg->constant_epsilon = 1.0e-8;
    cfg->precision = HMR_PRECISION_FAST;
    return HMR_OK;
}

int hmr_ctx_create(const hmr_config* cfg, hmr_ctx** out) {
    if (!cfg || !out) return HMR_ERR_ARGUMENT;
    *out = nullptr;
    if (cfg->dim != 2 && cfg->dim != 3) return HMR_ERR_ARGUMENT;
    if (cfg->num_species < 1 || cfg->num_species > HMR_MAX_SPECIES) return HMR_ERR_ARGUMENT;
    if (!reconstructor_known(cfg->convective_flux_reconstructor)) return HMR_ERR_UNSUPPORTED;
    if (cfg->precision != HMR_PRECISION_FAST && cfg->precision != HMR_PRECISION_EXACT) return HMR_ERR_ARGUMENT;
    {
        Params probe;  // scheme constants in range (and, for WCNS6-CU-M2, the grid spacing set)
        const int r = scheme_params(cfg, probe);
        if (r) return r;
    }
    int neq = 0, ncomp = 0;
    if (cfg->flow_model == HMR_SINGLE_SPECIES) {
        if (cfg->num_species != 1) return HMR_ERR_ARGUMENT;
        neq = cfg->dim + 2;
        ncomp = neq;
    } else if (cfg->flow_model == HMR_FIVE_EQN_ALLAIRE) {
        if (cfg->num_species != 2) return HMR_ERR_UNSUPPORTED;
        neq = cfg->dim + 2 * cfg->num_species;
        ncomp = neq + 1;
    } else if (cfg->flow_model == HMR_FOUR_EQN_CONSERVATIVE) {
        if (cfg->num_species != 2) return HMR_ERR_UNSUPPORTED;
        neq = cfg->num_species + cfg->dim + 1;
        ncomp = neq;
    } else {
        return HMR_ERR_UNSUPPORTED;
    }
    for (int s = 0; s < cfg->num_species; s++) {
        if (!(cfg->species_gamma[s] > 1.0)) return HMR_ERR_ARGUMENT;
        if (cfg->flow_model == HMR_FOUR_EQN_CONSERVATIVE && !(cfg->species_R[s] > 0.0)) return HMR_ERR_ARGUMENT;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        return HMR_ERR_NO_DEVICE;
    }
    hmr_ctx* c = new (std::nothrow) hmr_ctx();
    if (!c) return HMR_ERR_ARGUMENT;
    c->v.dim = cfg->dim;
    c->v.model = cfg->flow_model;
    c->v.nsp = cfg->num_species;
    c->v.scheme = cfg->convective_flux_reconstructor;
    c->v.dorder = cfg->diffusive_flux_reconstructor;
    species_params(cfg->species_gamma, cfg->species_R, cfg->num_species, c->P);
    scheme_params(cfg, c->P);
    c->precision = cfg->precision;
    c->neq = neq;
    c->ncomp = ncomp;
    cudaError_t e = cudaMalloc(&c->counters, sizeof(Counters));
    if (e == cudaSuccess) e = cudaMemset(c->counters, 0, sizeof(Counters));
    // the queue's length, the three lists' lengths and the number of HLLC-HLL faces sorted
    if (e == cudaSuccess) e = cudaMalloc(&c->redo_count, 5 * sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMalloc(&c->d_bvals, sizeof(c->h_bvals));
    if (e == cudaSuccess) e = cudaMemset(c->d_bvals, 0, sizeof(c->h_bvals));
    if (e != cudaSuccess) {
        hmr_ctx_destroy(c);
        return cuda_status(e);
    }
    *out = c;
    return HMR_OK;
}

int hmr_ctx_destroy(hmr_ctx* c) {
    if (!c) return HMR_ERR_ARGUMENT;
    if (c->scratch) cudaFree(c->scratch);
    if (c->counters) cudaFree(c->counters);
    if (c->redo_count) cudaFree(c->redo_count);
    if (c->vjp) cudaFree(c->vjp);
    if (c->d_bvals) cudaFree(c->d_bvals);
    delete c;
    return HMR_OK;
}

int hmr_set_dirichlet_values(hmr_ctx* c, int axis, int side, const double* values) {
    if (!c || axis < 0 || axis >= c->v.dim || (side != 0 && side != 1) || !values) return HMR_ERR_ARGUMENT;
    for (int e = 0; e < c->ncomp; e++)
        if (!std::isfinite(values[e])) return HMR_ERR_ARGUMENT;
    std::memcpy(c->h_bvals + (2 * axis + side) * c->ncomp, values, sizeof(double) * (size_t)c->ncomp);
    return cuda_status(cudaMemcpy(c->d_bvals, c->h_bvals, sizeof(c->h_bvals), cudaMemcpyHostToDevice));
}

int hmr_num_equations(const hmr_ctx* c) { return c ? c->neq : HMR_ERR_ARGUMENT; }
int hmr_num_components(const hmr_ctx* c) { return c ? c->ncomp : HMR_ERR_ARGUMENT; }
int hmr_num_ghosts(const hmr_ctx* c) { return c ? GHOST : HMR_ERR_ARGUMENT; }
int hmr_num_patch_ghosts(const hmr_ctx* c) { return c ? patch_ghosts(c->v) : HMR_ERR_ARGUMENT; }

int hmr_ctx_reserve(hmr_ctx* c, const hmr_patch_geometry* pg) {
    if (!c || !valid_geom(c->v.dim, pg)) return HMR_ERR_ARGUMENT;
    return ensure_scratch(c, make_geom(c->v.dim, pg, patch_ghosts(c->v)));
}

int hmr_read_counters(hmr_ctx* c, unsigned long long out[2], int reset) {
    if (!c || !out) return HMR_ERR_ARGUMENT;
    Counters h;
    cudaError_t e = cudaMemcpy(&h, c->counters, sizeof(h), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_status(e);
    out[0] = h.fallback;
    out[1] = h.hllc_hll;
    if (reset) e = cudaMemset(c->counters, 0, sizeof(Counters));
    return cuda_status(e);
}

// Cells + sensor + faces of one patch into the context scratch (and, with diff, the
// midpoint diffusive fluxes).
static int patch_faces(hmr_ctx* c, const Geom& g, const Comp& Q, Scratch& S, cudaStream_t st, bool diff = false) {
    int r = ensure_scratch(c, g);
    if (r) return r;
    S = carve_scratch(c, g, c->scratch);
    r = hmr_cells::launch_cells(c->v, c->P, g, Q, S, st);
    if (r) return r;
    if (diff) {
        r = diff_launch(c, g, S, st);
        if (r) return r;
    }
    r = hmr_cells::launch_sensor(c->v, g, S, st);
    if (r) return r;
    return face_launch(c, g, S, st);
}

int hmr_conv_flux_source_patch(hmr_ctx* c, const hmr_patch_geometry* pg, const double* const* Q, double dt,
                               double* const* flux, double* const* source, void* stream) {
    if (!c || !valid_geom(c->v.dim, pg)) return HMR_ERR_ARGUMENT;
    Comp q, S;
    FluxComp F;
    if (!load_comp(q, Q, c->ncomp)) return HMR_ERR_ARGUMENT;
    if (!load_flux(F, flux, c->v.dim * c->neq)) return HMR_ERR_ARGUMENT;
    if (!load_comp(S, source, c->neq)) return HMR_ERR_ARGUMENT;
    const Geom g = make_geom(c->v.dim, pg, patch_ghosts(c->v));
    cudaStream_t st = as_stream(stream);
    Scratch scr;
    int r = patch_faces(c, g, q, scr, st);
    if (r) return r;
    UpdateArgs U;
    std::memset(&U, 0, sizeof(U));
    U.Qint[0] = q;
    U.nst = 1;
    U.alpha[0] = 0.0;
    U.beta = 0.0;
    U.dt = dt;
    U.Fout = F;
    U.Sout = S;
    for (int e = 0; e < MAX_COMP; e++) U.Qout.p[e] = nullptr;
    return update_launch(c, g, scr, U, st);
}

int hmr_rk_substep_patch(hmr_ctx* c, const hmr_patch_geometry* pg, int stage, const double* alpha, double beta,
                         const double* const* const* Q_int, double dt, double* const* Q_out, void* stream) {
    if (!c || !valid_geom(c->v.dim, pg) || !alpha || !Q_int || stage < 0 || stage > 2) return HMR_ERR_ARGUMENT;
    UpdateArgs U;
    std::memset(&U, 0, sizeof(U));
    for (int s = 0; s <= stage; s++)
        if (!load_comp(U.Qint[s], Q_int[s], c->ncomp)) return HMR_ERR_ARGUMENT;
    if (!load_comp(U.Qout, Q_out, c->ncomp)) return HMR_ERR_ARGUMENT;
    for (int s = 0; s <= stage; s++) U.alpha[s] = alpha[s];
    U.nst = stage + 1;
    U.beta = beta;
    U.dt = dt;
    for (int e = 0; e < 3 * MAX_COMP; e++) U.Fout.p[e] = nullptr;
    for (int e = 0; e < MAX_COMP; e++) U.Sout.p[e] = nullptr;
    U.dorder = c->P.dorder;
    const Geom g = make_geom(c->v.dim, pg, patch_ghosts(c->v));
    cudaStream_t st = as_stream(stream);
    Scratch scr;
    int r = patch_faces(c, g, U.Qint[stage], scr, st, c->P.dorder != 0);
    if (r) return r;
    return update_launch(c, g, scr, U, st);
}

int hmr_diff_flux_patch(hmr_ctx* c, const hmr_patch_geometry* pg, const double* const* Q, double dt,
                        double* const* flux, void* stream) {
    if (!c || !valid_geom(c->v.dim, pg)) return HMR_ERR_ARGUMENT;
    if (!c->P.dorder) return HMR_ERR_UNSUPPORTED;
    Comp q;
    FluxComp F;
    if (!load_comp(q, Q, c->ncomp)) return HMR_ERR_ARGUMENT;
    if (!load_flux(F, flux, c->v.dim * c->neq)) return HMR_ERR_ARGUMENT;
    const Geom g = make_geom(c->v.dim, pg, patch_ghosts(c->v));
    cudaStream_t st = as_stream(stream);
    int r = ensure_scratch(c, g);
    if (r) return r;
    const Scratch S = carve_scratch(c, g, c->scratch);
    r = hmr_cells::launch_cells(c->v, c->P, g, q, S, st);
    if (r) return r;
    r = diff_launch(c, g, S, st);
    if (r) return r;
    if (c->precision == HMR_PRECISION_EXACT) return hmr_diff_exact::launch_diff_faces_out(c->v, c->P, g, S, dt, F, st);
    return hmr_diff_fast::launch_diff_faces_out(c->v, c->P, g, S, dt, F, st);
}

int hmr_rk_stage_ns_patch(hmr_ctx* c, const hmr_patch_geometry* pg, int ncoef, const double* alpha,
                          const double* beta, const double* gamma, const double* const* const* Q_int,
                          const double* const* const* F_int, const double* const* const* Fd_int,
                          const double* const* const* S_int, double* const* Q, double* const* flux_acc,
                          double* const* diff_flux_acc, double* const* source_acc, void* stream) {
    if (!c || !valid_geom(c->v.dim, pg) || ncoef < 1 || ncoef > 4 || !alpha || !beta) return HMR_ERR_ARGUMENT;
    if (!c->P.dorder) return HMR_ERR_UNSUPPORTED;
    if (!Q_int || !F_int || !Fd_int || !S_int) return HMR_ERR_ARGUMENT;
    Comp Qi[4], Si[4], Qo, Sa;
    FluxComp Fi[4], Di[4], Fa, Da;
    for (int n = 0; n < ncoef; n++) {
        if (!load_comp(Qi[n], Q_int[n], c->ncomp)) return HMR_ERR_ARGUMENT;
        if (!load_flux(Fi[n], F_int[n], c->v.dim * c->neq)) return HMR_ERR_ARGUMENT;
        if (!load_flux(Di[n], Fd_int[n], c->v.dim * c->neq)) return HMR_ERR_ARGUMENT;
        if (!load_comp(Si[n], S_int[n], c->neq)) return HMR_ERR_ARGUMENT;
    }
    if (!load_comp(Qo, Q, c->ncomp)) return HMR_ERR_ARGUMENT;
    const bool acc = flux_acc != nullptr || diff_flux_acc != nullptr || source_acc != nullptr;
    if (acc) {
        if (!gamma || !load_flux(Fa, flux_acc, c->v.dim * c->neq) ||
            !load_flux(Da, diff_flux_acc, c->v.dim * c->neq) || !load_comp(Sa, source_acc, c->neq))
            return HMR_ERR_ARGUMENT;
    } else {
        for (int e = 0; e < 3 * MAX_COMP; e++) Fa.p[e] = Da.p[e] = nullptr;
        for (int e = 0; e < MAX_COMP; e++) Sa.p[e] = nullptr;
    }
    const Geom g = make_geom(c->v.dim, pg, patch_ghosts(c->v));
    return hmr_cells::launch_rk_stage(c->v, g, ncoef, alpha, beta, acc ? gamma : nullptr, Qi, Fi, Si, Qo, Fa, Sa,
                                      as_stream(stream), Di, acc ? &Da : nullptr);
}

int hmr_rk_stage_patch(hmr_ctx* c, const hmr_patch_geometry* pg, int ncoef, const double* alpha,
                       const double* beta, const double* gamma, const double* const* const* Q_int,
                       const double* const* const* F_int, const double* const* const* S_int, double* const* Q,
                       double* const* flux_acc, double* const* source_acc, void* stream) {
    if (!c || !valid_geom(c->v.dim, pg) || ncoef < 1 || ncoef > 4 || !alpha || !beta) return HMR_ERR_ARGUMENT;
    if (!Q_int || !F_int || !S_int) return HMR_ERR_ARGUMENT;
    Comp Qi[4], Si[4], Qo, Sa;
    FluxComp Fi[4], Fa;
    for (int n = 0; n < ncoef; n++) {
        if (!load_comp(Qi[n], Q_int[n], c->ncomp)) return HMR_ERR_ARGUMENT;
        if (!load_flux(Fi[n], F_int[n], c->v.dim * c->neq)) return HMR_ERR_ARGUMENT;
        if (!load_comp(Si[n], S_int[n], c->neq)) return HMR_ERR_ARGUMENT;
    }
    if (!load_comp(Qo, Q, c->ncomp)) return HMR_ERR_ARGUMENT;
    const bool acc = flux_acc != nullptr || source_acc != nullptr;
    if (acc) {
        if (!gamma || !load_flux(Fa, flux_acc, c->v.dim * c->neq) || !load_comp(Sa, source_acc, c->neq))
            return HMR_ERR_ARGUMENT;
    } else {
        for (int e = 0; e < 3 * MAX_COMP; e++) Fa.p[e] = nullptr;
        for (int e = 0; e < MAX_COMP; e++) Sa.p[e] = nullptr;
    }
    const Geom g = make_geom(c->v.dim, pg, patch_ghosts(c->v));
    return hmr_cells::launch_rk_stage(c->v, g, ncoef, alpha, beta, acc ? gamma : nullptr, Qi, Fi, Si, Qo, Fa, Sa,
                                      as_stream(stream));
}

int hmr_rk_substep_vjp_patch(hmr_ctx* c, const hmr_patch_geometry* pg, int stage, const double* alpha,
                             double beta, const double* const* const* Q_int, double dt,
                             const double* const* Qbar_out, double* const* const* Qbar_int, void* stream) {
    if (!c || !valid_geom(c->v.dim, pg) || !alpha || !Q_int || !Qbar_out || !Qbar_int || stage < 0 || stage > 2)
        return HMR_ERR_ARGUMENT;
    VjpArgs A;
    std::memset(&A, 0, sizeof(A));
    if (!load_comp(A.Qs, Q_int[stage], c->ncomp)) return HMR_ERR_ARGUMENT;
    if (!load_comp(A.Qbo, Qbar_out, c->ncomp)) return HMR_ERR_ARGUMENT;
    for (int s = 0; s <= stage; s++)
        if (!load_comp(A.Qbi[s], Qbar_int[s], c->ncomp)) return HMR_ERR_ARGUMENT;
    for (int s = 0; s <= stage; s++) A.alpha[s] = alpha[s];
    A.nst = stage + 1;
    A.beta = beta;
    A.dt = dt;
    const Geom g = make_geom(c->v.dim, pg, patch_ghosts(c->v));
    cudaStream_t st = as_stream(stream);
    int r = ensure_scratch(c, g);
    if (r) return r;
    const Scratch S = carve_scratch(c, g, c->scratch);
    // per face: contributions (6 neq + 2), reconstructed-value adjoints (2 neq) and values
    // (2 neq), smoothness indicators (9 neq), projection factors and their partial
    // adjoints (9 + 4 nsp), bounds flag (1)
    const size_t per_face = (size_t)(6 * c->neq + 2) + (size_t)(2 * c->neq) + (size_t)(2 * c->neq) +
                            (size_t)(9 * c->neq) + (size_t)(9 + 4 * c->v.nsp) + 1;
    size_t need = 0;
    for (int a = 0; a < c->v.dim; a++) need += per_face * nface_of(g, a);
    // Navier-Stokes: midpoint adjoints, node-gradient and primitive-variable adjoints
    const int nmb = c->v.dim + (c->v.dim + 1) + 2 * (c->v.dim - 1);
    if (c->P.dorder) {
        for (int a = 0; a < c->v.dim; a++) need += (size_t)nmb * nface_w(g, a, diff_half_width(c->v));
        need += (size_t)(c->v.dim * c->v.dim + c->neq) * ncell_of(g);
    }
    need *= sizeof(double);
    const size_t rec_bytes = (sizeof(VjpWork) + 255) / 256 * 256;   // the one-patch record, first
    need += rec_bytes;
    if (need > c->vjp_bytes) {
        if (c->vjp) cudaFree(c->vjp);
        c->vjp = nullptr;
        c->vjp_bytes = 0;
        cudaError_t e = cudaMalloc(&c->vjp, need);
        if (e != cudaSuccess) return cuda_status(e);
        c->vjp_bytes = need;
    }
    VjpWork* d_rec = reinterpret_cast<VjpWork*>(c->vjp);
    double* p = reinterpret_cast<double*>(reinterpret_cast<unsigned char*>(c->vjp) + rec_bytes);
    for (int a = 0; a < 3; a++) {
        A.Cb[a] = A.Wb[a] = A.Wv[a] = A.Kb[a] = A.Fp[a] = nullptr;
        A.okf[a] = nullptr;
        if (a >= c->v.dim) continue;
        const long nf = nface_of(g, a);
        A.Cb[a] = p; p += (size_t)(6 * c->neq + 2) * nf;
        A.Wb[a] = p; p += (size_t)(2 * c->neq) * nf;
        A.Wv[a] = p; p += (size_t)(2 * c->neq) * nf;
        A.Kb[a] = p; p += (size_t)(9 * c->neq) * nf;
        A.Fp[a] = p; p += (size_t)(9 + 4 * c->v.nsp) * nf;
        A.okf[a] = reinterpret_cast<unsigned char*>(p); p += nf;   // one double per face reserved
    }
    for (int a = 0; a < 3; a++) A.Mb[a] = nullptr;
    A.Gdb = A.Dv = nullptr;
    if (c->P.dorder) {
        for (int a = 0; a < c->v.dim; a++) {
            A.Mb[a] = p;
            p += (size_t)nmb * nface_w(g, a, diff_half_width(c->v));
        }
        A.Gdb = p; p += (size_t)c->v.dim * c->v.dim * ncell_of(g);
        A.Dv = p; p += (size_t)c->neq * ncell_of(g);
    }
    if (beta != 0.0) {
        r = hmr_cells::launch_cells(c->v, c->P, g, A.Qs, S, st);
        if (r) return r;
        if (c->P.dorder) {
            r = hmr_cells::launch_diff_grad(c->v, c->P, g, S, st);
            if (r) return r;
        }
        r = hmr_cells::launch_sensor(c->v, g, S, st);
        if (r) return r;
    }
    return hmr_vjp::launch_vjp(c->v, c->P, g, S, A, d_rec, st);
}

int hmr_sync_fluxes_patch(hmr_ctx* c, const hmr_patch_geometry* pg, double* const* Q, const double* const* flux,
                          const double* const* diff_flux, const double* const* source, void* stream) {
    if (!c || !valid_geom(c->v.dim, pg)) return HMR_ERR_ARGUMENT;
    if (diff_flux && !c->P.dorder) return HMR_ERR_UNSUPPORTED;
    Comp q, S;
    FluxComp F, D;
    if (!load_comp(q, Q, c->ncomp) || !load_flux(F, flux, c->v.dim * c->neq) || !load_comp(S, source, c->neq))
        return HMR_ERR_ARGUMENT;
    if (diff_flux && !load_flux(D, diff_flux, c->v.dim * c->neq)) return HMR_ERR_ARGUMENT;
    const Geom g = make_geom(c->v.dim, pg, patch_ghosts(c->v));
    return hmr_cells::launch_sync(c->v, g, q, F, diff_flux ? &D : nullptr, S, as_stream(stream));
}

// Placement of a fine patch over a coarse patch; HMR_ERR_ARGUMENT unless the ratio is at
// least 1 and the fine box is aligned with it.
static int coarsen_args(const hmr_ctx* c, const hmr_patch_geometry* coarse, const int* coarse_lo,
                        const hmr_patch_geometry* fine, const int* fine_lo, const int* ratio, CoarsenArgs& C) {
    const int dim = c->v.dim;
    if (!valid_geom(dim, coarse) || !valid_geom(dim, fine) || !coarse_lo || !fine_lo || !ratio)
        return HMR_ERR_ARGUMENT;
    std::memset(&C, 0, sizeof(C));
    C.gc = make_geom(dim, coarse, patch_ghosts(c->v));
    C.gf = make_geom(dim, fine, patch_ghosts(c->v));
    for (int d = 0; d < 3; d++) {
        if (d >= dim) {
            C.r[d] = 1; C.clo[d] = C.flo[d] = 0; C.lo[d] = 0; C.hi[d] = 1;
            continue;
        }
        if (ratio[d] < 1 || ratio[d] > 64) return HMR_ERR_ARGUMENT;
        C.r[d] = ratio[d];
        C.clo[d] = coarse_lo[d];
        C.flo[d] = fine_lo[d];
        const long flo = fine_lo[d], fhi = (long)fine_lo[d] + fine->n[d];
        if (((flo % ratio[d]) + ratio[d]) % ratio[d] != 0 || ((fhi % ratio[d]) + ratio[d]) % ratio[d] != 0)
            return HMR_ERR_ARGUMENT;
        const long lo = std::max<long>(flo / ratio[d], coarse_lo[d]) - coarse_lo[d];
        const long hi = std::min<long>(fhi / ratio[d], (long)coarse_lo[d] + coarse->n[d]) - coarse_lo[d];
        C.lo[d] = (int)lo;
        C.hi[d] = (int)std::max(hi, lo);
    }
    return HMR_OK;
}

int hmr_refine_ghosts_patch(hmr_ctx* c, const hmr_patch_geometry* fine, const int* fine_lo,
                            const hmr_patch_geometry* coarse, const int* coarse_lo, const int* ratio,
                            const double* const* Q_coarse_old, const double* const* Q_coarse_new, double theta,
                            double* const* Q_fine, void* stream) {
    if (!c || !(theta >= 0.0 && theta <= 1.0)) return HMR_ERR_ARGUMENT;
    CoarsenArgs C;
    int r = coarsen_args(c, coarse, coarse_lo, fine, fine_lo, ratio, C);
    if (r) return r;
    Comp qo, qn, qf;
    if (!load_comp(qo, Q_coarse_old, c->ncomp) || !load_comp(qn, Q_coarse_new, c->ncomp) ||
        !load_comp(qf, Q_fine, c->ncomp))
        return HMR_ERR_ARGUMENT;
    return hmr_cells::launch_refine_ghosts(c->v.dim, C, qo, qn, theta, qf, c->ncomp, as_stream(stream));
}

int hmr_coarsen_patch(hmr_ctx* c, const hmr_patch_geometry* coarse, const int* coarse_lo,
                      const hmr_patch_geometry* fine, const int* fine_lo, const int* ratio,
                      const double* const* Q_fine, double* const* Q_coarse, void* stream) {
    if (!c) return HMR_ERR_ARGUMENT;
    CoarsenArgs C;
    int r = coarsen_args(c, coarse, coarse_lo, fine, fine_lo, ratio, C);
    if (r) return r;
    Comp qf, qc;
    if (!load_comp(qf, Q_fine, c->ncomp) || !load_comp(qc, Q_coarse, c->ncomp)) return HMR_ERR_ARGUMENT;
    return hmr_cells::launch_coarsen_cells(c->v.dim, C, qf, qc, c->ncomp, as_stream(stream));
}

int hmr_coarsen_fluxsum_patch(hmr_ctx* c, const hmr_patch_geometry* coarse, const int* coarse_lo,
                              const hmr_patch_geometry* fine, const int* fine_lo, const int* ratio,
                              const double* const* fine_flux, double* const* coarse_flux, void* stream) {
    if (!c) return HMR_ERR_ARGUMENT;
    CoarsenArgs C;
    int r = coarsen_args(c, coarse, coarse_lo, fine, fine_lo, ratio, C);
    if (r) return r;
    FluxComp ff, fc;
    if (!load_flux(ff, fine_flux, c->v.dim * c->neq) || !load_flux(fc, coarse_flux, c->v.dim * c->neq))
        return HMR_ERR_ARGUMENT;
    return hmr_cells::launch_coarsen_fluxsum(c->v.dim, C, ff, fc, c->neq, as_stream(stream));
}

int hmr_spectral_radius_patch(hmr_ctx* c, const hmr_patch_geometry* pg, const double* const* Q, double* d_max,
                              void* stream) {
    if (!c || !valid_geom(c->v.dim, pg) || !d_max) return HMR_ERR_ARGUMENT;
    Comp q;
    if (!load_comp(q, Q, c->ncomp)) return HMR_ERR_ARGUMENT;
    const Geom g = make_geom(c->v.dim, pg, patch_ghosts(c->v));
    return hmr_cells::launch_spectral_patch(c->v, c->P, g, q, reinterpret_cast<unsigned long long*>(d_max),
                                            as_stream(stream));
}

int hmr_fill_ghosts_vjp_patch(hmr_ctx* c, const hmr_patch_geometry* pg, double* const* Qbar, const int* periodic,
                              void* stream) {
    if (!c || !valid_geom(c->v.dim, pg) || !valid_fill_modes(c->v.dim, pg, periodic, patch_ghosts(c->v))) return HMR_ERR_ARGUMENT;
    Comp q;
    if (!load_comp(q, Qbar, c->ncomp)) return HMR_ERR_ARGUMENT;
    const Geom g = make_geom(c->v.dim, pg, patch_ghosts(c->v));
    return hmr_cells::launch_fill_vjp(c->v.dim, g, q, c->ncomp, periodic, momentum0(c->v), as_stream(stream));
}

int hmr_fill_ghosts_patch(hmr_ctx* c, const hmr_patch_geometry* pg, double* const* Q, const int* periodic,
                          void* stream) {
    if (!c || !valid_geom(c->v.dim, pg) || !valid_fill_modes(c->v.dim, pg, periodic, patch_ghosts(c->v))) return HMR_ERR_ARGUMENT;
    Comp q;
    if (!load_comp(q, Q, c->ncomp)) return HMR_ERR_ARGUMENT;
    const Geom g = make_geom(c->v.dim, pg, patch_ghosts(c->v));
    return hmr_cells::launch_fill(c->v.dim, g, q, c->ncomp, periodic, momentum0(c->v), c->d_bvals,
                                  as_stream(stream));
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batched level.
// ---------------------------------------------------------------------------
static const double RK3_ALPHA[3][3] = {{1.0, 0, 0}, {3.0/4.0, 1.0/4.0, 0}, {1.0/3.0, 0.0, 2.0/3.0}};
static const double RK3_BETA[3] = {1.0, 1.0/4.0, 2.0/3.0};

static int level_max_blocks(hmr_level* lv, int threads, int* blocks) {
    hmr_ctx* c = lv->ctx;
    if (c->precision == HMR_PRECISION_EXACT) return hmr_exact::level_max_blocks(c->v, threads, blocks);
    return hmr_fast::level_max_blocks(c->v, threads, blocks);
}

static LevelArgs stage_args(hmr_level* lv, int stage, double dt) {
    LevelArgs L = lv->L;
    L.work = lv->d_work + (size_t)stage * lv->npatch;
    for (int s = 0; s < 3; s++) L.alpha[s] = s <= stage ? RK3_ALPHA[stage][s] : 0.0;
    L.nst = stage + 1;
    L.beta = RK3_BETA[stage];
    L.dt = dt;
    L.dt_dev = nullptr;
    L.exchange = lv->exchange ? 1 : 0;
    L.copies = lv->d_copies;
    L.ncopy = lv->ncopy;
    L.total_copy = lv->total_copy;
    for (int a = 0; a < 3; a++) {
        L.dom[a] = lv->dom[a];
        L.dom_periodic[a] = lv->dom_periodic[a];
    }
    L.barrier = lv->d_barrier;
    L.status = lv->d_status;
    L.redo.list = lv->d_redo;
    L.redo.count = lv->d_barrier + 1;
    L.chunk = lv->d_barrier + 2;
    L.redo.cap = (unsigned long long)lv->redo_cap;
    L.sorted = lv->d_sorted;
    L.sort_count = lv->d_barrier + 10;
    L.sort_off[0] = 0;
    for (int a = 1; a < 3; a++) L.sort_off[a] = L.sort_off[a - 1] + L.total_face[a - 1];
    return L;
}

// Barrier reset + persistent kernel of one substep, enqueued on st.
static int level_enqueue(hmr_level* lv, int stage, double dt, int threads, int blocks, cudaStream_t st) {
    hmr_ctx* c = lv->ctx;
    cudaError_t e = cudaMemsetAsync(lv->d_barrier, 0, LEVEL_COUNTERS * sizeof(unsigned int), st);
    if (e != cudaSuccess) return cuda_status(e);
    const LevelArgs L = stage_args(lv, stage, dt);
    if (c->precision == HMR_PRECISION_EXACT) return hmr_exact::launch_level(c->v, c->P, L, blocks, threads, st);
    return hmr_fast::launch_level(c->v, c->P, L, blocks, threads, st);
}

// Rebuilds the three per-stage worklists (they differ only in the output slot) and uploads them.
static int level_upload(hmr_level* lv) {
    std::vector<PatchWork> all((size_t)3 * lv->npatch);
    for (int s = 0; s < 3; s++) {
        const int out_slot = s == 2 ? 0 : s + 1;
        for (int p = 0; p < lv->npatch; p++) {
            PatchWork w = lv->work[p];
            w.Qout = w.Q[out_slot];
            all[(size_t)s * lv->npatch + p] = w;
        }
    }
    cudaError_t e = cudaMemcpy(lv->d_work, all.data(), all.size() * sizeof(PatchWork), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_status(e);
    lv->dirty = false;
    for (int s = 0; s < 3; s++) lv->graph_ok[s] = false;
    return HMR_OK;
}

static void level_drop_graphs(hmr_level* lv) {
    for (int s = 0; s < 3; s++) {
        if (lv->graph[s]) cudaGraphExecDestroy(lv->graph[s]);
        lv->graph[s] = nullptr;
        lv->graph_ok[s] = false;
    }
    if (lv->cfl_graph) cudaGraphExecDestroy(lv->cfl_graph);
    lv->cfl_graph = nullptr;
}

// Captures (memset + persistent kernel) of one substep into a graph.
static int level_capture(hmr_level* lv, int stage, double dt) {
    if (lv->graph[stage]) {
        cudaGraphExecDestroy(lv->graph[stage]);
        lv->graph[stage] = nullptr;
    }
    cudaStream_t cs;
    cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_status(e);
    cudaGraph_t graph = nullptr;
    int r = cuda_status(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    if (r == HMR_OK) {
        r = level_enqueue(lv, stage, dt, lv->threads, lv->blocks, cs);
        cudaError_t e2 = cudaStreamEndCapture(cs, &graph);
        if (r == HMR_OK && e2 != cudaSuccess) r = cuda_status(e2);
    }
    if (r == HMR_OK) {
        e = cudaGraphInstantiate(&lv->graph[stage], graph, 0);
        if (e != cudaSuccess) r = cuda_status(e);
    }
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(cs);
    if (r == HMR_OK) {
        lv->graph_ok[stage] = true;
        lv->graph_dt[stage] = dt;
    }
    return r;
}

extern "C" {

int hmr_level_create(hmr_ctx* c, int np, const hmr_patch_geometry* geoms, hmr_level** out) {
    if (!c || np < 1 || !geoms || !out) return HMR_ERR_ARGUMENT;
    *out = nullptr;
    for (int p = 0; p < np; p++)
        if (!valid_geom(c->v.dim, &geoms[p])) return HMR_ERR_ARGUMENT;
    hmr_level* lv = new (std::nothrow) hmr_level();
    if (!lv) return HMR_ERR_ARGUMENT;
    lv->ctx = c;
    lv->npatch = np;
    size_t state_tot = 0, scratch_tot = 0;
    std::vector<size_t> scr_off(np);
    long off_fill = 0, off_cells = 0, off_sensor = 0, off_face[3] = {0, 0, 0}, off_dface[3] = {0, 0, 0};
    long off_update = 0;
    lv->work.resize(np);
    for (int p = 0; p < np; p++) {
        const Geom g = make_geom(c->v.dim, &geoms[p], patch_ghosts(c->v));
        lv->geoms.push_back(g);
        lv->state_off.push_back(state_tot);
        state_tot += (size_t)2 * c->ncomp * ncell_of(g);
        scr_off[p] = scratch_tot;
        scratch_tot += (scratch_doubles(c, g) + 31) / 32 * 32;
        PatchWork& w = lv->work[p];
        w.g = g;
        for (int a = 0; a < 3; a++) {
            w.periodic[a] = 0;
            w.lo[a] = 0;
        }
        w.off_fill = off_fill;
        off_fill += ncell_of(g);
        w.off_cells = off_cells;
        off_cells += ncell_of(g);
        w.off_sensor = off_sensor;
        off_sensor += (long)(g.n[0] + 4) * (g.n[1] + 4) * (c->v.dim == 3 ? g.n[2] + 4 : 1);
        for (int a = 0; a < 3; a++) {
            w.off_face[a] = off_face[a];
            w.off_dface[a] = off_dface[a];
            if (a < c->v.dim) {
                off_face[a] += nface_of(g, a);
                off_dface[a] += nface_w(g, a, diff_half_width(c->v));
            }
        }
        w.off_update = off_update;
        off_update += ninterior_of(g);
        lv->redo_cap += total_faces(c, g);
    }
    cudaError_t e = cudaMalloc(&lv->d_state, state_tot * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&lv->d_redo, (size_t)lv->redo_cap * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(&lv->d_sorted, (size_t)lv->redo_cap * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(lv->d_state, 0, state_tot * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&lv->d_scratch, scratch_tot * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&lv->d_work, (size_t)3 * np * sizeof(PatchWork));
    if (e == cudaSuccess) e = cudaMalloc(&lv->d_barrier, LEVEL_COUNTERS * sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMalloc(&lv->d_status, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(lv->d_status, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&lv->d_srmax, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(&lv->d_dt, sizeof(double));
    if (e != cudaSuccess) {
        hmr_level_destroy(lv);
        return cuda_status(e);
    }
    for (int p = 0; p < np; p++) {
        PatchWork& w = lv->work[p];
        const long nc = ncell_of(w.g);
        w.S = carve_scratch(c, w.g, lv->d_scratch + scr_off[p]);
        for (int comp = 0; comp < MAX_COMP; comp++) w.Q[0].p[comp] = nullptr;
        for (int s = 1; s < 3; s++)
            for (int comp = 0; comp < MAX_COMP; comp++)
                w.Q[s].p[comp] = comp < c->ncomp
                    ? lv->d_state + lv->state_off[p] + (size_t)(s - 1) * c->ncomp * nc + (size_t)comp * nc
                    : nullptr;
        w.Qout = w.Q[1];
    }
    lv->L.npatch = np;
    lv->L.ncomp = c->ncomp;
    lv->L.total_fill = off_fill;
    lv->L.total_cells = off_cells;
    lv->L.total_sensor = off_sensor;
    for (int a = 0; a < 3; a++) {
        lv->L.total_face[a] = off_face[a];
        lv->L.total_dface[a] = off_dface[a];
    }
    lv->L.total_update = off_update;
    lv->L.timeout_ns = 2000000000ull;
    lv->L.barrier_extra = 0;
    lv->L.chunk_mult = 1;
    lv->L.split_mode = 0;
    lv->L.mom0 = momentum0(c->v);
    lv->L.bvals = c->d_bvals;
    lv->threads = 128;
    int r = level_max_blocks(lv, lv->threads, &lv->blocks);
    if (r || lv->blocks < 1) {
        hmr_level_destroy(lv);
        return r ? r : HMR_ERR_UNSUPPORTED;
    }
    *out = lv;
    return HMR_OK;
}

int hmr_level_destroy(hmr_level* lv) {
    if (!lv) return HMR_ERR_ARGUMENT;
    level_drop_graphs(lv);
    if (lv->d_state) cudaFree(lv->d_state);
    if (lv->d_scratch) cudaFree(lv->d_scratch);
    if (lv->d_work) cudaFree(lv->d_work);
    if (lv->d_barrier) cudaFree(lv->d_barrier);
    if (lv->d_status) cudaFree(lv->d_status);
    if (lv->d_redo) cudaFree(lv->d_redo);
    if (lv->d_sorted) cudaFree(lv->d_sorted);
    if (lv->d_srmax) cudaFree(lv->d_srmax);
    if (lv->d_copies) cudaFree(lv->d_copies);
    if (lv->d_dt) cudaFree(lv->d_dt);
    if (lv->d_vjp) cudaFree(lv->d_vjp);
    if (lv->d_vjpwork) cudaFree(lv->d_vjpwork);
    if (lv->d_fillvjp) cudaFree(lv->d_fillvjp);
    delete lv;
    return HMR_OK;
}

int hmr_level_bind_state(hmr_level* lv, int p, double* const* comps) {
    if (!lv || p < 0 || p >= lv->npatch) return HMR_ERR_ARGUMENT;
    Comp q;
    if (!load_comp(q, comps, lv->ctx->ncomp)) return HMR_ERR_ARGUMENT;
    if (lv->work[p].Q[0].p[0] == nullptr) lv->bound++;
    lv->work[p].Q[0] = q;
    lv->dirty = true;
    return HMR_OK;
}

int hmr_level_set_periodic(hmr_level* lv, int p, const int* periodic) {
    if (!lv || p < 0 || p >= lv->npatch || !periodic) return HMR_ERR_ARGUMENT;
    for (int a = 0; a < 3; a++) {
        if (a < lv->ctx->v.dim && (periodic[a] < HMR_FILL_ZERO_GRADIENT || periodic[a] > HMR_FILL_SYMMETRY))
            return HMR_ERR_ARGUMENT;
        if (a < lv->ctx->v.dim && (periodic[a] == HMR_FILL_REFLECT || periodic[a] == HMR_FILL_SYMMETRY) &&
            lv->geoms[p].n[a] < lv->geoms[p].gh)
            return HMR_ERR_ARGUMENT;
        lv->work[p].periodic[a] = a < lv->ctx->v.dim ? periodic[a] : 0;
    }
    lv->dirty = true;
    return HMR_OK;
}

int hmr_level_set_layout(hmr_level* lv, const int* lo, const int* domain, const int* periodic) {
    if (!lv || !lo || !domain || !periodic) return HMR_ERR_ARGUMENT;
    const int dim = lv->ctx->v.dim;
    const int gh = patch_ghosts(lv->ctx->v);
    int dom[3] = {1, 1, 1}, per[3] = {0, 0, 0};
    for (int a = 0; a < dim; a++) {
        if (domain[a] < 1 || (periodic[a] != 0 && periodic[a] != 1 && periodic[a] != HMR_FILL_REFLECT &&
                              periodic[a] != HMR_FILL_DIRICHLET && periodic[a] != HMR_FILL_SYMMETRY))
            return HMR_ERR_ARGUMENT;
        // the mirror images of a reflecting wall's ghost cells lie in the domain
        if ((periodic[a] == HMR_FILL_REFLECT || periodic[a] == HMR_FILL_SYMMETRY) && domain[a] < gh)
            return HMR_ERR_ARGUMENT;
        dom[a] = domain[a];
        per[a] = periodic[a];
    }
    const int np = lv->npatch;
    // boxes in the level's index space; they must lie in the domain and not overlap
    std::vector<std::array<int, 3>> blo(np), bhi(np);
    for (int p = 0; p < np; p++) {
        for (int a = 0; a < 3; a++) {
            blo[p][a] = a < dim ? lo[3 * p + a] : 0;
            bhi[p][a] = blo[p][a] + lv->geoms[p].n[a];
            if (blo[p][a] < 0 || bhi[p][a] > dom[a]) return HMR_ERR_ARGUMENT;
        }
    }
    for (int p = 0; p < np; p++)
        for (int q = p + 1; q < np; q++) {
            bool overlap = true;
            for (int a = 0; a < dim; a++) overlap = overlap && blo[p][a] < bhi[q][a] && blo[q][a] < bhi[p][a];
            if (overlap) return HMR_ERR_ARGUMENT;
        }
    // ghost-cell copies: the ghost box of every patch against the interior of every patch
    // and of its periodic images
    std::vector<GhostCopy> copies;
    long total = 0;
    int kmax[3] = {0, 0, 0};
    for (int a = 0; a < dim; a++)
        if (per[a] == 1) kmax[a] = (gh + dom[a] - 1) / dom[a];
    for (int p = 0; p < np; p++) {
        int glo[3], ghi[3];
        for (int a = 0; a < 3; a++) {
            glo[a] = a < dim ? blo[p][a] - gh : 0;
            ghi[a] = a < dim ? bhi[p][a] + gh : 1;
        }
        for (int q = 0; q < np; q++)
            for (int k0 = -kmax[0]; k0 <= kmax[0]; k0++)
                for (int k1 = -kmax[1]; k1 <= kmax[1]; k1++)
                    for (int k2 = -kmax[2]; k2 <= kmax[2]; k2++) {
                        const int sh[3] = {k0 * dom[0], k1 * dom[1], k2 * dom[2]};
                        if (q == p && k0 == 0 && k1 == 0 && k2 == 0) continue;
                        GhostCopy cp;
                        bool empty = false;
                        for (int a = 0; a < 3; a++) {
                            const int il = std::max(glo[a], blo[q][a] + sh[a]);
                            const int ih = std::min(ghi[a], bhi[q][a] + sh[a]);
                            if (ih <= il) { empty = true; break; }
                            cp.dlo[a] = il - blo[p][a];
                            cp.slo[a] = il - (blo[q][a] + sh[a]);
                            cp.ext[a] = ih - il;
                        }
                        if (empty) continue;
                        cp.dst = p;
                        cp.src = q;
                        cp.off = total;
                        total += (long)cp.ext[0] * cp.ext[1] * cp.ext[2];
                        copies.push_back(cp);
                    }
    }
    if (lv->d_copies) cudaFree(lv->d_copies);
    lv->d_copies = nullptr;
    lv->ncopy = (int)copies.size();
    lv->total_copy = total;
    if (!copies.empty()) {
        cudaError_t e = cudaMalloc(&lv->d_copies, copies.size() * sizeof(GhostCopy));
        if (e == cudaSuccess)
            e = cudaMemcpy(lv->d_copies, copies.data(), copies.size() * sizeof(GhostCopy), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_status(e);
    }
    for (int p = 0; p < np; p++)
        for (int a = 0; a < 3; a++) lv->work[p].lo[a] = blo[p][a];
    for (int a = 0; a < 3; a++) {
        lv->dom[a] = dom[a];
        lv->dom_periodic[a] = per[a];
    }
    lv->exchange = true;
    lv->dirty = true;
    level_drop_graphs(lv);
    return HMR_OK;
}

int hmr_level_state(hmr_level* lv, int p, int slot, double** comps_out) {
    if (!lv || p < 0 || p >= lv->npatch || slot < 0 || slot > 2 || !comps_out) return HMR_ERR_ARGUMENT;
    for (int e = 0; e < lv->ctx->ncomp; e++) comps_out[e] = lv->work[p].Q[slot].p[e];
    return HMR_OK;
}

// Doubles of the per-face reverse buffers of one patch's substep VJP (Euler equations): per face
// the contributions (6 neq + 2), reconstructed-value adjoints (2 neq) and values (2 neq),
// smoothness indicators (9 neq), projection factors and their partial adjoints (9 + 4 nsp) and
// the bounds flag (one double reserved).
static size_t vjp_face_doubles(const hmr_ctx* c) {
    return (size_t)(6 * c->neq + 2) + (size_t)(2 * c->neq) + (size_t)(2 * c->neq) + (size_t)(9 * c->neq) +
           (size_t)(9 + 4 * c->v.nsp) + 1;
}

int hmr_level_set_vjp_budget(hmr_level* lv, unsigned long long bytes) {
    if (!lv) return HMR_ERR_ARGUMENT;
    lv->vjp_budget = (size_t)bytes;
    return HMR_OK;
}

int hmr_level_fill_vjp(hmr_level* lv, double* const* const* Qbar, void* stream) {
    if (!lv || !Qbar) return HMR_ERR_ARGUMENT;
    hmr_ctx* c = lv->ctx;
    const int np = lv->npatch;
    const int mom0 = momentum0(c->v);
    cudaStream_t st = as_stream(stream);
    std::vector<Comp> qb(np);
    for (int p = 0; p < np; p++)
        if (!Qbar[p] || !load_comp(qb[p], Qbar[p], c->ncomp)) return HMR_ERR_ARGUMENT;
    if (!lv->exchange) {
        // each patch's own fill (hmr_level_set_periodic modes)
        for (int p = 0; p < np; p++) {
            int r = hmr_cells::launch_fill_vjp(c->v.dim, lv->geoms[p], qb[p], c->ncomp, lv->work[p].periodic, mom0, st);
            if (r) return r;
        }
        return HMR_OK;
    }
    std::vector<hmr_cells::LevelFillVjpPatch> rec(np);
    long total = 0;
    for (int p = 0; p < np; p++) {
        rec[p].g = lv->geoms[p];
        rec[p].Qb = qb[p];
        for (int a = 0; a < 3; a++) rec[p].lo[a] = lv->work[p].lo[a];
        rec[p].off = total;
        total += ncell_of(lv->geoms[p]);
    }
    if (!lv->d_fillvjp) {
        cudaError_t e = cudaMalloc(&lv->d_fillvjp, (size_t)np * sizeof(hmr_cells::LevelFillVjpPatch));
        if (e != cudaSuccess) return cuda_status(e);
    }
    cudaError_t e = cudaMemcpyAsync(lv->d_fillvjp, rec.data(), (size_t)np * sizeof(hmr_cells::LevelFillVjpPatch),
                                    cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_status(e);
    return hmr_cells::launch_level_fill_vjp(c->v.dim, lv->d_fillvjp, np, total, lv->d_copies, lv->ncopy,
                                            lv->total_copy, c->ncomp, lv->dom, lv->dom_periodic, mom0, st);
}

int hmr_level_substep_vjp(hmr_level* lv, int stage, double dt, const double* const* const* Qbar_out,
                          double* const* const* const* Qbar_int, void* stream) {
    if (!lv || stage < 0 || stage > 2 || !Qbar_out || !Qbar_int) return HMR_ERR_ARGUMENT;
    hmr_ctx* c = lv->ctx;
    if (lv->bound != lv->npatch) return HMR_ERR_STATE;
    const int np = lv->npatch;
    const double beta = RK3_BETA[stage];
    const size_t per_face = vjp_face_doubles(c);
    // Navier-Stokes: midpoint adjoints, node-gradient and primitive-variable adjoints
    const int nmb = c->v.dim + (c->v.dim + 1) + 2 * (c->v.dim - 1);
    // per-patch buffer sizes (doubles, rounded to 32 for alignment)
    std::vector<size_t> need(np);
    size_t largest = 0, total = 0;
    for (int p = 0; p < np; p++) {
        size_t n = 0;
        for (int a = 0; a < c->v.dim; a++) n += per_face * nface_of(lv->geoms[p], a);
        if (c->P.dorder) {
            for (int a = 0; a < c->v.dim; a++) n += (size_t)nmb * nface_w(lv->geoms[p], a, diff_half_width(c->v));
            n += (size_t)(c->v.dim * c->v.dim + c->neq) * ncell_of(lv->geoms[p]);
        }
        need[p] = (n + 31) / 32 * 32;
        largest = std::max(largest, need[p]);
        total += need[p];
    }
    if (lv->vjp_budget == 0) {
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
            cudaGetLastError();
            free_b = (size_t)1 << 32;
        }
        lv->vjp_budget = free_b / 4;
    }
    const size_t cap = std::max(largest, std::min(total, lv->vjp_budget / sizeof(double)));
    if (cap * sizeof(double) > lv->vjp_bytes) {
        if (lv->d_vjp) cudaFree(lv->d_vjp);
        lv->d_vjp = nullptr;
        lv->vjp_bytes = 0;
        cudaError_t e = cudaMalloc(&lv->d_vjp, cap * sizeof(double));
        if (e != cudaSuccess) return cuda_status(e);
        lv->vjp_bytes = cap * sizeof(double);
    }
    if (!lv->d_vjpwork) {
        cudaError_t e = cudaMalloc(&lv->d_vjpwork, (size_t)np * sizeof(VjpWork));
        if (e != cudaSuccess) return cuda_status(e);
    }
    // records: each patch's buffers at its offset inside its group's share of d_vjp, prefix
    // offsets of its items relative to the first patch of its group
    std::vector<VjpWork> work(np);
    std::vector<int> group_first;
    std::vector<std::array<long, VJP_NPH * 3>> group_totals;
    size_t used = 0;
    std::array<long, VJP_NPH * 3> acc{};
    for (int p = 0; p < np; p++) {
        if (p == 0 || used + need[p] > cap) {
            if (p > 0) group_totals.push_back(acc);
            group_first.push_back(p);
            used = 0;
            acc.fill(0);
        }
        VjpWork& w = work[p];
        std::memset(&w, 0, sizeof(w));
        const Geom& g = lv->geoms[p];
        w.g = g;
        w.S = lv->work[p].S;
        VjpArgs& A = w.A;
        A.Qs = lv->work[p].Q[stage];
        if (!Qbar_out[p] || !load_comp(A.Qbo, Qbar_out[p], c->ncomp) || !Qbar_int[p]) return HMR_ERR_ARGUMENT;
        for (int st = 0; st <= stage; st++)
            if (!load_comp(A.Qbi[st], Qbar_int[p][st], c->ncomp)) return HMR_ERR_ARGUMENT;
        for (int st = 0; st < 3; st++) A.alpha[st] = st <= stage ? RK3_ALPHA[stage][st] : 0.0;
        A.nst = stage + 1;
        A.beta = beta;
        A.dt = dt;
        double* q = lv->d_vjp + used;
        for (int a = 0; a < c->v.dim; a++) {
            const long nf = nface_of(g, a);
            A.Cb[a] = q; q += (size_t)(6 * c->neq + 2) * nf;
            A.Wb[a] = q; q += (size_t)(2 * c->neq) * nf;
            A.Wv[a] = q; q += (size_t)(2 * c->neq) * nf;
            A.Kb[a] = q; q += (size_t)(9 * c->neq) * nf;
            A.Fp[a] = q; q += (size_t)(9 + 4 * c->v.nsp) * nf;
            A.okf[a] = reinterpret_cast<unsigned char*>(q); q += nf;
        }
        if (c->P.dorder) {
            for (int a = 0; a < c->v.dim; a++) {
                A.Mb[a] = q;
                q += (size_t)nmb * nface_w(g, a, diff_half_width(c->v));
            }
            A.Gdb = q; q += (size_t)c->v.dim * c->v.dim * ncell_of(g);
            A.Dv = q; q += (size_t)c->neq * ncell_of(g);
        }
        used += need[p];
        long items[VJP_NPH * 3];
        vjp_item_counts(c->v, g, items);
        for (int k = 0; k < VJP_NPH * 3; k++) {
            w.off[k] = acc[k];
            acc[k] += items[k];
        }
    }
    group_totals.push_back(acc);
    if (lv->dirty) {
        int r = level_upload(lv);
        if (r) return r;
    }
    cudaStream_t st = as_stream(stream);
    if (beta != 0.0) {
        // the forward values the reverse sweep starts from: cell data and sensor of slot `stage`
        // (the exact-form cell unit, as the forward computes them)
        int r = hmr_cells::launch_cells_level(c->v, c->P, lv->d_work, np, lv->L.total_cells, stage, st);
        if (r) return r;
        if (c->P.dorder) {
            r = hmr_cells::launch_diff_grad_level(c->v, c->P, lv->d_work, np, lv->L.total_cells, st);
            if (r) return r;
        }
        r = hmr_cells::launch_sensor_level(c->v, lv->d_work, np, lv->L.total_sensor, st);
        if (r) return r;
    }
    cudaError_t e = cudaMemcpyAsync(lv->d_vjpwork, work.data(), (size_t)np * sizeof(VjpWork),
                                    cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_status(e);
    const size_t ng = group_first.size();
    for (size_t k = 0; k < ng; k++) {
        const int first = group_first[k];
        const int count = (k + 1 < ng ? group_first[k + 1] : np) - first;
        const int r = hmr_vjp::launch_vjp_level(c->v, c->P, lv->d_vjpwork + first, count, group_totals[k].data(),
                                                beta != 0.0, st);
        if (r) return r;
    }
    return HMR_OK;
}

int hmr_level_substep(hmr_level* lv, int stage, double dt, void* stream) {
    if (!lv || stage < 0 || stage > 2) return HMR_ERR_ARGUMENT;
    if (lv->bound != lv->npatch) return HMR_ERR_STATE;
    if (lv->dirty) {
        int r = level_upload(lv);
        if (r) return r;
    }
    if (!lv->graph_ok[stage] || lv->graph_dt[stage] != dt) {
        int r = level_capture(lv, stage, dt);
        if (r) return r;
    }
    return cuda_status(cudaGraphLaunch(lv->graph[stage], as_stream(stream)));
}

int hmr_level_step(hmr_level* lv, double dt, void* stream) {
    for (int s = 0; s < 3; s++) {
        int r = hmr_level_substep(lv, s, dt, stream);
        if (r) return r;
    }
    return HMR_OK;
}

// One graph: running max of the spectral radius over the slot-0 states -> dt = (1/max)*cfl on
// the device -> the three substeps reading that dt.
static int level_capture_cfl(hmr_level* lv, double cfl) {
    if (lv->cfl_graph) {
        cudaGraphExecDestroy(lv->cfl_graph);
        lv->cfl_graph = nullptr;
    }
    hmr_ctx* c = lv->ctx;
    cudaStream_t cs;
    cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_status(e);
    cudaGraph_t graph = nullptr;
    int r = cuda_status(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    if (r == HMR_OK) {
        r = cuda_status(cudaMemsetAsync(lv->d_srmax, 0, sizeof(unsigned long long), cs));
        if (r == HMR_OK)
            r = hmr_cells::launch_spectral_level(c->v, c->P, lv->d_work, lv->npatch, lv->L.total_cells,
                                                 lv->d_srmax, cs);
        if (r == HMR_OK) r = hmr_cells::launch_stable_dt(lv->d_srmax, cfl, lv->d_dt, cs, c->P.dorder != 0);
        for (int stage = 0; stage < 3 && r == HMR_OK; stage++) {
            r = cuda_status(cudaMemsetAsync(lv->d_barrier, 0, LEVEL_COUNTERS * sizeof(unsigned int), cs));
            if (r != HMR_OK) break;
            LevelArgs L = stage_args(lv, stage, 0.0);
            L.dt_dev = lv->d_dt;
            r = c->precision == HMR_PRECISION_EXACT
                ? hmr_exact::launch_level(c->v, c->P, L, lv->blocks, lv->threads, cs)
                : hmr_fast::launch_level(c->v, c->P, L, lv->blocks, lv->threads, cs);
        }
        cudaError_t e2 = cudaStreamEndCapture(cs, &graph);
        if (r == HMR_OK && e2 != cudaSuccess) r = cuda_status(e2);
    }
    if (r == HMR_OK) {
        e = cudaGraphInstantiate(&lv->cfl_graph, graph, 0);
        if (e != cudaSuccess) r = cuda_status(e);
    }
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(cs);
    if (r == HMR_OK) lv->cfl_graph_cfl = cfl;
    return r;
}

int hmr_level_step_cfl(hmr_level* lv, double cfl, void* stream) {
    if (!lv || !(cfl > 0.0)) return HMR_ERR_ARGUMENT;
    if (lv->bound != lv->npatch) return HMR_ERR_STATE;
    if (lv->dirty) {
        int r = level_upload(lv);
        if (r) return r;
        if (lv->cfl_graph) {
            cudaGraphExecDestroy(lv->cfl_graph);
            lv->cfl_graph = nullptr;
        }
    }
    if (!lv->cfl_graph || lv->cfl_graph_cfl != cfl) {
        int r = level_capture_cfl(lv, cfl);
        if (r) return r;
    }
    return cuda_status(cudaGraphLaunch(lv->cfl_graph, as_stream(stream)));
}

int hmr_level_last_dt(hmr_level* lv, double* dt) {
    if (!lv || !dt) return HMR_ERR_ARGUMENT;
    return cuda_status(cudaMemcpy(dt, lv->d_dt, sizeof(double), cudaMemcpyDeviceToHost));
}

int hmr_level_check(hmr_level* lv) {
    if (!lv) return HMR_ERR_ARGUMENT;
    int status = 0;
    cudaError_t e = cudaMemcpy(&status, lv->d_status, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_status(e);
    if (status) {
        e = cudaMemset(lv->d_status, 0, sizeof(int));
        if (e != cudaSuccess) return cuda_status(e);
        return HMR_ERR_BARRIER;
    }
    return HMR_OK;
}

int hmr_level_barrier_diagnostic(hmr_level* lv, unsigned int extra_arrivals, unsigned long long timeout_ns) {
    if (!lv || timeout_ns == 0 || timeout_ns > 10000000000ull || extra_arrivals > 1) return HMR_ERR_ARGUMENT;
    lv->L.barrier_extra = extra_arrivals;
    lv->L.timeout_ns = timeout_ns;
    level_drop_graphs(lv);
    return HMR_OK;
}

int hmr_level_set_launch(hmr_level* lv, int threads, int blocks_per_sm) {
    if (!lv || (threads != 64 && threads != 128) || blocks_per_sm < 1) return HMR_ERR_ARGUMENT;
    int dev = 0, sms = 1, maxb = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int r = level_max_blocks(lv, threads, &maxb);
    if (r) return r;
    if (blocks_per_sm * sms > maxb) return HMR_ERR_ARGUMENT;   // more than can be resident
    if (threads != lv->threads || blocks_per_sm * sms != lv->blocks) level_drop_graphs(lv);
    lv->threads = threads;
    lv->blocks = blocks_per_sm * sms;
    return HMR_OK;
}

int hmr_level_set_work_split(hmr_level* lv, int chunk_blocks, int mode) {
    if (!lv || (chunk_blocks != 1 && chunk_blocks != 2 && chunk_blocks != 4) || mode < 0 || mode > 3)
        return HMR_ERR_ARGUMENT;
    if (chunk_blocks != lv->L.chunk_mult || mode != lv->L.split_mode) level_drop_graphs(lv);
    lv->L.chunk_mult = chunk_blocks;
    lv->L.split_mode = mode;
    return HMR_OK;
}

int hmr_level_work_split(hmr_level* lv, int* chunk_blocks, int* mode) {
    if (!lv || !chunk_blocks || !mode) return HMR_ERR_ARGUMENT;
    *chunk_blocks = lv->L.chunk_mult;
    *mode = lv->L.split_mode;
    return HMR_OK;
}

int hmr_level_autotune(hmr_level* lv, double dt, int* threads_out, int* bpsm_out, void* stream) {
    if (!lv) return HMR_ERR_ARGUMENT;
    if (lv->bound != lv->npatch) return HMR_ERR_STATE;
    if (lv->dirty) {
        int r = level_upload(lv);
        if (r) return r;
    }
    cudaStream_t st = as_stream(stream);
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int cand_threads[2] = {64, 128};   // the level kernel's launch bound is 128 threads
    // launch shapes first, with one-block chunks for every phase
    const int mult0 = lv->L.chunk_mult, mode0 = lv->L.split_mode;
    lv->L.chunk_mult = 1;
    lv->L.split_mode = 0;
    float best = 1e30f;
    int best_t = lv->threads, best_b = lv->blocks;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (int ti = 0; ti < 2; ti++) {
        const int t = cand_threads[ti];
        int maxb = 0;
        if (level_max_blocks(lv, t, &maxb) || maxb < 1) continue;
        const int max_per_sm = std::max(1, maxb / sms);
        for (int bps = 1; bps <= max_per_sm; bps++) {
            // Substep 0 reads slot 0 and writes slot 1: repeated launches leave the state unchanged.
            if (level_enqueue(lv, 0, dt, t, bps * sms, st)) continue;
            cudaEventRecord(e0, st);
            for (int rep = 0; rep < 2; rep++) level_enqueue(lv, 0, dt, t, bps * sms, st);
            cudaEventRecord(e1, st);
            if (cudaEventSynchronize(e1) != cudaSuccess) continue;
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best) {
                best = ms;
                best_t = t;
                best_b = bps * sms;
            }
        }
    }
    // then the work splitting at the chosen shape: chunk width (1, 2, 4 block widths) and the
    // hand-out of the cell-wise phases (chunks or grid stride)
    int best_m = 1, best_s = 0;
    const int splits[4][2] = {{1, 0}, {2, 0}, {4, 0}, {1, 1}};
    for (int k = 0; k < 4; k++) {
        lv->L.chunk_mult = splits[k][0];
        lv->L.split_mode = splits[k][1];
        if (level_enqueue(lv, 0, dt, best_t, best_b, st)) continue;
        cudaEventRecord(e0, st);
        for (int rep = 0; rep < 2; rep++) level_enqueue(lv, 0, dt, best_t, best_b, st);
        cudaEventRecord(e1, st);
        if (cudaEventSynchronize(e1) != cudaSuccess) continue;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (k == 0 || ms < best) {
            best = ms;
            best_m = splits[k][0];
            best_s = splits[k][1];
        }
    }
    // and, in the fast form, the faces sorted by their sensor first (split_mode bit 1)
    if (lv->ctx->precision == HMR_PRECISION_FAST) {
        lv->L.chunk_mult = best_m;
        lv->L.split_mode = best_s | 2;
        if (level_enqueue(lv, 0, dt, best_t, best_b, st) == HMR_OK) {
            cudaEventRecord(e0, st);
            for (int rep = 0; rep < 2; rep++) level_enqueue(lv, 0, dt, best_t, best_b, st);
            cudaEventRecord(e1, st);
            float ms = 0.f;
            if (cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess &&
                ms < best)
                best_s |= 2;
        }
    }
    lv->L.chunk_mult = best_m;
    lv->L.split_mode = best_s;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (best_t != lv->threads || best_b != lv->blocks || best_m != mult0 || best_s != mode0) level_drop_graphs(lv);
    lv->threads = best_t;
    lv->blocks = best_b;
    if (threads_out) *threads_out = best_t;
    if (bpsm_out) *bpsm_out = best_b / sms;
    return hmr_level_check(lv);
}

}  // extern "C"
