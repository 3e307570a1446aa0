// hmr_rk_substep_patch_noalloc: the fused per-patch flux + stage update with
// no device allocation of any kind (contract in include/hmr.h).
//
// Its scratch (cell data, midpoint fluxes, the queue of faces handed to the
// exact form) lives in one file-scope __device__ array of
// HMR_NOALLOC_SCRATCH_BYTES.  Every GPU that loads the library holds that
// array until the process exits.  Host code must not use the array's name as
// a device address: the address is obtained with cudaGetSymbolAddress once
// per device and CUDA context (with that device current) and cached.
#include <cuda.h>            // CUcontext and the driver's function types only; libcuda is not linked
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "../../include/hmr.h"
#include "hmr_launch.h"

using namespace hmr;

namespace {

constexpr size_t kScratchBytes = (size_t)HMR_NOALLOC_SCRATCH_BYTES;
constexpr size_t kHeaderBytes = 256;   // redo-queue length lives here
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mu;

// A symbol's device address belongs to the CUDA context that loaded the module, not to the
// device: after cudaDeviceReset, or under a driver-API context of the host's own, the array
// has another address.  Each cached address therefore carries the id of the context it was
// resolved in (cuCtxGetId: unique for the life of the process) and is resolved again when
// the current context's id differs.
struct Slot {
    void* addr = nullptr;
    unsigned long long ctx_id = 0;
};
Slot g_slot[kMaxDevices];

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

// Id of the current context, or 0 when none is current or the driver cannot say.
unsigned long long current_context_id() {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static bool looked_up = false;
    if (!looked_up) {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<CtxGetCurrentFn>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetIdFn>(f);
        cudaGetLastError();
        looked_up = true;
    }
    if (!get_current || !get_id) return 0;
    CUcontext ctx = nullptr;
    if (get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr) return 0;
    unsigned long long id = 0;
    if (get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Device address of the scratch array in the current device's current context.
int scratch_address(void** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return HMR_ERR_NO_DEVICE;
    }
    if (dev < 0 || dev >= kMaxDevices) return HMR_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_mu);
    Slot& s = g_slot[dev];
    unsigned long long id = current_context_id();
    // id 0: no context is current yet (the symbol lookup below creates the primary one) or
    // the driver cannot name it; either way the address is resolved now, not reused.
    if (s.addr == nullptr || id == 0 || id != s.ctx_id) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            cudaGetLastError();
            return e != cudaSuccess ? (int)e : HMR_ERR_STATE;
        }
        s.addr = p;
        s.ctx_id = current_context_id();
    }
    *out = s.addr;
    return HMR_OK;
}

bool ptrs(Comp& C, const double* const* p, int n) {
    for (int e = 0; e < MAX_COMP; e++) C.p[e] = nullptr;
    if (!p || n < 1 || n > MAX_COMP) return false;
    for (int e = 0; e < n; e++) {
        if (!p[e]) return false;
        C.p[e] = const_cast<double*>(p[e]);
    }
    return true;
}

}  // namespace

extern "C" int hmr_rk_substep_patch_noalloc(const hmr_config* cfg, const hmr_patch_geometry* pg, int stage,
                                            const double* alpha, double beta,
                                            const double* const* const* Q_int, double dt, double* const* Q_out,
                                            void* stream) {
    // Configuration, checked as hmr_ctx_create checks it.
    if (!cfg || !pg || !alpha || !Q_int || !Q_out || stage < 0 || stage > 2) return HMR_ERR_ARGUMENT;
    const int dim = cfg->dim;
    if (dim != 2 && dim != 3) return HMR_ERR_ARGUMENT;
    if (!reconstructor_known(cfg->convective_flux_reconstructor)) return HMR_ERR_UNSUPPORTED;
    if (cfg->diffusive_flux_reconstructor != HMR_DIFFUSIVE_NONE) return HMR_ERR_UNSUPPORTED;
    if (cfg->precision != HMR_PRECISION_FAST && cfg->precision != HMR_PRECISION_EXACT) return HMR_ERR_ARGUMENT;
    {
        Params probe;  // scheme constants in range (and, for WCNS6-CU-M2, the grid spacing set)
        const int r = scheme_params(cfg, probe);
        if (r) return r;
    }
    int neq = 0, ncomp = 0;
    if (cfg->flow_model == HMR_SINGLE_SPECIES && cfg->num_species == 1) {
        neq = dim + 2;
        ncomp = neq;
    } else if (cfg->flow_model == HMR_FIVE_EQN_ALLAIRE && cfg->num_species == 2) {
        neq = dim + 4;
        ncomp = neq + 1;
    } else if (cfg->flow_model == HMR_FOUR_EQN_CONSERVATIVE && cfg->num_species == 2) {
        neq = dim + 3;
        ncomp = neq;
    } else {
        return HMR_ERR_UNSUPPORTED;
    }
    for (int s = 0; s < cfg->num_species; s++) {
        if (!(cfg->species_gamma[s] > 1.0)) return HMR_ERR_ARGUMENT;
        if (cfg->flow_model == HMR_FOUR_EQN_CONSERVATIVE && !(cfg->species_R[s] > 0.0)) return HMR_ERR_ARGUMENT;
    }

    // The allocating entry points' geometry bounds (at most 2^20 cells per axis, fewer than
    // 2^40 ghost-box cells), so that no size below can overflow.
    Geom g;
    long ghost_cells = 1;
    for (int d = 0; d < 3; d++) {
        if (d < dim && (pg->n[d] < 1 || pg->n[d] > (1 << 20) || !(pg->dx[d] > 0.0))) return HMR_ERR_ARGUMENT;
        g.n[d] = d < dim ? pg->n[d] : 1;
        g.G[d] = d < dim ? g.n[d] + 2 * GHOST : 1;
        g.dx[d] = d < dim ? pg->dx[d] : 1.0;
        ghost_cells *= g.G[d];
    }
    if (ghost_cells >= (1L << 40)) return HMR_ERR_ARGUMENT;

    // Scratch layout and the size check, before touching the device.
    const long nc = ncell_of(g);
    if ((size_t)nc > kScratchBytes / sizeof(double)) return HMR_ERR_CAPACITY;
    size_t need = (size_t)(neq + 4) * nc;            // V, rho, cs, theta, Omega
    size_t nfaces = 0;
    for (int a = 0; a < dim; a++) {
        need += (size_t)(neq + 1) * nface_of(g, a);  // midpoint fluxes + midpoint velocity
        nfaces += (size_t)nface_of(g, a);
    }
    need += nfaces;                                  // queue of faces for the exact pass
    if (kHeaderBytes + need * sizeof(double) > kScratchBytes) return HMR_ERR_CAPACITY;

    UpdateArgs U;
    std::memset(&U, 0, sizeof(U));
    for (int s = 0; s <= stage; s++)
        if (!ptrs(U.Qint[s], Q_int[s], ncomp)) return HMR_ERR_ARGUMENT;
    if (!ptrs(U.Qout, Q_out, ncomp)) return HMR_ERR_ARGUMENT;
    for (int s = 0; s <= stage; s++) U.alpha[s] = alpha[s];
    U.nst = stage + 1;
    U.beta = beta;
    U.dt = dt;

    void* base = nullptr;
    int r = scratch_address(&base);
    if (r) return r;

    Variant v;
    v.dim = dim;
    v.model = cfg->flow_model;
    v.nsp = cfg->num_species;
    v.scheme = cfg->convective_flux_reconstructor;
    Params P;
    species_params(cfg->species_gamma, cfg->species_R, cfg->num_species, P);
    scheme_params(cfg, P);

    unsigned char* bytes = static_cast<unsigned char*>(base);
    double* p = reinterpret_cast<double*>(bytes + kHeaderBytes);
    Scratch S;
    S.V = p; p += (size_t)neq * nc;
    S.rho = p; p += nc;
    S.cs = p; p += nc;
    S.theta = p; p += nc;
    S.Omega = p; p += nc;
    for (int a = 0; a < 3; a++) {
        if (a < dim) {
            const long nf = nface_of(g, a);
            S.Fm[a] = p; p += (size_t)neq * nf;
            S.um[a] = p; p += nf;
        } else {
            S.Fm[a] = nullptr;
            S.um[a] = nullptr;
        }
    }
    S.Td = S.Gd = nullptr;   // Euler equations only
    for (int a = 0; a < 3; a++) S.Fd[a] = nullptr;
    Redo R;
    R.list = reinterpret_cast<unsigned long long*>(p);
    R.count = reinterpret_cast<unsigned int*>(bytes);   // zeroed by the fast face launch before use
    R.cap = (unsigned long long)nfaces;

    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    r = hmr_cells::launch_cells(v, P, g, U.Qint[stage], S, st);
    if (r) return r;
    r = hmr_cells::launch_sensor(v, g, S, st);
    if (r) return r;
    if (cfg->precision == HMR_PRECISION_EXACT) {
        r = hmr_exact::launch_faces(v, P, g, S, nullptr, R, st);
        if (r) return r;
        return hmr_exact::launch_update(v, g, S, U, st);
    }
    r = hmr_fast::launch_faces(v, P, g, S, nullptr, R, st);
    if (r) return r;
    return hmr_fast::launch_update(v, g, S, U, st);
}
