// Kernels of the vector-Jacobian product of one fused RK substep of one patch
// (the adjoint of hmr_rk_substep_patch; items in hmr_vjp_items.cuh), for one
// flow model.  Built once per model (-DHMR_MODEL=0/1/2, namespace
// hmr_vjp_m<model>).  The forward values it recomputes are evaluated with
// explicitly rounded operations (the X = true forms), so they are the
// reference's bits -- and every branch the forward's -- while the reverse
// arithmetic may be contracted into FMAs.
#include <cuda_runtime.h>

#include "hmr_launch.h"
#include "hmr_vjp_items.cuh"

#ifndef HMR_MODEL
#error "HMR_MODEL must be defined: 0 single species, 1 four-equation, 2 five-equation"
#endif

#define HMR_CAT2(a, b) a##b
#define HMR_CAT(a, b) HMR_CAT2(a, b)
#define HMR_NS HMR_CAT(hmr_vjp_m, HMR_MODEL)

namespace HMR_NS {

using namespace hmr;

template <int D, int M, int N, int S>
struct VT {
    static constexpr int DIM = D, MODEL = M, NSP = N, SCHEME = S;
};

template <class F>
static int dispatch(const Variant& v, F f) {
    constexpr int M_ = HMR_MODEL;
    constexpr int N_ = M_ == SINGLE_SPECIES ? 1 : 2;
    if (v.model != M_ || v.nsp != N_) return -2;
    if (v.dim == 2 && v.scheme == WCNS5_JS) return f(VT<2, M_, N_, WCNS5_JS>{});
    if (v.dim == 2 && v.scheme == WCNS6_LD) return f(VT<2, M_, N_, WCNS6_LD>{});
    if (v.dim == 2 && v.scheme == WCNS5_Z) return f(VT<2, M_, N_, WCNS5_Z>{});
    if (v.dim == 2 && v.scheme == WCNS6_CU_M2) return f(VT<2, M_, N_, WCNS6_CU_M2>{});
    if (v.dim == 3 && v.scheme == WCNS5_JS) return f(VT<3, M_, N_, WCNS5_JS>{});
    if (v.dim == 3 && v.scheme == WCNS6_LD) return f(VT<3, M_, N_, WCNS6_LD>{});
    if (v.dim == 3 && v.scheme == WCNS5_Z) return f(VT<3, M_, N_, WCNS5_Z>{});
    if (v.dim == 3 && v.scheme == WCNS6_CU_M2) return f(VT<3, M_, N_, WCNS6_CU_M2>{});
    return -2;
}

constexpr int VJP_THREADS = 128;

static inline int grid_for(long items, int threads) {
    long b = (items + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > (1L << 30)) b = 1L << 30;
    return (int)b;
}

// ---------------------------------------------------------------------------
// One launch per phase over the flat item space of a group of patches (device records W,
// patch by binary search over the prefix offsets).  The per-patch form runs the same kernels
// on a one-patch group, so that a patch's result is bitwise the same in both forms: the
// reverse arithmetic is FMA-contracted, and contraction is decided per kernel, so only the
// same kernels give the same bits.
// ---------------------------------------------------------------------------
template <int PH, int AX>
__device__ __forceinline__ int vjp_find(const VjpWork* W, int np, long t) {
    int lo = 0, hi = np - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (W[mid].off[PH * 3 + AX] <= t) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <int DIM, int MODEL, int NSP, int SCHEME, int ORD, int PH, int AX>
__global__ void __launch_bounds__(VJP_THREADS)
level_vjp_kernel(Params P, const VjpWork* W, int np, long total) {
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int p = vjp_find<PH, AX>(W, np, t);
        const VjpWork& w = W[p];
        const long u = t - w.off[PH * 3 + AX];
        if constexpr (PH == VJP_PH_PROJ) face_proj_item<DIM, MODEL, NSP, AX>(w.g, w.S, w.A, u);
        else if constexpr (PH == VJP_PH_FWD) face_fwd_weno_item<DIM, MODEL, NSP, SCHEME, AX>(P, w.g, w.S, w.A, u);
        else if constexpr (PH == VJP_PH_RIEM) face_bwd_riemann_item<DIM, MODEL, NSP, SCHEME, AX>(P, w.g, w.S, w.A, u);
        else if constexpr (PH == VJP_PH_BWDW) face_bwd_weno_item<DIM, MODEL, NSP, SCHEME, AX>(P, w.g, w.S, w.A, u);
        else if constexpr (PH == VJP_PH_CHAR) face_bwd_char_item<DIM, MODEL, NSP, AX>(w.g, w.S, w.A, u);
        else if constexpr (PH == VJP_PH_DMID) diff_mid_bwd_item<DIM, ORD, AX>(P, w.g, w.S, w.A, u);
        else if constexpr (PH == VJP_PH_DGD) diff_gd_bwd_item<DIM, ORD>(w.g, w.A, u);
        else if constexpr (PH == VJP_PH_DCELL) diff_cell_bwd_item<DIM, ORD>(P, w.g, w.S, w.A, u);
        else cell_bwd_item<DIM, MODEL, NSP>(P, w.g, w.S, w.A, u);
    }
}

template <class T, int ORD, int PH, int AX>
static void launch_phase(const Params& P, const VjpWork* W, int np, const long* totals, cudaStream_t st) {
    const long n = totals[PH * 3 + AX];
    if (n <= 0) return;
    level_vjp_kernel<T::DIM, T::MODEL, T::NSP, T::SCHEME, ORD, PH, AX>
        <<<grid_for(n, VJP_THREADS), VJP_THREADS, 0, st>>>(P, W, np, n);
}

template <class T, int ORD, int AX>
static void launch_axis(const Params& P, const VjpWork* W, int np, const long* totals, cudaStream_t st) {
    launch_phase<T, ORD, VJP_PH_PROJ, AX>(P, W, np, totals, st);
    launch_phase<T, ORD, VJP_PH_FWD, AX>(P, W, np, totals, st);
    launch_phase<T, ORD, VJP_PH_RIEM, AX>(P, W, np, totals, st);
    launch_phase<T, ORD, VJP_PH_BWDW, AX>(P, W, np, totals, st);
    launch_phase<T, ORD, VJP_PH_CHAR, AX>(P, W, np, totals, st);
}

// Navier-Stokes: the diffusive flux's share of the primitive-variable adjoints (into VA.Dv).
template <class T, int ORD>
static void launch_diff(const Params& P, const VjpWork* W, int np, const long* totals, cudaStream_t st) {
    launch_phase<T, ORD, VJP_PH_DMID, 0>(P, W, np, totals, st);
    launch_phase<T, ORD, VJP_PH_DMID, 1>(P, W, np, totals, st);
    if constexpr (T::DIM == 3) launch_phase<T, ORD, VJP_PH_DMID, 2>(P, W, np, totals, st);
    launch_phase<T, ORD, VJP_PH_DGD, 0>(P, W, np, totals, st);
    launch_phase<T, ORD, VJP_PH_DCELL, 0>(P, W, np, totals, st);
}

// The convective and cell phases do not depend on the diffusive order: one instantiation
// (ORD 0) serves the Euler and every Navier-Stokes order.
template <class T, int ORD>
static int launch_group(const Params& P, const VjpWork* W, int np, const long* totals, bool flux_terms,
                        cudaStream_t st) {
    if (flux_terms) {
        launch_axis<T, 0, 0>(P, W, np, totals, st);
        launch_axis<T, 0, 1>(P, W, np, totals, st);
        if constexpr (T::DIM == 3) launch_axis<T, 0, 2>(P, W, np, totals, st);
        if constexpr (ORD != 0) launch_diff<T, ORD>(P, W, np, totals, st);
    }
    launch_phase<T, 0, VJP_PH_CELLB, 0>(P, W, np, totals, st);
    return (int)cudaPeekAtLastError();
}

int launch_vjp_level(const Variant& v, const Params& P, const VjpWork* W, int np, const long* totals,
                     bool flux_terms, cudaStream_t st) {
    return dispatch(v, [&](auto t) {
        using T = decltype(t);
        if constexpr (T::MODEL == SINGLE_SPECIES) {
            if (P.dorder == 4) return launch_group<T, 4>(P, W, np, totals, flux_terms, st);
            if (P.dorder == 2) return launch_group<T, 2>(P, W, np, totals, flux_terms, st);
            if (P.dorder == 6) return launch_group<T, 6>(P, W, np, totals, flux_terms, st);
        }
        if (P.dorder != 0) return -2;
        return launch_group<T, 0>(P, W, np, totals, flux_terms, st);
    });
}

// The one-patch record, written on the device (a kernel argument, so nothing waits on the host).
__global__ void store_record_kernel(VjpWork w, VjpWork* dst) { *dst = w; }

int launch_vjp(const Variant& v, const Params& P, const Geom& g, const Scratch& S, const VjpArgs& A,
               VjpWork* d_rec, cudaStream_t st) {
    VjpWork w;
    w.g = g;
    w.S = S;
    w.A = A;
    long totals[VJP_NPH * 3];
    for (int k = 0; k < VJP_NPH * 3; k++) w.off[k] = 0;
    vjp_item_counts(v, g, totals);
    store_record_kernel<<<1, 1, 0, st>>>(w, d_rec);
    return launch_vjp_level(v, P, d_rec, 1, totals, A.beta != 0.0, st);
}

}  // namespace HMR_NS
