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

template <int DIM, int MODEL, int NSP, int AX>
__global__ void __launch_bounds__(VJP_THREADS)
face_proj_kernel(Geom g, Scratch S, VjpArgs VA) {
    const long nf = nface_of(g, AX);
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < nf; t += (long)gridDim.x * blockDim.x)
        face_proj_item<DIM, MODEL, NSP, AX>(g, S, VA, t);
}

template <int DIM, int MODEL, int NSP, int SCHEME, int AX>
__global__ void __launch_bounds__(VJP_THREADS)
face_fwd_weno_kernel(Params P, Geom g, Scratch S, VjpArgs VA) {
    const long n = nface_of(g, AX) * Model<DIM, MODEL, NSP>::NEQ;
    for (long u = (long)blockIdx.x * blockDim.x + threadIdx.x; u < n; u += (long)gridDim.x * blockDim.x)
        face_fwd_weno_item<DIM, MODEL, NSP, SCHEME, AX>(P, g, S, VA, u);
}

template <int DIM, int MODEL, int NSP, int SCHEME, int AX>
__global__ void __launch_bounds__(VJP_THREADS)
face_bwd_riemann_kernel(Params P, Geom g, Scratch S, VjpArgs VA) {
    const long nf = nface_of(g, AX);
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < nf; t += (long)gridDim.x * blockDim.x)
        face_bwd_riemann_item<DIM, MODEL, NSP, SCHEME, AX>(P, g, S, VA, t);
}

template <int DIM, int MODEL, int NSP, int SCHEME, int AX>
__global__ void __launch_bounds__(VJP_THREADS)
face_bwd_weno_kernel(Params P, Geom g, Scratch S, VjpArgs VA) {
    const long n = nface_of(g, AX) * Model<DIM, MODEL, NSP>::NEQ;
    for (long u = (long)blockIdx.x * blockDim.x + threadIdx.x; u < n; u += (long)gridDim.x * blockDim.x)
        face_bwd_weno_item<DIM, MODEL, NSP, SCHEME, AX>(P, g, S, VA, u);
}

template <int DIM, int MODEL, int NSP, int AX>
__global__ void __launch_bounds__(VJP_THREADS)
face_bwd_char_kernel(Geom g, Scratch S, VjpArgs VA) {
    const long nf = nface_of(g, AX);
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < nf; t += (long)gridDim.x * blockDim.x)
        face_bwd_char_item<DIM, MODEL, NSP, AX>(g, S, VA, t);
}

template <class T, int AX>
static void launch_face_axis(const Params& P, const Geom& g, const Scratch& S, const VjpArgs& A, cudaStream_t st) {
    const long nf = nface_of(g, AX);
    constexpr int NEQ = Model<T::DIM, T::MODEL, T::NSP>::NEQ;
    face_proj_kernel<T::DIM, T::MODEL, T::NSP, AX><<<grid_for(nf, VJP_THREADS), VJP_THREADS, 0, st>>>(g, S, A);
    face_fwd_weno_kernel<T::DIM, T::MODEL, T::NSP, T::SCHEME, AX>
        <<<grid_for(nf * NEQ, VJP_THREADS), VJP_THREADS, 0, st>>>(P, g, S, A);
    face_bwd_riemann_kernel<T::DIM, T::MODEL, T::NSP, T::SCHEME, AX>
        <<<grid_for(nf, VJP_THREADS), VJP_THREADS, 0, st>>>(P, g, S, A);
    face_bwd_weno_kernel<T::DIM, T::MODEL, T::NSP, T::SCHEME, AX>
        <<<grid_for(nf * NEQ, VJP_THREADS), VJP_THREADS, 0, st>>>(P, g, S, A);
    face_bwd_char_kernel<T::DIM, T::MODEL, T::NSP, AX><<<grid_for(nf, VJP_THREADS), VJP_THREADS, 0, st>>>(g, S, A);
}

template <int DIM, int MODEL, int NSP>
__global__ void __launch_bounds__(VJP_THREADS)
cell_bwd_kernel(Params P, Geom g, Scratch S, VjpArgs VA) {
    const long nc = ncell_of(g);
    for (long x = (long)blockIdx.x * blockDim.x + threadIdx.x; x < nc; x += (long)gridDim.x * blockDim.x)
        cell_bwd_item<DIM, MODEL, NSP>(P, g, S, VA, x);
}

template <int DIM, int ORD, int AX>
__global__ void __launch_bounds__(VJP_THREADS)
diff_mid_bwd_kernel(Params P, Geom g, Scratch S, VjpArgs VA) {
    const long nf = nface_of(g, AX);
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < nf; t += (long)gridDim.x * blockDim.x)
        diff_mid_bwd_item<DIM, ORD, AX>(P, g, S, VA, t);
}

template <int DIM, int ORD>
__global__ void __launch_bounds__(VJP_THREADS) diff_gd_bwd_kernel(Geom g, VjpArgs VA) {
    const long nc = ncell_of(g);
    for (long x = (long)blockIdx.x * blockDim.x + threadIdx.x; x < nc; x += (long)gridDim.x * blockDim.x)
        diff_gd_bwd_item<DIM, ORD>(g, VA, x);
}

template <int DIM, int ORD>
__global__ void __launch_bounds__(VJP_THREADS) diff_cell_bwd_kernel(Params P, Geom g, Scratch S, VjpArgs VA) {
    const long nc = ncell_of(g);
    for (long x = (long)blockIdx.x * blockDim.x + threadIdx.x; x < nc; x += (long)gridDim.x * blockDim.x)
        diff_cell_bwd_item<DIM, ORD>(P, g, S, VA, x);
}

// Navier-Stokes: the diffusive flux's share of the primitive-variable adjoints (into VA.Dv).
template <int DIM, int ORD>
static void launch_diff_bwd(const Params& P, const Geom& g, const Scratch& S, const VjpArgs& A, cudaStream_t st) {
    diff_mid_bwd_kernel<DIM, ORD, 0><<<grid_for(nface_of(g, 0), VJP_THREADS), VJP_THREADS, 0, st>>>(P, g, S, A);
    diff_mid_bwd_kernel<DIM, ORD, 1><<<grid_for(nface_of(g, 1), VJP_THREADS), VJP_THREADS, 0, st>>>(P, g, S, A);
    if constexpr (DIM == 3)
        diff_mid_bwd_kernel<DIM, ORD, 2><<<grid_for(nface_of(g, 2), VJP_THREADS), VJP_THREADS, 0, st>>>(P, g, S, A);
    diff_gd_bwd_kernel<DIM, ORD><<<grid_for(ncell_of(g), VJP_THREADS), VJP_THREADS, 0, st>>>(g, A);
    diff_cell_bwd_kernel<DIM, ORD><<<grid_for(ncell_of(g), VJP_THREADS), VJP_THREADS, 0, st>>>(P, g, S, A);
}

int launch_vjp(const Variant& v, const Params& P, const Geom& g, const Scratch& S, const VjpArgs& A,
               cudaStream_t st) {
    return dispatch(v, [&](auto t) {
        using T = decltype(t);
        if (A.beta != 0.0) {
            launch_face_axis<T, 0>(P, g, S, A, st);
            launch_face_axis<T, 1>(P, g, S, A, st);
            if constexpr (T::DIM == 3) launch_face_axis<T, 2>(P, g, S, A, st);
        }
        if constexpr (T::MODEL == SINGLE_SPECIES) {
            if (A.beta != 0.0 && A.Dv != nullptr) {
                if (P.dorder == 4) launch_diff_bwd<T::DIM, 4>(P, g, S, A, st);
                else if (P.dorder == 2) launch_diff_bwd<T::DIM, 2>(P, g, S, A, st);
                else return -2;
            }
        }
        cell_bwd_kernel<T::DIM, T::MODEL, T::NSP>
            <<<grid_for(ncell_of(g), VJP_THREADS), VJP_THREADS, 0, st>>>(P, g, S, A);
        return (int)cudaPeekAtLastError();
    });
}

}  // namespace HMR_NS
