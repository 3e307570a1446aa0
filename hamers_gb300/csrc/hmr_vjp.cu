// Kernels of the vector-Jacobian product of one fused RK substep of one patch
// (the adjoint of hmr_rk_substep_patch; items in hmr_vjp_items.cuh), for one
// flow model.  Built once per model (-DHMR_MODEL=0/1/2, namespace
// hmr_vjp_m<model>), with --fmad=false so that the forward values recomputed
// here are the reference's bits.
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
    if (v.dim == 3 && v.scheme == WCNS5_JS) return f(VT<3, M_, N_, WCNS5_JS>{});
    if (v.dim == 3 && v.scheme == WCNS6_LD) return f(VT<3, M_, N_, WCNS6_LD>{});
    return -2;
}

constexpr int VJP_THREADS = 128;

template <int DIM, int MODEL, int NSP, int SCHEME, int AX>
__global__ void __launch_bounds__(VJP_THREADS)
face_bwd_kernel(Params P, Geom g, Scratch S, VjpArgs VA) {
    const long nf = nface_of(g, AX);
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < nf; t += (long)gridDim.x * blockDim.x)
        face_bwd_item<DIM, MODEL, NSP, SCHEME, AX>(P, g, S, VA, t);
}

template <int DIM, int MODEL, int NSP>
__global__ void __launch_bounds__(VJP_THREADS)
cell_bwd_kernel(Params P, Geom g, Scratch S, VjpArgs VA) {
    const long nc = ncell_of(g);
    for (long x = (long)blockIdx.x * blockDim.x + threadIdx.x; x < nc; x += (long)gridDim.x * blockDim.x)
        cell_bwd_item<DIM, MODEL, NSP>(P, g, S, VA, x);
}

static inline int grid_for(long items, int threads) {
    long b = (items + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > (1L << 30)) b = 1L << 30;
    return (int)b;
}

int launch_vjp(const Variant& v, const Params& P, const Geom& g, const Scratch& S, const VjpArgs& A,
               cudaStream_t st) {
    return dispatch(v, [&](auto t) {
        using T = decltype(t);
        if (A.beta != 0.0) {
            face_bwd_kernel<T::DIM, T::MODEL, T::NSP, T::SCHEME, 0>
                <<<grid_for(nface_of(g, 0), VJP_THREADS), VJP_THREADS, 0, st>>>(P, g, S, A);
            face_bwd_kernel<T::DIM, T::MODEL, T::NSP, T::SCHEME, 1>
                <<<grid_for(nface_of(g, 1), VJP_THREADS), VJP_THREADS, 0, st>>>(P, g, S, A);
            if constexpr (T::DIM == 3)
                face_bwd_kernel<T::DIM, T::MODEL, T::NSP, T::SCHEME, 2>
                    <<<grid_for(nface_of(g, 2), VJP_THREADS), VJP_THREADS, 0, st>>>(P, g, S, A);
        }
        cell_bwd_kernel<T::DIM, T::MODEL, T::NSP>
            <<<grid_for(ncell_of(g), VJP_THREADS), VJP_THREADS, 0, st>>>(P, g, S, A);
        return (int)cudaPeekAtLastError();
    });
}

}  // namespace HMR_NS
