// Midpoint and face kernels of the Navier-Stokes diffusive flux (items in
// hmr_diffusive.cuh).  Built twice: -DHMR_FAST=0 --fmad=false (namespace
// hmr_diff_exact, the reference's rounding) and -DHMR_FAST=1 --fmad=true
// (namespace hmr_diff_fast, contracted into FMAs).
#include <cuda_runtime.h>

#include "hmr_launch.h"

#if HMR_FAST
#define HMR_NS hmr_diff_fast
#else
#define HMR_NS hmr_diff_exact
#endif

namespace HMR_NS {

using namespace hmr;

constexpr int DIFF_THREADS = 128;

static inline int grid_for(long items) {
    long b = (items + DIFF_THREADS - 1) / DIFF_THREADS;
    if (b < 1) b = 1;
    if (b > (1L << 30)) b = 1L << 30;
    return (int)b;
}

template <int DIM, int ORD, int A>
__global__ void __launch_bounds__(DIFF_THREADS) diff_mid_kernel(Params P, Geom g, Scratch S) {
    const long nf = nface_w(g, A, diff_w<ORD>());
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < nf; t += (long)gridDim.x * blockDim.x)
        diff_mid_item<DIM, ORD, A>(P, g, S, t);
}

// One face of the SAMRAI side layout (n_A + 1 faces along A, interior elsewhere).
template <int DIM, int ORD, int A>
__global__ void __launch_bounds__(DIFF_THREADS) diff_out_kernel(Geom g, Scratch S, double dt, FluxComp F) {
    constexpr int NEQ = DIM + 2;
    const int e0 = g.n[0] + (A == 0), e1 = g.n[1] + (A == 1), e2 = g.n[2] + (A == 2);
    const long nout = (long)e0 * e1 * (DIM == 3 ? e2 : 1);
    const long fst = A == 0 ? 1 : (A == 1 ? (long)g.n[0] : (long)g.n[0] * g.n[1]);
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < nout; t += (long)gridDim.x * blockDim.x) {
        const int i = (int)(t % e0), j = (int)((t / e0) % e1), k = DIM == 3 ? (int)(t / ((long)e0 * e1)) : 0;
        const long f = dfidx<A, diff_w<ORD>()>(g, i, j, k);
#pragma unroll
        for (int e = 0; e < NEQ; e++) F.p[A * NEQ + e][t] = diff_face<ORD, A>(g, S, dt, f, fst, e);
    }
}

template <int DIM, int ORD>
static void mid_axes(const Params& P, const Geom& g, const Scratch& S, cudaStream_t st) {
    constexpr int W = diff_w<ORD>();
    diff_mid_kernel<DIM, ORD, 0><<<grid_for(nface_w(g, 0, W)), DIFF_THREADS, 0, st>>>(P, g, S);
    diff_mid_kernel<DIM, ORD, 1><<<grid_for(nface_w(g, 1, W)), DIFF_THREADS, 0, st>>>(P, g, S);
    if constexpr (DIM == 3)
        diff_mid_kernel<DIM, ORD, 2><<<grid_for(nface_w(g, 2, W)), DIFF_THREADS, 0, st>>>(P, g, S);
}

template <int DIM, int ORD>
static void out_axes(const Geom& g, const Scratch& S, double dt, const FluxComp& F, cudaStream_t st) {
    long n[3];
    for (int a = 0; a < 3; a++) {
        n[a] = 1;
        for (int d = 0; d < DIM; d++) n[a] *= g.n[d] + (d == a);
    }
    diff_out_kernel<DIM, ORD, 0><<<grid_for(n[0]), DIFF_THREADS, 0, st>>>(g, S, dt, F);
    diff_out_kernel<DIM, ORD, 1><<<grid_for(n[1]), DIFF_THREADS, 0, st>>>(g, S, dt, F);
    if constexpr (DIM == 3) diff_out_kernel<DIM, ORD, 2><<<grid_for(n[2]), DIFF_THREADS, 0, st>>>(g, S, dt, F);
}

int launch_diff_mid(const Variant& v, const Params& P, const Geom& g, const Scratch& S, cudaStream_t st) {
    if (v.model != SINGLE_SPECIES || (P.dorder != 2 && P.dorder != 4 && P.dorder != 6)) return -2;
    if (P.dorder == 6 && g.gh < 5) return -2;
    if (v.dim == 2) {
        if (P.dorder == 2) mid_axes<2, 2>(P, g, S, st);
        else if (P.dorder == 4) mid_axes<2, 4>(P, g, S, st);
        else mid_axes<2, 6>(P, g, S, st);
    } else {
        if (P.dorder == 2) mid_axes<3, 2>(P, g, S, st);
        else if (P.dorder == 4) mid_axes<3, 4>(P, g, S, st);
        else mid_axes<3, 6>(P, g, S, st);
    }
    return (int)cudaPeekAtLastError();
}

int launch_diff_faces_out(const Variant& v, const Params& P, const Geom& g, const Scratch& S, double dt,
                          const FluxComp& F, cudaStream_t st) {
    if (v.model != SINGLE_SPECIES || (P.dorder != 2 && P.dorder != 4 && P.dorder != 6)) return -2;
    if (v.dim == 2) {
        if (P.dorder == 2) out_axes<2, 2>(g, S, dt, F, st);
        else if (P.dorder == 4) out_axes<2, 4>(g, S, dt, F, st);
        else out_axes<2, 6>(g, S, dt, F, st);
    } else {
        if (P.dorder == 2) out_axes<3, 2>(g, S, dt, F, st);
        else if (P.dorder == 4) out_axes<3, 4>(g, S, dt, F, st);
        else out_axes<3, 6>(g, S, dt, F, st);
    }
    return (int)cudaPeekAtLastError();
}

}  // namespace HMR_NS
