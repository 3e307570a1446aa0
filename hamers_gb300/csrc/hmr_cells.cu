// Cell-centred kernels, always in the reference's operation order
// (built with -DHMR_FAST=0 --fmad=false): derived cell data, shock-sensor
// inputs, single-patch ghost fill and the general Runge-Kutta stage
// combination of Euler::advanceSingleStepOnPatch (src/apps/Euler/Euler.cpp:1003-1680).
#include <cuda_runtime.h>

#include <cstring>

#include "hmr_launch.h"

namespace hmr_cells {

using namespace hmr;

template <int D, int M, int N>
struct VT {
    static constexpr int DIM = D, MODEL = M, NSP = N;
};

template <class F>
static int dispatch(const Variant& v, F f) {
    if (v.model == SINGLE_SPECIES && v.nsp == 1) {
        if (v.dim == 2) return f(VT<2, SINGLE_SPECIES, 1>{});
        if (v.dim == 3) return f(VT<3, SINGLE_SPECIES, 1>{});
    }
    if (v.model == FIVE_EQN_ALLAIRE && v.nsp == 2) {
        if (v.dim == 2) return f(VT<2, FIVE_EQN_ALLAIRE, 2>{});
        if (v.dim == 3) return f(VT<3, FIVE_EQN_ALLAIRE, 2>{});
    }
    if (v.model == FOUR_EQN_CONSERVATIVE && v.nsp == 2) {
        if (v.dim == 2) return f(VT<2, FOUR_EQN_CONSERVATIVE, 2>{});
        if (v.dim == 3) return f(VT<3, FOUR_EQN_CONSERVATIVE, 2>{});
    }
    return -2;
}

constexpr int THREADS = 256;

static inline int grid_for(long items) {
    long b = (items + THREADS - 1) / THREADS;
    if (b < 1) b = 1;
    if (b > (1L << 30)) b = 1L << 30;
    return (int)b;
}

template <int DIM, int MODEL, int NSP>
__global__ void __launch_bounds__(THREADS) cells_kernel(Params P, Geom g, Comp Q, Scratch S) {
    const long n = ncell_of(g);
    for (long x = (long)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (long)gridDim.x * blockDim.x)
        cells_item<DIM, MODEL, NSP>(P, g, Q, S, x);
}

template <int DIM, int MODEL, int NSP>
__global__ void __launch_bounds__(THREADS) sensor_kernel(Geom g, Scratch S) {
    const long n = (long)(g.n[0] + 4) * (g.n[1] + 4) * (DIM == 3 ? g.n[2] + 4 : 1);
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x)
        sensor_item<DIM, MODEL, NSP>(g, S, t);
}

struct Periodic {
    int p[3];
};

template <int DIM>
__global__ void __launch_bounds__(THREADS) fill_kernel(Geom g, Comp Q, int ncomp, Periodic per, int mom0,
                                                       const double* bv) {
    const long n = ncell_of(g);
    for (long x = (long)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (long)gridDim.x * blockDim.x)
        fill_item<DIM>(g, Q, ncomp, per.p, x, mom0, bv);
}

int launch_cells(const Variant& v, const Params& P, const Geom& g, const Comp& Q, const Scratch& S,
                 cudaStream_t st) {
    return dispatch(v, [&](auto t) {
        using T = decltype(t);
        cells_kernel<T::DIM, T::MODEL, T::NSP><<<grid_for(ncell_of(g)), THREADS, 0, st>>>(P, g, Q, S);
        return (int)cudaPeekAtLastError();
    });
}

int launch_sensor(const Variant& v, const Geom& g, const Scratch& S, cudaStream_t st) {
    return dispatch(v, [&](auto t) {
        using T = decltype(t);
        const long n = (long)(g.n[0] + 4) * (g.n[1] + 4) * (T::DIM == 3 ? g.n[2] + 4 : 1);
        sensor_kernel<T::DIM, T::MODEL, T::NSP><<<grid_for(n), THREADS, 0, st>>>(g, S);
        return (int)cudaPeekAtLastError();
    });
}

int launch_fill(int dim, const Geom& g, const Comp& Q, int ncomp, const int* periodic, int mom0, const double* bv,
                cudaStream_t st) {
    Periodic per;
    for (int a = 0; a < 3; a++) per.p[a] = periodic ? periodic[a] : 0;
    if (dim == 2) fill_kernel<2><<<grid_for(ncell_of(g)), THREADS, 0, st>>>(g, Q, ncomp, per, mom0, bv);
    else fill_kernel<3><<<grid_for(ncell_of(g)), THREADS, 0, st>>>(g, Q, ncomp, per, mom0, bv);
    return (int)cudaPeekAtLastError();
}

// Adjoint of the single-patch ghost fill: every ghost cell's adjoint is added
// to the interior cell it was copied from (a gather per interior cell over the
// ghost cells of its preimage, so no two threads write one cell), then the
// ghost adjoints are cleared.  Ghost cells beyond a Dirichlet side are copies of
// no cell (their adjoints are cleared only).
__device__ __forceinline__ int fill_src(int v, int n, int periodic) {
    if (v >= 0 && v < n) return v;
    if (periodic == 1) return ((v % n) + n) % n;
    if (periodic == 3 || periodic == 5) return v < 0 ? -v - 1 : 2 * n - 1 - v;
    return v < 0 ? 0 : n - 1;
}

template <int DIM>
__global__ void __launch_bounds__(THREADS) fill_vjp_gather_kernel(Geom g, Comp Qb, int ncomp, Periodic per,
                                                                  int mom0) {
    const long n = ninterior_of(g);
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
        const int c[3] = {(int)(t % g.n[0]), (int)((t / g.n[0]) % g.n[1]),
                          DIM == 3 ? (int)(t / ((long)g.n[0] * g.n[1])) : 0};
        // per axis: the coordinates (this one first) whose fill source is c[a]
        int pre[3][9], np[3];
        for (int a = 0; a < 3; a++) {
            pre[a][0] = c[a];
            np[a] = 1;
            if (a >= DIM || per.p[a] == 2 || per.p[a] == 4) continue;   // provided or Dirichlet: no copies
            for (int v = -g.gh; v < g.n[a] + g.gh; v++) {
                if (v >= 0 && v < g.n[a]) continue;
                if (fill_src(v, g.n[a], per.p[a]) == c[a] && np[a] < 9) pre[a][np[a]++] = v;
            }
        }
        const long y = cidx<DIM>(g, c[0], c[1], c[2]);
        for (int e = 0; e < ncomp; e++) {
            double acc = 0.0;
            for (int a2 = 0; a2 < np[2]; a2++)
                for (int a1 = 0; a1 < np[1]; a1++)
                    for (int a0 = 0; a0 < np[0]; a0++) {
                        if (a0 == 0 && a1 == 0 && a2 == 0) continue;
                        const double v = Qb.p[e][cidx<DIM>(g, pre[0][a0], pre[1][a1], pre[2][a2])];
                        // a reflecting wall negated the normal momentum of the copy
                        const bool flip = (per.p[0] == 3 && a0 > 0 && e == mom0) != (per.p[1] == 3 && a1 > 0 && e == mom0 + 1) !=
                                          (DIM == 3 && per.p[2] == 3 && a2 > 0 && e == mom0 + 2);
                        acc += flip ? -v : v;
                    }
            if (acc != 0.0) Qb.p[e][y] += acc;
        }
    }
}

template <int DIM>
__global__ void __launch_bounds__(THREADS) fill_vjp_clear_kernel(Geom g, Comp Qb, int ncomp, Periodic per) {
    const long n = ncell_of(g);
    for (long x = (long)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (long)gridDim.x * blockDim.x) {
        const int c[3] = {(int)(x % g.G[0]) - g.gh, (int)((x / g.G[0]) % g.G[1]) - g.gh,
                          DIM == 3 ? (int)(x / ((long)g.G[0] * g.G[1])) - g.gh : 0};
        bool inside = true, provided = false;
        for (int a = 0; a < DIM; a++) {
            if (c[a] < 0 || c[a] >= g.n[a]) {
                inside = false;
                provided = provided || per.p[a] == 2;
            }
        }
        // provided ghosts keep their adjoints (they belong to whatever supplied the values)
        if (inside || provided) continue;
        for (int e = 0; e < ncomp; e++) Qb.p[e][x] = 0.0;
    }
}

int launch_fill_vjp(int dim, const Geom& g, const Comp& Qb, int ncomp, const int* periodic, int mom0,
                    cudaStream_t st) {
    Periodic per;
    for (int a = 0; a < 3; a++) per.p[a] = periodic ? periodic[a] : 0;
    if (dim == 2) {
        fill_vjp_gather_kernel<2><<<grid_for(ninterior_of(g)), THREADS, 0, st>>>(g, Qb, ncomp, per, mom0);
        fill_vjp_clear_kernel<2><<<grid_for(ncell_of(g)), THREADS, 0, st>>>(g, Qb, ncomp, per);
    } else {
        fill_vjp_gather_kernel<3><<<grid_for(ninterior_of(g)), THREADS, 0, st>>>(g, Qb, ncomp, per, mom0);
        fill_vjp_clear_kernel<3><<<grid_for(ncell_of(g)), THREADS, 0, st>>>(g, Qb, ncomp, per);
    }
    return (int)cudaPeekAtLastError();
}

// ---------------------------------------------------------------------------
// Stable time step: spectral radius sum_d (|u_d| + c)/dx_d, max over interior cells
// (Euler.cpp:489-900: MAX_WAVE_SPEED_d = |u_d| + c, FlowModelSingleSpecies.cpp:3959;
// spectral radius max_lambda_d/dx_d, summed over the directions in axis order; the
// level's dt is the minimum over patches of 1/max times the CFL number,
// RungeKuttaLevelIntegrator.cpp:1846-1916).  The max of non-negative doubles is taken
// on their bit patterns, which order like the values; the result does not depend on
// the order of the reduction.
// ---------------------------------------------------------------------------
template <int DIM, int MODEL, int NSP>
__device__ __forceinline__ double spectral_cell(const Params& P, const Geom& g, const Comp& Q, long x) {
    using M = Model<DIM, MODEL, NSP>;
    double q[M::NCOMP], V[M::NEQ], rho, cs;
#pragma unroll
    for (int e = 0; e < M::NCOMP; e++) q[e] = Q.p[e][x];
    cell_derived<DIM, MODEL, NSP>(P, q, V, rho, cs);
    double s = add_(fabs(V[M::IU]), cs)/g.dx[0];
#pragma unroll
    for (int d = 1; d < DIM; d++) s = add_(s, add_(fabs(V[M::IU + d]), cs)/g.dx[d]);
    if constexpr (MODEL == SINGLE_SPECIES) {
        if (P.dorder != 0) {
            // NavierStokes.cpp:1074-1078: 2 max_d(D/dx_d^2), D = max(mu/rho, mu_v/rho, kappa/(rho c_p))
            // (FlowModelSingleSpecies.cpp:4569-4573); the patch value is the max of both radii
            const double r = V[0];
            double Dm = fmax(P.cmu/r, P.cmu_v/r);
            Dm = fmax(Dm, P.ckappa/mul_(r, P.cp[0]));
            double q = Dm/mul_(g.dx[0], g.dx[0]);
            if constexpr (DIM == 2) q = fmax(q, Dm/mul_(g.dx[1], g.dx[1]));
            else q = fmax(q, fmax(Dm/mul_(g.dx[1], g.dx[1]), Dm/mul_(g.dx[2], g.dx[2])));
            s = fmax(s, mul_(double(2), q));
        }
    }
    return s;
}

__device__ __forceinline__ void block_max_to(double v, unsigned long long* d_max) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    __shared__ double s_w[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) s_w[warp] = v;
    __syncthreads();
    if (warp == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        v = lane < nw ? s_w[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (lane == 0 && v > 0.0) atomicMax(d_max, (unsigned long long)__double_as_longlong(v));
    }
}

// Item: a cell of the ghost box (the reference's loops cover the ghost cells too).
template <int DIM, int MODEL, int NSP>
__global__ void __launch_bounds__(THREADS) spectral_patch_kernel(Params P, Geom g, Comp Q, unsigned long long* d_max) {
    const long n = ncell_of(g);
    double m = 0.0;
    for (long x = (long)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (long)gridDim.x * blockDim.x)
        m = fmax(m, spectral_cell<DIM, MODEL, NSP>(P, g, Q, x));
    block_max_to(m, d_max);
}

template <int DIM, int MODEL, int NSP>
__global__ void __launch_bounds__(THREADS) spectral_level_kernel(Params P, const PatchWork* W, int np, long total,
                                                                  unsigned long long* d_max) {
    double m = 0.0;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        int lo = 0, hi = np - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (W[mid].off_cells <= t) lo = mid;
            else hi = mid - 1;
        }
        m = fmax(m, spectral_cell<DIM, MODEL, NSP>(P, W[lo].g, W[lo].Q[0], t - W[lo].off_cells));
    }
    block_max_to(m, d_max);
}

// Euler: dt = (1/max)*cfl (Euler.cpp:729, 881; RungeKuttaLevelIntegrator.cpp:1914-1916);
// NavierStokes: dt = (1/(max + eps))*cfl (NavierStokes.cpp:893, 1085).
__global__ void stable_dt_kernel(const unsigned long long* d_max, double cfl, double* d_dt, int ns) {
    const double m = __longlong_as_double((long long)*d_max);
    *d_dt = mul_(ns ? double(1)/add_(m, HMR_EPS) : double(1)/m, cfl);
}

int launch_spectral_patch(const Variant& v, const Params& P, const Geom& g, const Comp& Q,
                          unsigned long long* d_max, cudaStream_t st) {
    return dispatch(v, [&](auto t) {
        using T = decltype(t);
        int blocks = grid_for(ncell_of(g));
        if (blocks > 4096) blocks = 4096;
        spectral_patch_kernel<T::DIM, T::MODEL, T::NSP><<<blocks, THREADS, 0, st>>>(P, g, Q, d_max);
        return (int)cudaPeekAtLastError();
    });
}

int launch_spectral_level(const Variant& v, const Params& P, const PatchWork* work, int npatch, long total,
                          unsigned long long* d_max, cudaStream_t st) {
    return dispatch(v, [&](auto t) {
        using T = decltype(t);
        int blocks = grid_for(total);
        if (blocks > 4096) blocks = 4096;
        spectral_level_kernel<T::DIM, T::MODEL, T::NSP><<<blocks, THREADS, 0, st>>>(P, work, npatch, total, d_max);
        return (int)cudaPeekAtLastError();
    });
}

template <int DIM, int MODEL, int NSP>
__global__ void __launch_bounds__(THREADS)
cells_level_kernel(Params P, const PatchWork* W, int np, long total, int slot) {
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        int lo = 0, hi = np - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (W[mid].off_cells <= t) lo = mid;
            else hi = mid - 1;
        }
        cells_item<DIM, MODEL, NSP>(P, W[lo].g, W[lo].Q[slot], W[lo].S, t - W[lo].off_cells);
    }
}

template <int DIM, int MODEL, int NSP>
__global__ void __launch_bounds__(THREADS) sensor_level_kernel(const PatchWork* W, int np, long total) {
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        int lo = 0, hi = np - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (W[mid].off_sensor <= t) lo = mid;
            else hi = mid - 1;
        }
        sensor_item<DIM, MODEL, NSP>(W[lo].g, W[lo].S, t - W[lo].off_sensor);
    }
}

int launch_cells_level(const Variant& v, const Params& P, const PatchWork* work, int npatch, long total, int slot,
                       cudaStream_t st) {
    if (slot < 0 || slot > 2) return -1;
    return dispatch(v, [&](auto t) {
        using T = decltype(t);
        cells_level_kernel<T::DIM, T::MODEL, T::NSP><<<grid_for(total), THREADS, 0, st>>>(P, work, npatch, total, slot);
        return (int)cudaPeekAtLastError();
    });
}

int launch_sensor_level(const Variant& v, const PatchWork* work, int npatch, long total, cudaStream_t st) {
    return dispatch(v, [&](auto t) {
        using T = decltype(t);
        sensor_level_kernel<T::DIM, T::MODEL, T::NSP><<<grid_for(total), THREADS, 0, st>>>(work, npatch, total);
        return (int)cudaPeekAtLastError();
    });
}

int launch_stable_dt(const unsigned long long* d_max, double cfl, double* d_dt, cudaStream_t st, bool ns) {
    stable_dt_kernel<<<1, 1, 0, st>>>(d_max, cfl, d_dt, ns ? 1 : 0);
    return (int)cudaPeekAtLastError();
}

// ---------------------------------------------------------------------------
// General stage combination (any number of coefficient sets), one thread per
// interior cell and equation set:  Q = 0; for n: Q += alpha_n Q_n;
// Q += beta_n (-(F_R-F_L)/dx - ... + S_n); F += gamma_n F_n; S += gamma_n S_n.
// ---------------------------------------------------------------------------
struct StageArgs {
    int ncoef;
    double alpha[4], beta[4], gamma[4];
    Comp Q[4];
    FluxComp F[4];
    Comp S[4];
    Comp Qout;
    FluxComp Facc;
    Comp Sacc;
    int ns;              // NavierStokes: the diffusive fluxes Fd enter the divergence (and Fdacc)
    FluxComp Fd[4];
    FluxComp Fdacc;
};

template <int DIM, int MODEL, int NSP>
__global__ void __launch_bounds__(THREADS) rk_stage_kernel(Geom g, StageArgs A) {
    using M = Model<DIM, MODEL, NSP>;
    constexpr int NEQ = M::NEQ;
    const long nint = ninterior_of(g);
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < nint; t += (long)gridDim.x * blockDim.x) {
        const int i = (int)(t % g.n[0]);
        const int j = (int)((t / g.n[0]) % g.n[1]);
        const int k = DIM == 3 ? (int)(t / ((long)g.n[0] * g.n[1])) : 0;
        const long x = cidx<DIM>(g, i, j, k);
        const long fx0 = side_idx<DIM, 0>(g, i, j, k), fx1 = side_idx<DIM, 0>(g, i + 1, j, k);
        const long fy0 = side_idx<DIM, 1>(g, i, j, k), fy1 = side_idx<DIM, 1>(g, i, j + 1, k);
        long fz0 = 0, fz1 = 0;
        if (DIM == 3) { fz0 = side_idx<DIM, 2>(g, i, j, k); fz1 = side_idx<DIM, 2>(g, i, j, k + 1); }
        double q[NEQ];
#pragma unroll
        for (int e = 0; e < NEQ; e++) q[e] = 0.0;
        for (int n = 0; n < A.ncoef; n++) {
            if (A.alpha[n] != 0.0) {
#pragma unroll
                for (int e = 0; e < NEQ; e++) q[e] = add_(q[e], mul_(A.alpha[n], A.Q[n].p[e][x]));
            }
            if (A.beta[n] != 0.0) {
#pragma unroll
                for (int e = 0; e < NEQ; e++) {
                    const double* Fx = A.F[n].p[e];
                    const double* Fy = A.F[n].p[NEQ + e];
                    double div;
                    if (A.ns) {
                        // NavierStokes.cpp:1743-1749 (2D), 2085-2092 (3D)
                        const double* Dx = A.Fd[n].p[e];
                        const double* Dy = A.Fd[n].p[NEQ + e];
                        div = -(Fx[fx1] - Fx[fx0] + Dx[fx1] - Dx[fx0])/g.dx[0] -
                              (Fy[fy1] - Fy[fy0] + Dy[fy1] - Dy[fy0])/g.dx[1];
                        if (DIM == 3) {
                            const double* Fz = A.F[n].p[2 * NEQ + e];
                            const double* Dz = A.Fd[n].p[2 * NEQ + e];
                            div = div - (Fz[fz1] - Fz[fz0] + Dz[fz1] - Dz[fz0])/g.dx[2];
                        }
                    } else {
                        div = sub_(-(Fx[fx1] - Fx[fx0])/g.dx[0], (Fy[fy1] - Fy[fy0])/g.dx[1]);
                        if (DIM == 3) {
                            const double* Fz = A.F[n].p[2 * NEQ + e];
                            div = sub_(div, (Fz[fz1] - Fz[fz0])/g.dx[2]);
                        }
                    }
                    q[e] = add_(q[e], mul_(A.beta[n], add_(div, A.S[n].p[e][t])));
                }
                if (MODEL == FIVE_EQN_ALLAIRE) {
                    double zl = 1.0;
#pragma unroll
                    for (int s = 0; s < NSP - 1; s++) zl = sub_(zl, q[M::IZ + s]);
                    A.Qout.p[M::NCOMP - 1][x] = zl;
                }
            }
            if (A.gamma[n] != 0.0 && A.Facc.p[0] != nullptr) {
                // Time-integrated flux and source for refluxing (Euler.cpp:1420-1470 / 1560-1640).
#pragma unroll
                for (int e = 0; e < NEQ; e++) {
                    double* Fx = A.Facc.p[e];
                    double* Fy = A.Facc.p[NEQ + e];
                    Fx[fx0] = add_(Fx[fx0], mul_(A.gamma[n], A.F[n].p[e][fx0]));
                    if (i == g.n[0] - 1) Fx[fx1] = add_(Fx[fx1], mul_(A.gamma[n], A.F[n].p[e][fx1]));
                    Fy[fy0] = add_(Fy[fy0], mul_(A.gamma[n], A.F[n].p[NEQ + e][fy0]));
                    if (j == g.n[1] - 1) Fy[fy1] = add_(Fy[fy1], mul_(A.gamma[n], A.F[n].p[NEQ + e][fy1]));
                    if (DIM == 3) {
                        double* Fz = A.Facc.p[2 * NEQ + e];
                        Fz[fz0] = add_(Fz[fz0], mul_(A.gamma[n], A.F[n].p[2 * NEQ + e][fz0]));
                        if (k == g.n[2] - 1) Fz[fz1] = add_(Fz[fz1], mul_(A.gamma[n], A.F[n].p[2 * NEQ + e][fz1]));
                    }
                    A.Sacc.p[e][t] = add_(A.Sacc.p[e][t], mul_(A.gamma[n], A.S[n].p[e][t]));
                }
                if (A.ns && A.Fdacc.p[0] != nullptr) {
                    // NavierStokes.cpp:2170-2260: the diffusive fluxes are accumulated alike
#pragma unroll
                    for (int e = 0; e < NEQ; e++) {
                        double* Fx = A.Fdacc.p[e];
                        double* Fy = A.Fdacc.p[NEQ + e];
                        Fx[fx0] = add_(Fx[fx0], mul_(A.gamma[n], A.Fd[n].p[e][fx0]));
                        if (i == g.n[0] - 1) Fx[fx1] = add_(Fx[fx1], mul_(A.gamma[n], A.Fd[n].p[e][fx1]));
                        Fy[fy0] = add_(Fy[fy0], mul_(A.gamma[n], A.Fd[n].p[NEQ + e][fy0]));
                        if (j == g.n[1] - 1) Fy[fy1] = add_(Fy[fy1], mul_(A.gamma[n], A.Fd[n].p[NEQ + e][fy1]));
                        if (DIM == 3) {
                            double* Fz = A.Fdacc.p[2 * NEQ + e];
                            Fz[fz0] = add_(Fz[fz0], mul_(A.gamma[n], A.Fd[n].p[2 * NEQ + e][fz0]));
                            if (k == g.n[2] - 1)
                                Fz[fz1] = add_(Fz[fz1], mul_(A.gamma[n], A.Fd[n].p[2 * NEQ + e][fz1]));
                        }
                    }
                }
            }
        }
#pragma unroll
        for (int e = 0; e < NEQ; e++) A.Qout.p[e][x] = q[e];
    }
}

// ---------------------------------------------------------------------------
// Refluxing.  synchronizeFluxes (Euler.cpp:1682-1943, NavierStokes.cpp:2425-2700):
// Q += -div (F [+ Fd]) + S on the interior with the time-integrated fluxes, then the
// five-equation last volume fraction 1 - sum.
// ---------------------------------------------------------------------------
struct SyncArgs {
    Comp Q;
    FluxComp F, Fd;
    Comp S;
    int ns;
};

template <int DIM, int MODEL, int NSP>
__global__ void __launch_bounds__(THREADS) sync_kernel(Geom g, SyncArgs A) {
    using M = Model<DIM, MODEL, NSP>;
    constexpr int NEQ = M::NEQ;
    const long nint = ninterior_of(g);
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < nint; t += (long)gridDim.x * blockDim.x) {
        const int i = (int)(t % g.n[0]);
        const int j = (int)((t / g.n[0]) % g.n[1]);
        const int k = DIM == 3 ? (int)(t / ((long)g.n[0] * g.n[1])) : 0;
        const long x = cidx<DIM>(g, i, j, k);
        const long fx0 = side_idx<DIM, 0>(g, i, j, k), fx1 = side_idx<DIM, 0>(g, i + 1, j, k);
        const long fy0 = side_idx<DIM, 1>(g, i, j, k), fy1 = side_idx<DIM, 1>(g, i, j + 1, k);
        long fz0 = 0, fz1 = 0;
        if (DIM == 3) { fz0 = side_idx<DIM, 2>(g, i, j, k); fz1 = side_idx<DIM, 2>(g, i, j, k + 1); }
        double q[NEQ];
#pragma unroll
        for (int e = 0; e < NEQ; e++) {
            const double* Fx = A.F.p[e];
            const double* Fy = A.F.p[NEQ + e];
            double d;
            if (A.ns) {
                const double* Dx = A.Fd.p[e];
                const double* Dy = A.Fd.p[NEQ + e];
                d = -(Fx[fx1] - Fx[fx0] + Dx[fx1] - Dx[fx0])/g.dx[0] -
                    (Fy[fy1] - Fy[fy0] + Dy[fy1] - Dy[fy0])/g.dx[1];
                if (DIM == 3) {
                    const double* Fz = A.F.p[2 * NEQ + e];
                    const double* Dz = A.Fd.p[2 * NEQ + e];
                    d = d - (Fz[fz1] - Fz[fz0] + Dz[fz1] - Dz[fz0])/g.dx[2];
                }
            } else {
                d = -(Fx[fx1] - Fx[fx0])/g.dx[0] - (Fy[fy1] - Fy[fy0])/g.dx[1];
                if (DIM == 3) {
                    const double* Fz = A.F.p[2 * NEQ + e];
                    d = d - (Fz[fz1] - Fz[fz0])/g.dx[2];
                }
            }
            q[e] = A.Q.p[e][x] + (d + A.S.p[e][t]);
            A.Q.p[e][x] = q[e];
        }
        if constexpr (MODEL == FIVE_EQN_ALLAIRE) {
            double zl = 1.0;
#pragma unroll
            for (int s = 0; s < NSP - 1; s++) zl = zl - q[M::IZ + s];
            A.Q.p[M::NCOMP - 1][x] = zl;
        }
    }
}

int launch_sync(const Variant& v, const Geom& g, const Comp& Q, const FluxComp& F, const FluxComp* Fd,
                const Comp& S, cudaStream_t st) {
    if (Fd && v.model != SINGLE_SPECIES) return -2;
    SyncArgs A;
    std::memset(&A, 0, sizeof(A));
    A.Q = Q;
    A.F = F;
    A.S = S;
    A.ns = Fd != nullptr;
    if (Fd) A.Fd = *Fd;
    return dispatch(v, [&](auto t) {
        using T = decltype(t);
        sync_kernel<T::DIM, T::MODEL, T::NSP><<<grid_for(ninterior_of(g)), THREADS, 0, st>>>(g, A);
        return (int)cudaPeekAtLastError();
    });
}

// Coarsening between a fine patch and a coarse patch of the next coarser level (SAMRAI's
// CONSERVATIVE_COARSEN, restated: mean of the fine cells / faces, summed in fine index order
// and multiplied once by 1/r^k).  Placement: first interior cell lo and size n of each patch in
// its level's index space; the fine box is aligned with the ratio.
template <int DIM>
__global__ void __launch_bounds__(THREADS) coarsen_cells_kernel(CoarsenArgs C, Comp Qf, Comp Qc, int ncomp) {
    const long e0 = C.hi[0] - C.lo[0], e1 = C.hi[1] - C.lo[1], e2 = C.hi[2] - C.lo[2];
    const long ncov = e0 * e1 * e2;
    const double w = double(1)/double(C.r[0] * C.r[1] * C.r[2]);
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < ncov * ncomp; t += (long)gridDim.x * blockDim.x) {
        const int e = (int)(t / ncov);
        const long u = t % ncov;
        const int i = C.lo[0] + (int)(u % e0), j = C.lo[1] + (int)((u / e0) % e1), k = C.lo[2] + (int)(u / (e0 * e1));
        const int fi = (i + C.clo[0]) * C.r[0] - C.flo[0];
        const int fj = (j + C.clo[1]) * C.r[1] - C.flo[1];
        const int fk = (k + C.clo[2]) * C.r[2] - C.flo[2];
        double sum = 0.0;
        for (int q2 = 0; q2 < C.r[2]; q2++)
            for (int q1 = 0; q1 < C.r[1]; q1++)
                for (int q0 = 0; q0 < C.r[0]; q0++) sum += Qf.p[e][cidx<DIM>(C.gf, fi + q0, fj + q1, fk + q2)];
        Qc.p[e][cidx<DIM>(C.gc, i, j, k)] = sum*w;
    }
}

// One outer side of the fine patch normal to axis A: each coarse face it covers takes the
// mean of its fine faces.  ff, cf: face index along A in the fine and coarse patch.
template <int DIM, int A>
__global__ void __launch_bounds__(THREADS) coarsen_fluxsum_kernel(CoarsenArgs C, FluxComp Ff, FluxComp Fc, int neq,
                                                                 int ff, int cf) {
    const long e0 = A == 0 ? 1 : C.hi[0] - C.lo[0];
    const long e1 = A == 1 ? 1 : C.hi[1] - C.lo[1];
    const long e2 = A == 2 ? 1 : C.hi[2] - C.lo[2];
    const long nfc = e0 * e1 * e2;
    const int r0 = A == 0 ? 1 : C.r[0], r1 = A == 1 ? 1 : C.r[1], r2 = A == 2 ? 1 : C.r[2];
    const double w = double(1)/double(r0 * r1 * r2);
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < nfc * neq; t += (long)gridDim.x * blockDim.x) {
        const int e = (int)(t / nfc);
        const long u = t % nfc;
        int c[3] = {C.lo[0] + (int)(u % e0), C.lo[1] + (int)((u / e0) % e1), C.lo[2] + (int)(u / (e0 * e1))};
        c[A] = cf;
        int f0[3];
#pragma unroll
        for (int d = 0; d < 3; d++) f0[d] = (c[d] + C.clo[d]) * C.r[d] - C.flo[d];
        f0[A] = ff;
        double sum = 0.0;
        for (int q2 = 0; q2 < r2; q2++)
            for (int q1 = 0; q1 < r1; q1++)
                for (int q0 = 0; q0 < r0; q0++)
                    sum += Ff.p[A * neq + e][side_idx<DIM, A>(C.gf, f0[0] + q0, f0[1] + q1, f0[2] + q2)];
        Fc.p[A * neq + e][side_idx<DIM, A>(C.gc, c[0], c[1], c[2])] = sum*w;
    }
}

int launch_coarsen_cells(int dim, const CoarsenArgs& C, const Comp& Qf, const Comp& Qc, int ncomp, cudaStream_t st) {
    const long ncov = (long)(C.hi[0] - C.lo[0]) * (C.hi[1] - C.lo[1]) * (C.hi[2] - C.lo[2]);
    if (ncov <= 0) return 0;
    if (dim == 2) coarsen_cells_kernel<2><<<grid_for(ncov * ncomp), THREADS, 0, st>>>(C, Qf, Qc, ncomp);
    else coarsen_cells_kernel<3><<<grid_for(ncov * ncomp), THREADS, 0, st>>>(C, Qf, Qc, ncomp);
    return (int)cudaPeekAtLastError();
}

template <int DIM, int A>
static void fluxsum_sides(const CoarsenArgs& C, const FluxComp& Ff, const FluxComp& Fc, int neq, cudaStream_t st) {
    long nfc = 1;
    for (int d = 0; d < 3; d++) if (d != A) nfc *= C.hi[d] - C.lo[d];
    if (nfc <= 0) return;
    for (int side = 0; side < 2; side++) {
        const int ff = side == 0 ? 0 : C.gf.n[A];
        const int cf = (C.flo[A] + ff) / C.r[A] - C.clo[A];
        if (cf < 0 || cf > C.gc.n[A]) continue;
        coarsen_fluxsum_kernel<DIM, A><<<grid_for(nfc * neq), THREADS, 0, st>>>(C, Ff, Fc, neq, ff, cf);
    }
}

int launch_coarsen_fluxsum(int dim, const CoarsenArgs& C, const FluxComp& Ff, const FluxComp& Fc, int neq,
                           cudaStream_t st) {
    if (dim == 2) {
        fluxsum_sides<2, 0>(C, Ff, Fc, neq, st);
        fluxsum_sides<2, 1>(C, Ff, Fc, neq, st);
    } else {
        fluxsum_sides<3, 0>(C, Ff, Fc, neq, st);
        fluxsum_sides<3, 1>(C, Ff, Fc, neq, st);
        fluxsum_sides<3, 2>(C, Ff, Fc, neq, st);
    }
    return (int)cudaPeekAtLastError();
}

// Coarse-fine ghost cells of a fine patch: linear time interpolation of the coarse state,
// (1 - theta) old + theta new, then conservative linear refinement with monotonised-central
// slopes per coarse cell (SAMRAI's LINEAR_TIME_INTERPOLATE and CONSERVATIVE_LINEAR_REFINE,
// registered at FlowModelSingleSpecies.cpp:578-597; restated).  Item: a fine ghost-box cell.
__device__ __forceinline__ double mc_slope(double dm, double dp) {
    if (!(dm*dp > 0.0)) return 0.0;
    const double d = double(1)/double(2)*(dm + dp);
    const double b = double(2)*fmin(fabs(dm), fabs(dp));
    return fabs(d) < b ? d : (d > 0.0 ? b : -b);
}

template <int DIM>
__global__ void __launch_bounds__(THREADS) refine_ghosts_kernel(CoarsenArgs C, Comp Qo, Comp Qn, double theta,
                                                               Comp Qf, int ncomp) {
    const long nfc = ncell_of(C.gf);
    for (long x = (long)blockIdx.x * blockDim.x + threadIdx.x; x < nfc; x += (long)gridDim.x * blockDim.x) {
        const int f[3] = {(int)(x % C.gf.G[0]) - C.gf.gh, (int)((x / C.gf.G[0]) % C.gf.G[1]) - C.gf.gh,
                          DIM == 3 ? (int)(x / ((long)C.gf.G[0] * C.gf.G[1])) - C.gf.gh : 0};
        bool inside = true, covered = true;
        int c[3] = {0, 0, 0}, lev[3] = {0, 0, 0};
#pragma unroll
        for (int d = 0; d < DIM; d++) {
            if (f[d] < 0 || f[d] >= C.gf.n[d]) inside = false;
            lev[d] = C.flo[d] + f[d];
            const int cl = lev[d] >= 0 ? lev[d] / C.r[d] : -((-lev[d] + C.r[d] - 1) / C.r[d]);
            c[d] = cl - C.clo[d];
            if (c[d] < 0 || c[d] >= C.gc.n[d]) covered = false;
        }
        if (inside || !covered) continue;
        const long xc = cidx<DIM>(C.gc, c[0], c[1], c[2]);
        for (int e = 0; e < ncomp; e++) {
            const double* o = Qo.p[e];
            const double* nw = Qn.p[e];
            auto q = [&](long y) { return (double(1) - theta)*o[y] + theta*nw[y]; };
            const double q0 = q(xc);
            double v = q0;
#pragma unroll
            for (int d = 0; d < DIM; d++) {
                const long st = d == 0 ? 1 : (d == 1 ? (long)C.gc.G[0] : (long)C.gc.G[0] * C.gc.G[1]);
                const double s = mc_slope(q0 - q(xc - st), q(xc + st) - q0);
                const double off = (double(lev[d]) + 0.5)/double(C.r[d]) - (double(c[d] + C.clo[d]) + 0.5);
                v += s*off;
            }
            Qf.p[e][x] = v;
        }
    }
}

int launch_refine_ghosts(int dim, const CoarsenArgs& C, const Comp& Qo, const Comp& Qn, double theta,
                         const Comp& Qf, int ncomp, cudaStream_t st) {
    if (dim == 2) refine_ghosts_kernel<2><<<grid_for(ncell_of(C.gf)), THREADS, 0, st>>>(C, Qo, Qn, theta, Qf, ncomp);
    else refine_ghosts_kernel<3><<<grid_for(ncell_of(C.gf)), THREADS, 0, st>>>(C, Qo, Qn, theta, Qf, ncomp);
    return (int)cudaPeekAtLastError();
}

template <int DIM, int ORD>
__global__ void __launch_bounds__(THREADS) diff_grad_kernel(Params P, Geom g, Scratch S) {
    const long nc = ncell_of(g);
    for (long x = (long)blockIdx.x * blockDim.x + threadIdx.x; x < nc; x += (long)gridDim.x * blockDim.x)
        diff_grad_item<DIM, ORD>(P, g, S, x);
}

// The same over the patches of a level (their PatchWork records; cells numbered as off_cells).
template <int DIM, int ORD>
__global__ void __launch_bounds__(THREADS) diff_grad_level_kernel(Params P, const PatchWork* W, int np, long total) {
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        int lo = 0, hi = np - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (W[mid].off_cells <= t) lo = mid;
            else hi = mid - 1;
        }
        diff_grad_item<DIM, ORD>(P, W[lo].g, W[lo].S, t - W[lo].off_cells);
    }
}

int launch_diff_grad_level(const Variant& v, const Params& P, const PatchWork* work, int npatch, long total,
                           cudaStream_t st) {
    if (v.model != SINGLE_SPECIES || (P.dorder != 2 && P.dorder != 4 && P.dorder != 6)) return -2;
    const int b = grid_for(total);
    if (v.dim == 2 && P.dorder == 2) diff_grad_level_kernel<2, 2><<<b, THREADS, 0, st>>>(P, work, npatch, total);
    else if (v.dim == 2 && P.dorder == 4) diff_grad_level_kernel<2, 4><<<b, THREADS, 0, st>>>(P, work, npatch, total);
    else if (v.dim == 2) diff_grad_level_kernel<2, 6><<<b, THREADS, 0, st>>>(P, work, npatch, total);
    else if (P.dorder == 2) diff_grad_level_kernel<3, 2><<<b, THREADS, 0, st>>>(P, work, npatch, total);
    else if (P.dorder == 4) diff_grad_level_kernel<3, 4><<<b, THREADS, 0, st>>>(P, work, npatch, total);
    else diff_grad_level_kernel<3, 6><<<b, THREADS, 0, st>>>(P, work, npatch, total);
    return (int)cudaPeekAtLastError();
}

int launch_diff_grad(const Variant& v, const Params& P, const Geom& g, const Scratch& S, cudaStream_t st) {
    if (v.model != SINGLE_SPECIES || (P.dorder != 2 && P.dorder != 4 && P.dorder != 6)) return -2;
    const int b = grid_for(ncell_of(g));
    if (v.dim == 2 && P.dorder == 2) diff_grad_kernel<2, 2><<<b, THREADS, 0, st>>>(P, g, S);
    else if (v.dim == 2 && P.dorder == 4) diff_grad_kernel<2, 4><<<b, THREADS, 0, st>>>(P, g, S);
    else if (v.dim == 2) diff_grad_kernel<2, 6><<<b, THREADS, 0, st>>>(P, g, S);
    else if (P.dorder == 2) diff_grad_kernel<3, 2><<<b, THREADS, 0, st>>>(P, g, S);
    else if (P.dorder == 4) diff_grad_kernel<3, 4><<<b, THREADS, 0, st>>>(P, g, S);
    else diff_grad_kernel<3, 6><<<b, THREADS, 0, st>>>(P, g, S);
    return (int)cudaPeekAtLastError();
}

int launch_rk_stage(const Variant& v, const Geom& g, int ncoef, const double* alpha, const double* beta,
                    const double* gamma, const Comp* Qint, const FluxComp* Fint, const Comp* Sint, const Comp& Qout,
                    const FluxComp& Facc, const Comp& Sacc, cudaStream_t st, const FluxComp* Fdint,
                    const FluxComp* Fdacc) {
    if (ncoef < 1 || ncoef > 4) return -1;
    if (Fdint && v.model != SINGLE_SPECIES) return -2;
    StageArgs A;
    std::memset(&A, 0, sizeof(A));
    A.ns = Fdint != nullptr;
    for (int n = 0; Fdint && n < ncoef; n++) A.Fd[n] = Fdint[n];
    if (Fdacc) A.Fdacc = *Fdacc;
    A.ncoef = ncoef;
    for (int n = 0; n < ncoef; n++) {
        A.alpha[n] = alpha[n];
        A.beta[n] = beta[n];
        A.gamma[n] = gamma ? gamma[n] : 0.0;
        A.Q[n] = Qint[n];
        A.F[n] = Fint[n];
        A.S[n] = Sint[n];
    }
    A.Qout = Qout;
    A.Facc = Facc;
    A.Sacc = Sacc;
    return dispatch(v, [&](auto t) {
        using T = decltype(t);
        rk_stage_kernel<T::DIM, T::MODEL, T::NSP><<<grid_for(ninterior_of(g)), THREADS, 0, st>>>(g, A);
        return (int)cudaPeekAtLastError();
    });
}

// ---------------------------------------------------------------------------
// Adjoint of a level's ghost fill with a layout (see launch_level_fill_vjp).
// ---------------------------------------------------------------------------
struct DomainArgs {
    int dom[3], per[3];
};

template <int DIM>
__global__ void __launch_bounds__(THREADS) level_domain_vjp_kernel(const LevelFillVjpPatch* W, int np, long total,
                                                                   int ncomp, DomainArgs D, int mom0) {
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        int lo = 0, hi = np - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (W[mid].off <= t) lo = mid;
            else hi = mid - 1;
        }
        const LevelFillVjpPatch& w = W[lo];
        const Geom& g = w.g;
        const long x = t - w.off;
        int c[3], s[3];
        c[0] = (int)(x % g.G[0]) - g.gh;
        c[1] = (int)((x / g.G[0]) % g.G[1]) - g.gh;
        c[2] = DIM == 3 ? (int)(x / ((long)g.G[0] * g.G[1])) - g.gh : 0;
        bool physical = false, dirichlet = false;
        int flip[3] = {-1, -1, -1};
#pragma unroll
        for (int a = 0; a < 3; a++) {
            s[a] = c[a];
            if (a >= DIM || D.per[a] == 1) continue;
            const int G = w.lo[a] + c[a];
            if (G >= 0 && G < D.dom[a]) continue;
            physical = true;
            if (D.per[a] == 4) {
                dirichlet = true;   // a constant: its adjoint reaches no cell
            } else if (D.per[a] == 3 || D.per[a] == 5) {
                s[a] = (G < 0 ? -G - 1 : 2 * D.dom[a] - 1 - G) - w.lo[a];
                if (D.per[a] == 3) flip[a] = mom0 + a;
            } else {
                s[a] = G < 0 ? -w.lo[a] : D.dom[a] - 1 - w.lo[a];
            }
        }
        if (!physical) continue;
        if (dirichlet) {
            for (int e = 0; e < ncomp; e++) w.Qb.p[e][x] = 0.0;
            continue;
        }
        const long y = cidx<DIM>(g, s[0], s[1], s[2]);
        for (int e = 0; e < ncomp; e++) {
            const double v = w.Qb.p[e][x];
            if (v != 0.0) atomicAdd(&w.Qb.p[e][y], (e == flip[0] || e == flip[1] || e == flip[2]) ? -v : v);
            w.Qb.p[e][x] = 0.0;
        }
    }
}

template <int DIM>
__global__ void __launch_bounds__(THREADS) level_exchange_vjp_kernel(const LevelFillVjpPatch* W,
                                                                     const GhostCopy* copies, int ncopy, long total,
                                                                     int ncomp) {
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        int lo = 0, hi = ncopy - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (copies[mid].off <= t) lo = mid;
            else hi = mid - 1;
        }
        const GhostCopy& cp = copies[lo];
        const long u = t - cp.off;
        const int a0 = (int)(u % cp.ext[0]);
        const int a1 = (int)((u / cp.ext[0]) % cp.ext[1]);
        const int a2 = (int)(u / ((long)cp.ext[0] * cp.ext[1]));
        const LevelFillVjpPatch& wd = W[cp.dst];
        const LevelFillVjpPatch& ws = W[cp.src];
        const long xd = cidx<DIM>(wd.g, cp.dlo[0] + a0, cp.dlo[1] + a1, cp.dlo[2] + a2);
        const long xs = cidx<DIM>(ws.g, cp.slo[0] + a0, cp.slo[1] + a1, cp.slo[2] + a2);
        for (int e = 0; e < ncomp; e++) {
            const double v = wd.Qb.p[e][xd];
            wd.Qb.p[e][xd] = 0.0;
            if (v != 0.0) atomicAdd(&ws.Qb.p[e][xs], v);
        }
    }
}

int launch_level_fill_vjp(int dim, const LevelFillVjpPatch* d_patches, int npatch, long total_cells,
                          const GhostCopy* d_copies, int ncopy, long total_copy, int ncomp, const int* dom,
                          const int* dom_periodic, int mom0, cudaStream_t st) {
    DomainArgs D;
    for (int a = 0; a < 3; a++) {
        D.dom[a] = dom[a];
        D.per[a] = dom_periodic[a];
    }
    if (dim == 2) level_domain_vjp_kernel<2><<<grid_for(total_cells), THREADS, 0, st>>>(d_patches, npatch, total_cells, ncomp, D, mom0);
    else level_domain_vjp_kernel<3><<<grid_for(total_cells), THREADS, 0, st>>>(d_patches, npatch, total_cells, ncomp, D, mom0);
    if (ncopy > 0 && total_copy > 0) {
        if (dim == 2)
            level_exchange_vjp_kernel<2><<<grid_for(total_copy), THREADS, 0, st>>>(d_patches, d_copies, ncopy, total_copy, ncomp);
        else
            level_exchange_vjp_kernel<3><<<grid_for(total_copy), THREADS, 0, st>>>(d_patches, d_copies, ncopy, total_copy, ncomp);
    }
    return (int)cudaPeekAtLastError();
}

}  // namespace hmr_cells
