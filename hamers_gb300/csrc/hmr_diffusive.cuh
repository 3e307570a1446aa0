// Navier-Stokes diffusive flux of a single-species patch on the device:
// DiffusiveFluxReconstructorMidpoint::computeDiffusiveFluxOnPatch
//   src/flow/diffusive_flux_reconstructors/midpoint/DiffusiveFluxReconstructorMidpoint.cpp:38-2312
// with the second-, fourth- and sixth-order stencils
//   …/midpoint/DiffusiveFluxReconstructorMidpointSecondOrder.cpp, …FourthOrder.cpp, …SixthOrder.cpp
// (the sixth order reads five ghost cells: a patch's arrays then carry Geom::gh = 5)
// and the single-species coefficients of
//   src/flow/flow_models/single-species/FlowModelDiffusiveFluxUtilitiesSingleSpecies.cpp
//   (derivative variables :654-1505, side diffusivities :2471-2799, pairing :2800-3700).
//
// Three phases per substep:
//   diff_grad_item  (cells)     temperature and the node velocity gradient d_d u_c
//   diff_mid_item   (midpoints) F_mid = sum of D_k * derivative over the coefficient table
//   diff_face       (faces)     dt-scaled face flux reconstructed from three (five) midpoints
// The expressions keep the reference's operation order: bitwise in the exact
// form (built without FMA contraction), contracted in the fast form.
// Included by hmr_kernels.cuh after Geom, Scratch and the index helpers.
#pragma once

namespace hmr {

// Midpoint stencils.  ORD 2: 1*(R - L)/dx, 1/2*(p - m)/dx, 1/2*(R + L), dt*1*F.
//                     ORD 4: (9/8 (R - L) - 1/24 (RR - LL))/dx, (2/3 (p - m) - 1/12 (pp - mm))/dx,
//                            9/16 (R + L) - 1/16 (RR + LL), dt*(13/12 F - 1/24 (F_-1 + F_+1)).
//                     ORD 6 (…MidpointSixthOrder.cpp:80-117, 521-558, 962-1000, 1400-1440):
//                            (75/64 (R - L) - 25/384 (RR - LL) + 3/640 (RRR - LLL))/dx,
//                            (3/4 (p - m) - 3/20 (pp - mm) + 1/60 (ppp - mmm))/dx,
//                            75/128 (R + L) - 25/256 (RR + LL) + 3/256 (RRR + LLL),
//                            dt*(a_r F + b_r (F_-1 + F_+1) + c_r (F_-2 + F_+2)) with
//                            a_r = a + b + c, b_r = b + c, c_r = c of the midpoint derivative.
// Arguments: v[0 .. 2H-1], the cells at offsets -H .. H-1 from the midpoint (midpoint stencils)
// or -H .. -1, 1 .. H from the node (node stencil); H = ORD/2.
template <int ORD>
__device__ __forceinline__ double dmid_derivative(const double* v, double dx_inv) {
    if constexpr (ORD == 2) return double(1)*(v[1] - v[0])*dx_inv;
    else if constexpr (ORD == 4) return (double(9)/double(8)*(v[2] - v[1]) + -double(1)/double(24)*(v[3] - v[0]))*dx_inv;
    else return (double(75)/double(64)*(v[3] - v[2]) + -double(25)/double(384)*(v[4] - v[1]) +
                 double(3)/double(640)*(v[5] - v[0]))*dx_inv;
}
template <int ORD>
__device__ __forceinline__ double dnode_derivative(const double* v, double dx_inv) {
    if constexpr (ORD == 2) return double(1)/double(2)*(v[1] - v[0])*dx_inv;
    else if constexpr (ORD == 4) return (double(2)/double(3)*(v[2] - v[1]) + -double(1)/double(12)*(v[3] - v[0]))*dx_inv;
    else return (double(3)/double(4)*(v[3] - v[2]) + -double(3)/double(20)*(v[4] - v[1]) +
                 double(1)/double(60)*(v[5] - v[0]))*dx_inv;
}
template <int ORD>
__device__ __forceinline__ double dmid_value(const double* v) {
    if constexpr (ORD == 2) return double(1)/double(2)*(v[1] + v[0]);
    else if constexpr (ORD == 4) return double(9)/double(16)*(v[2] + v[1]) + -double(1)/double(16)*(v[3] + v[0]);
    else return (double(75)/double(128)*(v[3] + v[2]) + -double(25)/double(256)*(v[4] + v[1]) +
                 double(3)/double(256)*(v[5] + v[0]));
}
// Four-cell forms (cells -2 .. 1 from the midpoint) of the second- and fourth-order stencils.
template <int ORD>
__device__ __forceinline__ double dmid_derivative(double LL, double L, double R, double RR, double dx_inv) {
    static_assert(ORD == 2 || ORD == 4, "four-cell stencils");
    const double v[4] = {LL, L, R, RR};
    return dmid_derivative<ORD>(v + (ORD == 2 ? 1 : 0), dx_inv);
}
template <int ORD>
__device__ __forceinline__ double dmid_value(double LL, double L, double R, double RR) {
    static_assert(ORD == 2 || ORD == 4, "four-cell stencils");
    const double v[4] = {LL, L, R, RR};
    return dmid_value<ORD>(v + (ORD == 2 ? 1 : 0));
}
// Half-width of the midpoint set (faces -W .. n + W) the face formula reads.
template <int ORD>
__host__ __device__ constexpr int diff_w() { return ORD == 6 ? 2 : 1; }

// Coefficient table: terms (equation e, variable v, diffusivity k) of the flux
// normal to A differentiated along D, in the reference's per-equation order;
// v = 0..DIM-1 velocity components, 3 temperature.  D_k at a side normal to A:
//   D0 = -(4/3 mu + mu_v), D1 = 2/3 mu - mu_v, D2 = -mu, D3 = -u_A (4/3 mu + mu_v),
//   D4 = u_A (2/3 mu - mu_v), then -u_t mu for the transverse velocities t in
//   increasing axis order, and last -kappa.
template <int DIM, int A, int D, class F>
__device__ __forceinline__ void for_diff_terms(F&& f) {
    if constexpr (DIM == 3) {
        if constexpr (A == 0 && D == 0) { f(1, 0, 0); f(2, 1, 2); f(3, 2, 2); f(4, 0, 3); f(4, 1, 5); f(4, 2, 6); f(4, 3, 7); }
        if constexpr (A == 0 && D == 1) { f(1, 1, 1); f(2, 0, 2); f(4, 0, 5); f(4, 1, 4); }
        if constexpr (A == 0 && D == 2) { f(1, 2, 1); f(3, 0, 2); f(4, 0, 6); f(4, 2, 4); }
        if constexpr (A == 1 && D == 0) { f(1, 1, 2); f(2, 0, 1); f(4, 0, 4); f(4, 1, 5); }
        if constexpr (A == 1 && D == 1) { f(1, 0, 2); f(2, 1, 0); f(3, 2, 2); f(4, 0, 5); f(4, 1, 3); f(4, 2, 6); f(4, 3, 7); }
        if constexpr (A == 1 && D == 2) { f(2, 2, 1); f(3, 1, 2); f(4, 1, 6); f(4, 2, 4); }
        if constexpr (A == 2 && D == 0) { f(1, 2, 2); f(3, 0, 1); f(4, 0, 4); f(4, 2, 5); }
        if constexpr (A == 2 && D == 1) { f(2, 2, 2); f(3, 1, 1); f(4, 1, 4); f(4, 2, 6); }
        if constexpr (A == 2 && D == 2) { f(1, 0, 2); f(2, 1, 2); f(3, 2, 0); f(4, 0, 5); f(4, 1, 6); f(4, 2, 3); f(4, 3, 7); }
    } else {
        if constexpr (A == 0 && D == 0) { f(1, 0, 0); f(2, 1, 2); f(3, 0, 3); f(3, 1, 5); f(3, 3, 6); }
        if constexpr (A == 0 && D == 1) { f(1, 1, 1); f(2, 0, 2); f(3, 0, 5); f(3, 1, 4); }
        if constexpr (A == 1 && D == 0) { f(1, 1, 2); f(2, 0, 1); f(3, 0, 4); f(3, 1, 5); }
        if constexpr (A == 1 && D == 1) { f(1, 0, 2); f(2, 1, 0); f(3, 0, 5); f(3, 1, 3); f(3, 3, 6); }
    }
}

// Cell phase: temperature T = p/((gamma - 1) c_v rho) (EquationOfStateIdealGas.cpp:2157-2173)
// and the node derivatives d_d u_c (…MidpointFourthOrder.cpp:457-845) of every cell whose
// stencil along d lies in the ghost box (0 elsewhere).  Gd[(d*DIM + c)*nc + x].
template <int DIM, int ORD>
__device__ __forceinline__ void diff_grad_item(const Params& P, const Geom& g, const Scratch& S, long x) {
    const long nc = ncell_of(g);
    const int ii[3] = {(int)(x % g.G[0]), (int)((x / g.G[0]) % g.G[1]), (int)(x / ((long)g.G[0] * g.G[1]))};
    const double* V = S.V;
    S.Td[x] = V[(DIM + 1) * nc + x]/(P.dTc*V[x]);
    constexpr int H = ORD / 2;                 // stencil half-width
    constexpr int HR = ORD == 6 ? 3 : 2;       // cells this close to the ghost box's edge keep 0
#pragma unroll
    for (int d = 0; d < DIM; d++) {
        const long st = d == 0 ? 1 : (d == 1 ? (long)g.G[0] : (long)g.G[0] * g.G[1]);
        const bool in = ii[d] >= HR && ii[d] < g.G[d] - HR;
        const double dx_inv = double(1)/g.dx[d];
#pragma unroll
        for (int c = 0; c < DIM; c++) {
            const double* u = V + (1 + c) * nc;
            double v[2 * H];
            if (in) {
#pragma unroll
                for (int m = 0; m < H; m++) {
                    v[m] = u[x - (H - m) * st];
                    v[H + m] = u[x + (m + 1) * st];
                }
            }
            S.Gd[(long)(d * DIM + c) * nc + x] = in ? dnode_derivative<ORD>(v, dx_inv) : 0.0;
        }
    }
}

// Midpoint phase: F_mid of all equations at midpoint-set item t of axis A (the side
// between cells xR - e_A and xR; index along A in [-W, n_A+W]), into S.Fd[A].
// …Midpoint.cpp:1400-1620 (x-flux; y and z analogues), F_mid = 0 += D*derivative.
template <int DIM, int ORD, int A>
__device__ __forceinline__ void diff_mid_item(const Params& P, const Geom& g, const Scratch& S, long t) {
    constexpr int NEQ = DIM + 2;
    constexpr int W = diff_w<ORD>();
    constexpr int H = ORD == 2 ? 2 : ORD / 2;   // cells -H .. H-1 (second order reads the inner two)
    const long nc = ncell_of(g);
    const long nf = nface_w(g, A, W);
    const int e0 = g.n[0] + (A == 0 ? 1 + 2 * W : 0);
    const int e1 = g.n[1] + (A == 1 ? 1 + 2 * W : 0);
    const int i = (int)(t % e0) - (A == 0 ? W : 0);
    const int j = (int)((t / e0) % e1) - (A == 1 ? W : 0);
    const int k = DIM == 3 ? (int)(t / ((long)e0 * e1)) - (A == 2 ? W : 0) : 0;
    const long xR = cidx<DIM>(g, i, j, k);
    const long st = A == 0 ? 1 : (A == 1 ? (long)g.G[0] : (long)g.G[0] * g.G[1]);
    // the stencil cells, offset so that the stencil functions see theirs first
    constexpr int O = ORD == 2 ? 1 : 0;
    long xs[2 * H];
#pragma unroll
    for (int m = 0; m < 2 * H; m++) xs[m] = xR + (m - H) * st;
    auto gather = [&](const double* f, double* v) {
#pragma unroll
        for (int m = 0; m < 2 * H; m++) v[m] = f[xs[m]];
    };
    const double* V = S.V;
    double v[2 * H];
    // side velocity and the derivatives the table reads
    double um[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int c = 0; c < DIM; c++) {
        gather(V + (1 + c) * nc, v);
        um[c] = dmid_value<ORD>(v + O);
    }
    double gr[3][4] = {{0.0, 0.0, 0.0, 0.0}, {0.0, 0.0, 0.0, 0.0}, {0.0, 0.0, 0.0, 0.0}};
    const double dxa_inv = double(1)/g.dx[A];
#pragma unroll
    for (int c = 0; c < DIM; c++) {
        gather(V + (1 + c) * nc, v);
        gr[A][c] = dmid_derivative<ORD>(v + O, dxa_inv);
    }
    gather(S.Td, v);
    gr[A][3] = dmid_derivative<ORD>(v + O, dxa_inv);
#pragma unroll
    for (int d = 0; d < DIM; d++) {
        if (d == A) continue;
#pragma unroll
        for (int c = 0; c < DIM; c++) {
            if (c != A && c != d) continue;
            gather(S.Gd + (long)(d * DIM + c) * nc, v);
            gr[d][c] = dmid_value<ORD>(v + O);
        }
    }
    // side diffusivities
    double Dk[8];
    Dk[0] = -P.dS43;
    Dk[1] = P.dS23;
    Dk[2] = -P.dmu;
    Dk[3] = -um[A]*P.dS43;
    Dk[4] = um[A]*P.dS23;
    if constexpr (DIM == 3) {
        constexpr int t1 = A == 0 ? 1 : 0, t2 = A == 2 ? 1 : 2;
        Dk[5] = -um[t1]*P.dmu;
        Dk[6] = -um[t2]*P.dmu;
        Dk[7] = -P.dkappa;
    } else {
        Dk[5] = -um[1 - A]*P.dmu;
        Dk[6] = -P.dkappa;
        Dk[7] = 0.0;
    }
    double F[NEQ];
#pragma unroll
    for (int e = 0; e < NEQ; e++) F[e] = 0.0;
    for_diff_terms<DIM, A, 0>([&](int e, int v, int kk) { F[e] += Dk[kk]*gr[0][v]; });
    for_diff_terms<DIM, A, 1>([&](int e, int v, int kk) { F[e] += Dk[kk]*gr[1][v]; });
    if constexpr (DIM == 3) for_diff_terms<DIM, A, 2>([&](int e, int v, int kk) { F[e] += Dk[kk]*gr[2][v]; });
    double* Fd = S.Fd[A];
#pragma unroll
    for (int e = 0; e < NEQ; e++) Fd[(long)e * nf + t] = F[e];
}

// dt-scaled face flux of equation e at midpoint-set index f of axis A (neighbours
// f -+ fst along A): …MidpointSixthOrder.cpp:1400-1440 / …FourthOrder.cpp:1231-1384 /
// …SecondOrder.cpp:1060-1130, accumulated onto a zeroed face array.
template <int ORD, int A>
__device__ __forceinline__ double diff_face(const Geom& g, const Scratch& S, double dt, long f, long fst, int e) {
    const long nf = nface_w(g, A, diff_w<ORD>());
    const double* Fm = S.Fd[A] + (long)e * nf;
    if constexpr (ORD == 2) {
        return 0.0 + dt*double(1)*Fm[f];
    } else if constexpr (ORD == 4) {
        const double a_r = double(9)/double(8) + -double(1)/double(24);
        const double b_r = -double(1)/double(24);
        return 0.0 + dt*(a_r*(Fm[f]) + b_r*(Fm[f - fst] + Fm[f + fst]));
    } else {
        const double a_m = double(75)/double(64), b_m = -double(25)/double(384), c_m = double(3)/double(640);
        const double a_r = a_m + b_m + c_m, b_r = b_m + c_m, c_r = c_m;
        return 0.0 + dt*(a_r*(Fm[f]) + b_r*(Fm[f - fst] + Fm[f + fst]) + c_r*(Fm[f - 2 * fst] + Fm[f + 2 * fst]));
    }
}

// Diffusive fluxes of the two faces of cell (i, j, k) normal to each axis (left dl, right dr).
template <int DIM, int ORD, int NEQ>
__device__ __forceinline__ void diff_cell_faces(const Geom& g, const Scratch& S, double dt, int i, int j, int k,
                                                double (&dl)[3][NEQ], double (&dr)[3][NEQ]) {
    constexpr int W = diff_w<ORD>();
    const long f0 = dfidx<0, W>(g, i, j, k), f1 = dfidx<1, W>(g, i, j, k);
    const long s1 = g.n[0];
#pragma unroll
    for (int e = 0; e < NEQ; e++) {
        dl[0][e] = diff_face<ORD, 0>(g, S, dt, f0, 1, e);
        dr[0][e] = diff_face<ORD, 0>(g, S, dt, f0 + 1, 1, e);
        dl[1][e] = diff_face<ORD, 1>(g, S, dt, f1, s1, e);
        dr[1][e] = diff_face<ORD, 1>(g, S, dt, f1 + s1, s1, e);
    }
    if constexpr (DIM == 3) {
        const long f2 = dfidx<2, W>(g, i, j, k);
        const long s2 = (long)g.n[0] * g.n[1];
#pragma unroll
        for (int e = 0; e < NEQ; e++) {
            dl[2][e] = diff_face<ORD, 2>(g, S, dt, f2, s2, e);
            dr[2][e] = diff_face<ORD, 2>(g, S, dt, f2 + s2, s2, e);
        }
    }
}

}  // namespace hmr
