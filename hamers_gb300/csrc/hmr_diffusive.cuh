// Navier-Stokes diffusive flux of a single-species patch on the device:
// DiffusiveFluxReconstructorMidpoint::computeDiffusiveFluxOnPatch
//   src/flow/diffusive_flux_reconstructors/midpoint/DiffusiveFluxReconstructorMidpoint.cpp:38-2312
// with the second- and fourth-order stencils
//   …/midpoint/DiffusiveFluxReconstructorMidpointSecondOrder.cpp, …FourthOrder.cpp
// and the single-species coefficients of
//   src/flow/flow_models/single-species/FlowModelDiffusiveFluxUtilitiesSingleSpecies.cpp
//   (derivative variables :654-1505, side diffusivities :2471-2799, pairing :2800-3700).
//
// Three phases per substep:
//   diff_grad_item  (cells)     temperature and the node velocity gradient d_d u_c
//   diff_mid_item   (midpoints) F_mid = sum of D_k * derivative over the coefficient table
//   diff_face       (faces)     dt-scaled face flux reconstructed from three midpoints
// The expressions keep the reference's operation order: bitwise in the exact
// form (built without FMA contraction), contracted in the fast form.
// Included by hmr_kernels.cuh after Geom, Scratch and the index helpers.
#pragma once

namespace hmr {

// Midpoint stencils.  ORD 2: 1*(R - L)/dx, 1/2*(p - m)/dx, 1/2*(R + L), dt*1*F.
//                     ORD 4: (9/8 (R - L) - 1/24 (RR - LL))/dx, (2/3 (p - m) - 1/12 (pp - mm))/dx,
//                            9/16 (R + L) - 1/16 (RR + LL), dt*(13/12 F - 1/24 (F_-1 + F_+1)).
template <int ORD>
__device__ __forceinline__ double dmid_derivative(double LL, double L, double R, double RR, double dx_inv) {
    if constexpr (ORD == 2) return double(1)*(R - L)*dx_inv;
    else return (double(9)/double(8)*(R - L) + -double(1)/double(24)*(RR - LL))*dx_inv;
}
template <int ORD>
__device__ __forceinline__ double dnode_derivative(double mm, double m, double p, double pp, double dx_inv) {
    if constexpr (ORD == 2) return double(1)/double(2)*(p - m)*dx_inv;
    else return (double(2)/double(3)*(p - m) + -double(1)/double(12)*(pp - mm))*dx_inv;
}
template <int ORD>
__device__ __forceinline__ double dmid_value(double LL, double L, double R, double RR) {
    if constexpr (ORD == 2) return double(1)/double(2)*(R + L);
    else return double(9)/double(16)*(R + L) + -double(1)/double(16)*(RR + LL);
}

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
#pragma unroll
    for (int d = 0; d < DIM; d++) {
        const long st = d == 0 ? 1 : (d == 1 ? (long)g.G[0] : (long)g.G[0] * g.G[1]);
        const bool in = ii[d] >= 2 && ii[d] < g.G[d] - 2;
        const double dx_inv = double(1)/g.dx[d];
#pragma unroll
        for (int c = 0; c < DIM; c++) {
            const double* u = V + (1 + c) * nc;
            S.Gd[(long)(d * DIM + c) * nc + x] =
                in ? dnode_derivative<ORD>(u[x - 2 * st], u[x - st], u[x + st], u[x + 2 * st], dx_inv) : 0.0;
        }
    }
}

// Midpoint phase: F_mid of all equations at face-set item t of axis A (the side
// between cells xR - e_A and xR; index along A in [-1, n_A+1]), into S.Fd[A].
// …Midpoint.cpp:1400-1620 (x-flux; y and z analogues), F_mid = 0 += D*derivative.
template <int DIM, int ORD, int A>
__device__ __forceinline__ void diff_mid_item(const Params& P, const Geom& g, const Scratch& S, long t) {
    constexpr int NEQ = DIM + 2;
    const long nc = ncell_of(g);
    const long nf = nface_of(g, A);
    const int e0 = g.n[0] + (A == 0 ? 3 : 0);
    const int e1 = g.n[1] + (A == 1 ? 3 : 0);
    const int i = (int)(t % e0) - (A == 0 ? 1 : 0);
    const int j = (int)((t / e0) % e1) - (A == 1 ? 1 : 0);
    const int k = DIM == 3 ? (int)(t / ((long)e0 * e1)) - (A == 2 ? 1 : 0) : 0;
    const long xR = cidx<DIM>(g, i, j, k);
    const long st = A == 0 ? 1 : (A == 1 ? (long)g.G[0] : (long)g.G[0] * g.G[1]);
    const long xs[4] = {xR - 2 * st, xR - st, xR, xR + st};
    const double* V = S.V;
    // side velocity and the derivatives the table reads
    double um[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int c = 0; c < DIM; c++) {
        const double* u = V + (1 + c) * nc;
        um[c] = dmid_value<ORD>(u[xs[0]], u[xs[1]], u[xs[2]], u[xs[3]]);
    }
    double gr[3][4] = {{0.0, 0.0, 0.0, 0.0}, {0.0, 0.0, 0.0, 0.0}, {0.0, 0.0, 0.0, 0.0}};
    const double dxa_inv = double(1)/g.dx[A];
#pragma unroll
    for (int c = 0; c < DIM; c++) {
        const double* u = V + (1 + c) * nc;
        gr[A][c] = dmid_derivative<ORD>(u[xs[0]], u[xs[1]], u[xs[2]], u[xs[3]], dxa_inv);
    }
    gr[A][3] = dmid_derivative<ORD>(S.Td[xs[0]], S.Td[xs[1]], S.Td[xs[2]], S.Td[xs[3]], dxa_inv);
#pragma unroll
    for (int d = 0; d < DIM; d++) {
        if (d == A) continue;
#pragma unroll
        for (int c = 0; c < DIM; c++) {
            if (c != A && c != d) continue;
            const double* G = S.Gd + (long)(d * DIM + c) * nc;
            gr[d][c] = dmid_value<ORD>(G[xs[0]], G[xs[1]], G[xs[2]], G[xs[3]]);
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

// dt-scaled face flux of equation e at face-set index f of axis A (neighbours
// f -+ fst along A): …MidpointFourthOrder.cpp:1231-1384 / …SecondOrder.cpp:1060-1130,
// accumulated onto a zeroed face array.
template <int ORD, int A>
__device__ __forceinline__ double diff_face(const Geom& g, const Scratch& S, double dt, long f, long fst, int e) {
    const long nf = nface_of(g, A);
    const double* Fm = S.Fd[A] + (long)e * nf;
    if constexpr (ORD == 2) {
        return 0.0 + dt*double(1)*Fm[f];
    } else {
        const double a_r = double(9)/double(8) + -double(1)/double(24);
        const double b_r = -double(1)/double(24);
        return 0.0 + dt*(a_r*(Fm[f]) + b_r*(Fm[f - fst] + Fm[f + fst]));
    }
}

// Diffusive fluxes of the two faces of cell (i, j, k) normal to each axis (left dl, right dr).
template <int DIM, int ORD, int NEQ>
__device__ __forceinline__ void diff_cell_faces(const Geom& g, const Scratch& S, double dt, int i, int j, int k,
                                                double (&dl)[3][NEQ], double (&dr)[3][NEQ]) {
    const long f0 = fidx<0>(g, i, j, k), f1 = fidx<1>(g, i, j, k);
    const long s1 = g.n[0];
#pragma unroll
    for (int e = 0; e < NEQ; e++) {
        dl[0][e] = diff_face<ORD, 0>(g, S, dt, f0, 1, e);
        dr[0][e] = diff_face<ORD, 0>(g, S, dt, f0 + 1, 1, e);
        dl[1][e] = diff_face<ORD, 1>(g, S, dt, f1, s1, e);
        dr[1][e] = diff_face<ORD, 1>(g, S, dt, f1 + s1, s1, e);
    }
    if constexpr (DIM == 3) {
        const long f2 = fidx<2>(g, i, j, k);
        const long s2 = (long)g.n[0] * g.n[1];
#pragma unroll
        for (int e = 0; e < NEQ; e++) {
            dl[2][e] = diff_face<ORD, 2>(g, S, dt, f2, s2, e);
            dr[2][e] = diff_face<ORD, 2>(g, S, dt, f2 + s2, s2, e);
        }
    }
}

}  // namespace hmr
