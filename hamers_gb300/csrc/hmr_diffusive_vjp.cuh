// Reverse mode of the Navier-Stokes diffusive flux inside the substep adjoint
// (single species).  No counterpart in the reference.  Forward chain (see
// hmr_diffusive.cuh):
//   cells       T = p/((gamma - 1) c_v rho), node gradient Gd_{d,c} = stencil_d(u_c)
//   midpoints   F_mid = sum_terms D_k(u_mid) * g,  g a normal derivative of u_c or T,
//               or a transverse node gradient interpolated to the midpoint
//   faces       F_face = dt*(a_r F_mid + b_r (F_mid(-1) + F_mid(+1)))   (fourth order;
//               + c_r (F_mid(-2) + F_mid(+2)) at sixth order)
//   update      Q_out += beta*(-(F_face,R - F_face,L)/dx)
// The reverse pass gathers, so that every sum has a fixed order:
//   diff_mid_bwd_item  (midpoints)  adjoints of the side velocities, normal derivatives
//                                   and interpolated transverse gradients -> VA.Mb[A]
//   diff_gd_bwd_item   (cells)      adjoint of the node gradient          -> VA.Gdb
//   diff_cell_bwd_item (cells)      adjoints of rho, u, p                 -> VA.Dv
// and cell_bwd_item adds VA.Dv to the primitive-variable adjoints of the cell.
// The diffusive flux is smooth in the state: no branch to follow.
#pragma once

namespace hmr {

// Per-midpoint adjoints kept by diff_mid_bwd_item: DIM side velocities, DIM + 1 normal
// derivatives (velocity components, temperature), and two interpolated transverse
// gradients (of u_A and u_d) for every axis d != A.
template <int DIM>
__host__ __device__ constexpr int diff_nmb() { return DIM + (DIM + 1) + 2 * (DIM - 1); }

// Slot of the transverse gradient d_d u_c (c == A or c == d) at a midpoint of axis A.
template <int A>
__device__ __forceinline__ int diff_tslot(int dim, int d, int c) {
    const int rank = d < A ? d : d - 1;   // position of d among the axes other than A
    return dim + (dim + 1) + 2 * rank + (c == A ? 0 : 1);
}

// Midpoint-set index (index along A from -W to n_A + W, interior elsewhere; W = diff_w<ORD>)
// of the midpoint at coordinate f along A and the transverse coordinates of (i, j, k); -1 if
// outside.
template <int DIM, int A, int W>
__device__ __forceinline__ long diff_face_set_index(const Geom& g, int i, int j, int k, int f) {
    int c[3] = {i, j, k};
    c[A] = f;
    if (f < -W || f > g.n[A] + W) return -1;
#pragma unroll
    for (int b = 0; b < DIM; b++)
        if (b != A && (c[b] < 0 || c[b] >= g.n[b])) return -1;
    const long e0 = g.n[0] + (A == 0 ? 1 + 2 * W : 0);
    const long e1 = g.n[1] + (A == 1 ? 1 + 2 * W : 0);
    return (long)(c[0] + (A == 0 ? W : 0)) + (long)(c[1] + (A == 1 ? W : 0)) * e0 +
           (DIM == 3 ? (long)(c[2] + (A == 2 ? W : 0)) * e0 * e1 : 0);
}

// Stencil half-width of the midpoint stencils: cells xs[m] = x_f + (m - H) e_A, m = 0 .. 2H-1
// (the second order reads the inner two of four).
template <int ORD>
__host__ __device__ constexpr int diff_h() { return ORD == 6 ? 3 : 2; }

// Weights of the cells xs[m] of a midpoint: interpolation and normal derivative (without 1/dx).
template <int ORD>
__device__ __forceinline__ double dw_value(int m) {
    if constexpr (ORD == 2) return (m == 1 || m == 2) ? 0.5 : 0.0;
    else if constexpr (ORD == 4) return (m == 1 || m == 2) ? 9.0/16.0 : -1.0/16.0;
    else return (m == 2 || m == 3) ? 75.0/128.0 : ((m == 1 || m == 4) ? -25.0/256.0 : 3.0/256.0);
}
template <int ORD>
__device__ __forceinline__ double dw_deriv(int m) {
    if constexpr (ORD == 2) return m == 1 ? -1.0 : (m == 2 ? 1.0 : 0.0);
    else if constexpr (ORD == 4) return m == 0 ? 1.0/24.0 : (m == 1 ? -9.0/8.0 : (m == 2 ? 9.0/8.0 : -1.0/24.0));
    else return m == 0 ? -3.0/640.0 : m == 1 ? 25.0/384.0 : m == 2 ? -75.0/64.0 :
                m == 3 ? 75.0/64.0 : m == 4 ? -25.0/384.0 : 3.0/640.0;
}
// Weight of u(y + l e_d) in the node gradient at y (l = -H .. H, l != 0; without 1/dx).
template <int ORD>
__device__ __forceinline__ double dw_node(int l) {
    if constexpr (ORD == 2) return l == 1 ? 0.5 : (l == -1 ? -0.5 : 0.0);
    else if constexpr (ORD == 4) return l == 1 ? 2.0/3.0 : (l == -1 ? -2.0/3.0 : (l == 2 ? -1.0/12.0 : 1.0/12.0));
    else {
        const double w = (l == 1 || l == -1) ? 3.0/4.0 : ((l == 2 || l == -2) ? -3.0/20.0 : 1.0/60.0);
        return l > 0 ? w : -w;
    }
}

template <int DIM, int ORD, int A>
__device__ __forceinline__ void diff_mid_bwd_item(const Params& P, const Geom& g, const Scratch& S,
                                                  const VjpArgs& VA, long t) {
    constexpr int NEQ = DIM + 2;
    constexpr int NMB = diff_nmb<DIM>();
    constexpr int W = diff_w<ORD>();
    constexpr int H = diff_h<ORD>();
    const long nf = nface_w(g, A, W);
    const int e0 = g.n[0] + (A == 0 ? 1 + 2 * W : 0);
    const int e1 = g.n[1] + (A == 1 ? 1 + 2 * W : 0);
    const int i = (int)(t % e0) - (A == 0 ? W : 0);
    const int j = (int)((t / e0) % e1) - (A == 1 ? W : 0);
    const int k = DIM == 3 ? (int)(t / ((long)e0 * e1)) - (A == 2 ? W : 0) : 0;
    const long xR = cidx<DIM>(g, i, j, k);
    const long st = A == 0 ? 1 : (A == 1 ? (long)g.G[0] : (long)g.G[0] * g.G[1]);
    const int ia = A == 0 ? i : (A == 1 ? j : k);
    // adjoint of F_mid from the face fluxes that read it
    double Fmb[NEQ];
    bool any = false;
#pragma unroll
    for (int e = 0; e < NEQ; e++) {
        const double c0 = Fface_bar<DIM, SINGLE_SPECIES, 1, A>(g, VA, i, j, k, ia, e);
        if constexpr (ORD == 2) {
            Fmb[e] = VA.dt*c0;
        } else if constexpr (ORD == 4) {
            const double cm = Fface_bar<DIM, SINGLE_SPECIES, 1, A>(g, VA, i, j, k, ia - 1, e);
            const double cp = Fface_bar<DIM, SINGLE_SPECIES, 1, A>(g, VA, i, j, k, ia + 1, e);
            Fmb[e] = VA.dt*(13.0/12.0*c0 - 1.0/24.0*(cm + cp));
        } else {
            const double cm = Fface_bar<DIM, SINGLE_SPECIES, 1, A>(g, VA, i, j, k, ia - 1, e);
            const double cp = Fface_bar<DIM, SINGLE_SPECIES, 1, A>(g, VA, i, j, k, ia + 1, e);
            const double cmm = Fface_bar<DIM, SINGLE_SPECIES, 1, A>(g, VA, i, j, k, ia - 2, e);
            const double cpp = Fface_bar<DIM, SINGLE_SPECIES, 1, A>(g, VA, i, j, k, ia + 2, e);
            const double a_m = 75.0/64.0, b_m = -25.0/384.0, c_m = 3.0/640.0;
            Fmb[e] = VA.dt*((a_m + b_m + c_m)*c0 + (b_m + c_m)*(cm + cp) + c_m*(cmm + cpp));
        }
        any = any || Fmb[e] != 0.0;
    }
    double* Mb = VA.Mb[A];
    if (!any) {
#pragma unroll
        for (int q = 0; q < NMB; q++) Mb[(long)q * nf + t] = 0.0;
        return;
    }
    // forward values (as diff_mid_item)
    const long nc = ncell_of(g);
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
    double Dk[8];
    Dk[0] = -P.dS43;
    Dk[1] = P.dS23;
    Dk[2] = -P.dmu;
    Dk[3] = -um[A]*P.dS43;
    Dk[4] = um[A]*P.dS23;
    constexpr int t1 = DIM == 3 ? (A == 0 ? 1 : 0) : 1 - A;
    constexpr int t2 = A == 2 ? 1 : 2;
    Dk[5] = -um[t1]*P.dmu;
    Dk[6] = DIM == 3 ? -um[t2]*P.dmu : -P.dkappa;
    Dk[7] = -P.dkappa;
    // reverse of F_mid = sum D_k g
    double Dkb[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    double grb[3][4] = {{0.0, 0.0, 0.0, 0.0}, {0.0, 0.0, 0.0, 0.0}, {0.0, 0.0, 0.0, 0.0}};
    for_diff_terms<DIM, A, 0>([&](int e, int v, int kk) { Dkb[kk] += Fmb[e]*gr[0][v]; grb[0][v] += Fmb[e]*Dk[kk]; });
    for_diff_terms<DIM, A, 1>([&](int e, int v, int kk) { Dkb[kk] += Fmb[e]*gr[1][v]; grb[1][v] += Fmb[e]*Dk[kk]; });
    if constexpr (DIM == 3)
        for_diff_terms<DIM, A, 2>([&](int e, int v, int kk) { Dkb[kk] += Fmb[e]*gr[2][v]; grb[2][v] += Fmb[e]*Dk[kk]; });
    double umb[3] = {0.0, 0.0, 0.0};
    umb[A] += -P.dS43*Dkb[3] + P.dS23*Dkb[4];
    umb[t1] += -P.dmu*Dkb[5];
    if constexpr (DIM == 3) umb[t2] += -P.dmu*Dkb[6];
#pragma unroll
    for (int c = 0; c < DIM; c++) Mb[(long)c * nf + t] = umb[c];
#pragma unroll
    for (int c = 0; c < DIM; c++) Mb[(long)(DIM + c) * nf + t] = grb[A][c];
    Mb[(long)(2 * DIM) * nf + t] = grb[A][3];
#pragma unroll
    for (int d = 0; d < DIM; d++) {
        if (d == A) continue;
        Mb[(long)diff_tslot<A>(DIM, d, A) * nf + t] = grb[d][A];
        Mb[(long)diff_tslot<A>(DIM, d, d) * nf + t] = grb[d][d];
    }
}

// Cell coordinates (interior origin) of ghost-box cell x.
template <int DIM>
__device__ __forceinline__ void diff_cell_coords(const Geom& g, long x, int (&c)[3]) {
    c[0] = (int)(x % g.G[0]) - g.gh;
    c[1] = (int)((x / g.G[0]) % g.G[1]) - g.gh;
    c[2] = DIM == 3 ? (int)(x / ((long)g.G[0] * g.G[1])) - g.gh : 0;
}

// Adjoint of the node gradient Gd_{d,c} at cell x: the midpoints of every axis A != d
// whose interpolation read it.
template <int DIM, int ORD>
__device__ __forceinline__ void diff_gd_bwd_item(const Geom& g, const VjpArgs& VA, long x) {
    const long nc = ncell_of(g);
    int c[3];
    diff_cell_coords<DIM>(g, x, c);
    double Gb[DIM][DIM];
#pragma unroll
    for (int d = 0; d < DIM; d++)
#pragma unroll
        for (int q = 0; q < DIM; q++) Gb[d][q] = 0.0;
    constexpr int W = diff_w<ORD>();
    constexpr int H = diff_h<ORD>();
    auto axis = [&](auto AC) {
        constexpr int A = decltype(AC)::value;
        const long nf = nface_w(g, A, W);
        const double* Mb = VA.Mb[A];
#pragma unroll
        for (int m = 0; m < 2 * H; m++) {
            const long t = diff_face_set_index<DIM, A, W>(g, c[0], c[1], c[2], c[A] + H - m);
            if (t < 0) continue;
            const double w = dw_value<ORD>(m);
#pragma unroll
            for (int d = 0; d < DIM; d++) {
                if (d == A) continue;
                Gb[d][A] += w*Mb[(long)diff_tslot<A>(DIM, d, A) * nf + t];
                Gb[d][d] += w*Mb[(long)diff_tslot<A>(DIM, d, d) * nf + t];
            }
        }
    };
    axis(std::integral_constant<int, 0>{});
    axis(std::integral_constant<int, 1>{});
    if constexpr (DIM == 3) axis(std::integral_constant<int, 2>{});
#pragma unroll
    for (int d = 0; d < DIM; d++)
#pragma unroll
        for (int q = 0; q < DIM; q++) VA.Gdb[(long)(d * DIM + q) * nc + x] = Gb[d][q];
}

// Adjoints of rho, u and p of cell x from the diffusive flux: side velocities, normal
// derivatives and temperature (midpoints of every axis), node gradients (cells y with
// x = y + l e_d), and T = p/((gamma - 1) c_v rho).
template <int DIM, int ORD>
__device__ __forceinline__ void diff_cell_bwd_item(const Params& P, const Geom& g, const Scratch& S,
                                                   const VjpArgs& VA, long x) {
    const long nc = ncell_of(g);
    int c[3];
    diff_cell_coords<DIM>(g, x, c);
    double ub[3] = {0.0, 0.0, 0.0}, Tb = 0.0;
    constexpr int W = diff_w<ORD>();
    constexpr int H = diff_h<ORD>();
    auto axis = [&](auto AC) {
        constexpr int A = decltype(AC)::value;
        const long nf = nface_w(g, A, W);
        const double* Mb = VA.Mb[A];
        const double dxi = double(1)/g.dx[A];
#pragma unroll
        for (int m = 0; m < 2 * H; m++) {
            const long t = diff_face_set_index<DIM, A, W>(g, c[0], c[1], c[2], c[A] + H - m);
            if (t < 0) continue;
            const double wv = dw_value<ORD>(m), wd = dw_deriv<ORD>(m)*dxi;
#pragma unroll
            for (int q = 0; q < DIM; q++) ub[q] += wv*Mb[(long)q * nf + t] + wd*Mb[(long)(DIM + q) * nf + t];
            Tb += wd*Mb[(long)(2 * DIM) * nf + t];
        }
    };
    axis(std::integral_constant<int, 0>{});
    axis(std::integral_constant<int, 1>{});
    if constexpr (DIM == 3) axis(std::integral_constant<int, 2>{});
#pragma unroll
    for (int d = 0; d < DIM; d++) {
        const long st = d == 0 ? 1 : (d == 1 ? (long)g.G[0] : (long)g.G[0] * g.G[1]);
        const int cd = c[d] + g.gh;
        const double dxi = double(1)/g.dx[d];
#pragma unroll
        for (int l = -H; l <= H; l++) {
            if (l == 0 || cd - l < 0 || cd - l >= g.G[d]) continue;
            const long y = x - l * st;
            const double w = dw_node<ORD>(l)*dxi;
#pragma unroll
            for (int q = 0; q < DIM; q++) ub[q] += w*VA.Gdb[(long)(d * DIM + q) * nc + y];
        }
    }
    const double rho = S.V[x], p = S.V[(DIM + 1) * nc + x];
    const double den = P.dTc*rho;
    VA.Dv[x] = -Tb*(p/den)/rho;
#pragma unroll
    for (int q = 0; q < DIM; q++) VA.Dv[(long)(1 + q) * nc + x] = ub[q];
    VA.Dv[(long)(DIM + 1) * nc + x] = Tb/den;
}

}  // namespace hmr
