// Work items of the substep adjoint (vector-Jacobian product of one fused RK
// substep of one patch), written as device functions like the forward items
// of hmr_kernels.cuh.
//
// The forward substep is
//   Q_out = sum_n alpha_n Q_n + beta (-div F(Q_s) + S(Q_s))      (interior)
// with the five-equation model's last volume fraction rewritten as 1 - sum.
// For the adjoint Qb_out of Q_out, after the forward cell data and sensor of
// Q_s are in the scratch:
//   face items (per axis, per midpoint face; see the face phase below):
//     adjoint of the midpoint flux and midpoint velocity from the flux formula
//     and source; forward recompute of the face (projection, WCNS, inverse
//     projection, bounds, Riemann solve) and its reverse, down to the
//     primitive variables of the six stencil cells and the projection means,
//     written per face and stencil offset (no atomics, deterministic);
//   cell_bwd_item (per ghost-box cell): gathers those contributions, adds the
//     node-flux and advective-source terms, reverses the cell data (primitive
//     variables, density, sound speed) to the conserved variables and
//     accumulates into Qb_in[s]; adds alpha_n Qb_out into Qb_in[n].
#pragma once

#include <type_traits>

#include "hmr_adjoint.cuh"

namespace hmr {

// Arguments of the substep adjoint.
struct VjpArgs {
    Comp Qs;          // forward input of the flux: Q_int[stage] (ghost box)
    Comp Qbo;         // adjoint of the substep output (ghost box; interior read)
    Comp Qbi[3];      // adjoints of Q_int[0..stage] (ghost box), accumulated
    double alpha[3];
    int nst;
    double beta;
    double dt;
    double* Cb[3];    // per axis: (6*NEQ + 2) x nface(a) face contributions
    double* Wb[3];    // per axis: 2*NEQ x nface(a) adjoints of the reconstructed characteristic values
    double* Wv[3];    // per axis: 2*NEQ x nface(a) reconstructed characteristic values (forward)
    double* Kb[3];    // per axis: 9*NEQ x nface(a) forward smoothness indicators (and WCNS6-LD sigma)
    double* Fp[3];    // per axis: FaceLayout<NSP>::NFP x nface(a) projection factors and partial adjoints
    unsigned char* okf[3];   // per axis: nface(a) bounds flags
    // Navier-Stokes (null for the Euler equations): per axis diff_nmb<DIM>() x nface(a) midpoint
    // adjoints, DIM*DIM x ncell node-gradient adjoints, NEQ x ncell primitive-variable adjoints
    double* Mb[3];
    double* Gdb;
    double* Dv;
};

// One patch of a group whose substep VJPs run together, one launch per phase over the flat
// item space of all the group's patches (the per-patch form is a group of one).
// off[PH * 3 + axis] is the patch's prefix offset in the item space of phase PH (phases over
// cells use axis 0).  Phases: projection factors, WCNS forward keeping the smoothness
// indicators, Riemann reverse, WCNS reverse, projection reverse (per face axis); for
// NavierStokes the midpoint (per axis), node-gradient and cell reverses of the diffusive flux;
// the cell gather.
enum { VJP_PH_PROJ = 0, VJP_PH_FWD, VJP_PH_RIEM, VJP_PH_BWDW, VJP_PH_CHAR, VJP_PH_DMID, VJP_PH_DGD,
       VJP_PH_DCELL, VJP_PH_CELLB, VJP_NPH };
struct VjpWork {
    Geom g;
    Scratch S;
    VjpArgs A;
    long off[VJP_NPH * 3];
};

// Adjoint of the pre-rewrite stage output (component e < NEQ) at a cell:
// Qb_out, with the five-equation last volume fraction's adjoint moved onto
// the others (Z_N = 1 - sum Z_k, only written when beta != 0).
template <int DIM, int MODEL, int NSP>
__device__ __forceinline__ double qbar_eff(const VjpArgs& A, long x, int e) {
    using M = Model<DIM, MODEL, NSP>;
    double v = A.Qbo.p[e][x];
    if constexpr (MODEL == FIVE_EQN_ALLAIRE) {
        if (A.beta != 0.0 && e >= M::IZ && e < M::IZ + M::NZ) v -= A.Qbo.p[M::NCOMP - 1][x];
    }
    return v;
}

// Cell index of the cell at coordinate c along axis AX, other coordinates
// those of (i, j, k).
template <int DIM, int AX>
__device__ __forceinline__ long cell_along(const Geom& g, int i, int j, int k, int c) {
    return cidx<DIM>(g, AX == 0 ? c : i, AX == 1 ? c : j, AX == 2 ? c : k);
}

// Adjoint G_e = beta * qbar_eff at cell coordinate c along AX (zero outside the interior).
template <int DIM, int MODEL, int NSP, int AX>
__device__ __forceinline__ double G_at(const Geom& g, const VjpArgs& A, int i, int j, int k, int c, int e) {
    if (c < 0 || c >= g.n[AX]) return 0.0;
    return A.beta*qbar_eff<DIM, MODEL, NSP>(A, cell_along<DIM, AX>(g, i, j, k, c), e);
}

// Adjoint of the dt-scaled face flux F_face(f) (f in [0, n_AX]): from
// Q_out(x) += beta*(-(F(x+1/2) - F(x-1/2))/dx).
template <int DIM, int MODEL, int NSP, int AX>
__device__ __forceinline__ double Fface_bar(const Geom& g, const VjpArgs& A, int i, int j, int k, int f, int e) {
    if (f < 0 || f > g.n[AX]) return 0.0;
    return (G_at<DIM, MODEL, NSP, AX>(g, A, i, j, k, f, e) - G_at<DIM, MODEL, NSP, AX>(g, A, i, j, k, f - 1, e))/
           g.dx[AX];
}

// Adjoint of the advective-source speed term of cell c along AX (five-equation
// model): dt * sum_k G_{Z_k} Q_{Z_k}.
template <int DIM, int MODEL, int NSP, int AX>
__device__ __forceinline__ double usrc_bar(const Geom& g, const VjpArgs& A, int i, int j, int k, int c) {
    using M = Model<DIM, MODEL, NSP>;
    if (c < 0 || c >= g.n[AX]) return 0.0;
    const long x = cell_along<DIM, AX>(g, i, j, k, c);
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < M::NZ; q++) s += A.beta*qbar_eff<DIM, MODEL, NSP>(A, x, M::IZ + q)*A.Qs.p[M::IZ + q][x];
    return A.dt*s;
}

// ---------------------------------------------------------------------------
// Face phase of the adjoint (axis AX), in three items so that no kernel holds
// the whole face in registers:
//   face_bwd_riemann_item (per face): adjoints of the midpoint flux and velocity,
//     forward recompute of the face up to the Riemann solve and its reverse, the
//     inverse projection's reverse -> adjoints of the reconstructed
//     characteristic values (Wb) and partial adjoints of the projection factors;
//     first-order-fallback faces write their final contributions directly;
//   face_bwd_weno_item (per face and characteristic variable): reverse of the
//     WCNS interpolation -> adjoints of the six stencil values (into Cb);
//   face_bwd_char_item (per face): reverse of the characteristic projection and
//     of the projection means -> final per-face contributions (Cb).
// Per-face buffers of axis AX, nf faces each (VjpArgs):
//   Cb : (6*NEQ + 2) x nf   contributions to V of the six stencil cells, then rho, c
//   Wb : 2*NEQ x nf         adjoints of the minus/plus reconstructed values
//   Fp : NFP x nf           face projection factors, then their partial adjoints
//   okf: nf                 bounds flag of the face (0: first-order fallback)
// ---------------------------------------------------------------------------
template <int NSP>
struct FaceLayout {
    static constexpr int F = 6 + 3 * NSP;          // rb, cb, m_hrc, p_hrc, ic2, irc, zb[], zr[], hz[]
    static constexpr int NFP = F + 3 + NSP;         // + adjoints of p_hrc, ic2, irc, hz[]
};

template <int DIM, int MODEL, int NSP>
__device__ __forceinline__ void store_proj(double* Fp, long nf, long t, const FaceProj<DIM, MODEL, NSP>& F) {
    Fp[0 * nf + t] = F.rb; Fp[1 * nf + t] = F.cb; Fp[2 * nf + t] = F.m_hrc; Fp[3 * nf + t] = F.p_hrc;
    Fp[4 * nf + t] = F.ic2; Fp[5 * nf + t] = F.irc;
    if constexpr (MODEL == SINGLE_SPECIES) return;
#pragma unroll
    for (int q = 0; q < NSP; q++) {
        Fp[(6 + q) * nf + t] = F.zb[q];
        Fp[(6 + NSP + q) * nf + t] = F.zr[q];
        Fp[(6 + 2 * NSP + q) * nf + t] = F.hz[q];
    }
}

template <int DIM, int MODEL, int NSP>
__device__ __forceinline__ void load_proj(const double* Fp, long nf, long t, FaceProj<DIM, MODEL, NSP>& F) {
    F.rb = Fp[0 * nf + t]; F.cb = Fp[1 * nf + t]; F.m_hrc = Fp[2 * nf + t]; F.p_hrc = Fp[3 * nf + t];
    F.ic2 = Fp[4 * nf + t]; F.irc = Fp[5 * nf + t];
    if constexpr (MODEL == SINGLE_SPECIES) return;
#pragma unroll
    for (int q = 0; q < NSP; q++) {
        F.zb[q] = Fp[(6 + q) * nf + t];
        F.zr[q] = Fp[(6 + NSP + q) * nf + t];
        F.hz[q] = Fp[(6 + 2 * NSP + q) * nf + t];
    }
}

// Face coordinates of item t of axis AX: (i, j, k), the cell on the + side and the stride.
template <int DIM, int AX>
__device__ __forceinline__ void face_coords(const Geom& g, long t, int& i, int& j, int& k, long& xR, long& st) {
    const int e0 = g.n[0] + (AX == 0 ? 3 : 0);
    const int e1 = g.n[1] + (AX == 1 ? 3 : 0);
    i = (int)(t % e0) - (AX == 0);
    j = (int)((t / e0) % e1) - (AX == 1);
    k = DIM == 3 ? (int)(t / ((long)e0 * e1)) - (AX == 2) : 0;
    xR = cidx<DIM>(g, i, j, k);
    st = (AX == 0) ? 1 : (AX == 1 ? (long)g.G[0] : (long)g.G[0] * g.G[1]);
}

// Projection means and factors of face t (as face_item computes them).
template <int DIM, int MODEL, int NSP, int AX>
__device__ __forceinline__ void face_proj_item(const Geom& g, const Scratch& S, const VjpArgs& VA, long t) {
    const long nf = nface_of(g, AX);
    const long nc = ncell_of(g);
    int i, j, k;
    long xR, st;
    face_coords<DIM, AX>(g, t, i, j, k, xR, st);
    const long xL = xR - st;
    FaceProj<DIM, MODEL, NSP> F;
    F.rb = double(1)/double(2)*(S.rho[xL] + S.rho[xR]);
    F.cb = double(1)/double(2)*(S.cs[xL] + S.cs[xR]);
    if constexpr (MODEL != SINGLE_SPECIES) {
#pragma unroll
        for (int q = 0; q < NSP; q++) F.zb[q] = double(1)/double(2)*(S.V[q * nc + xL] + S.V[q * nc + xR]);
    }
    face_proj_setup(F);
    store_proj<DIM, MODEL, NSP>(VA.Fp[AX], nf, t, F);
}

// Characteristic stencil U[0..5] of variable e at face t.
template <int DIM, int MODEL, int NSP, int AX>
__device__ __forceinline__ void char_stencil(const Geom& g, const Scratch& S, const FaceProj<DIM, MODEL, NSP>& F,
                                             long xR, long st, int e, double* U) {
    constexpr int NEQ = Model<DIM, MODEL, NSP>::NEQ;
    const long nc = ncell_of(g);
#pragma unroll
    for (int m = 0; m < 6; m++) {
        double Vm[NEQ];
        const long x = xR + (m - 3) * st;
#pragma unroll
        for (int q = 0; q < NEQ; q++) Vm[q] = S.V[q * nc + x];
        U[m] = char_one<DIM, MODEL, NSP, AX>(F, Vm, e);
    }
}

// Forward values kept per characteristic variable and face for the reverse pass:
// the smoothness indicators of both sides (and WCNS6-LD's sigma).
template <int SCHEME>
__host__ __device__ constexpr int weno_kept() {
    return SCHEME == WCNS5_JS || SCHEME == WCNS5_Z ? 6 : (SCHEME == WCNS6_LD ? 9 : 8);
}

// Item u = e*nf + t: forward WCNS interpolation of variable e at face t, keeping
// the reconstructed values and the smoothness indicators.  The indicators and
// every WCNS decision are the reference's bits in both forms; the weighting is the
// exact form on HLLC-HLL faces (whose blending weight amplifies rounding) and the
// regrouped form elsewhere.
template <int DIM, int MODEL, int NSP, int SCHEME, int AX>
__device__ __forceinline__ void face_fwd_weno_item(const Params& P, const Geom& g, const Scratch& S,
                                                   const VjpArgs& VA, long u) {
    const long nf = nface_of(g, AX);
    const long t = u % nf;
    const int e = (int)(u / nf);
    int i, j, k;
    long xR, st;
    face_coords<DIM, AX>(g, t, i, j, k, xR, st);
    FaceProj<DIM, MODEL, NSP> F;
    load_proj<DIM, MODEL, NSP>(VA.Fp[AX], nf, t, F);
    double U[6], b[9], Wm, Wp;
    char_stencil<DIM, MODEL, NSP, AX>(g, S, F, xR, st, e, U);
    constexpr int NB = weno_kept<SCHEME>();
    const long xL = xR - st;
    const double theta_avg = 0.5*(S.theta[xL] + S.theta[xR]);
    const double Omega_avg = 0.5*(S.Omega[xL] + S.Omega[xR]);
    if (-theta_avg/(fabs(theta_avg) + Omega_avg + HMR_EPS) > 0.65) {
        if constexpr (SCHEME == WCNS5_JS) js_pair_keep<true>(U, P.p, Wm, Wp, b);
        else if constexpr (SCHEME == WCNS6_LD) ld_pair_keep<true>(U, P, Wm, Wp, b);
        else if constexpr (SCHEME == WCNS5_Z) z_pair_keep<true>(U, P.p, Wm, Wp, b);
        else cu_pair_keep<true, AX>(U, P, Wm, Wp, b);
    } else {
        if constexpr (SCHEME == WCNS5_JS) js_pair_keep<false>(U, P.p, Wm, Wp, b);
        else if constexpr (SCHEME == WCNS6_LD) ld_pair_keep<false>(U, P, Wm, Wp, b);
        else if constexpr (SCHEME == WCNS5_Z) z_pair_keep<false>(U, P.p, Wm, Wp, b);
        else cu_pair_keep<false, AX>(U, P, Wm, Wp, b);
    }
    VA.Wv[AX][(long)(2 * e) * nf + t] = Wm;
    VA.Wv[AX][(long)(2 * e + 1) * nf + t] = Wp;
#pragma unroll
    for (int q = 0; q < NB; q++) VA.Kb[AX][(long)(NB * e + q) * nf + t] = b[q];
}

template <int DIM, int MODEL, int NSP, int SCHEME, int AX>
__device__ __forceinline__ void face_bwd_riemann_item(const Params& P, const Geom& g, const Scratch& S,
                                                      const VjpArgs& VA, long t) {
    using M = Model<DIM, MODEL, NSP>;
    using FL = FaceLayout<NSP>;
    constexpr int NEQ = M::NEQ;
    const long nf = nface_of(g, AX);
    const long nc = ncell_of(g);
    int i, j, k;
    long xR, st;
    face_coords<DIM, AX>(g, t, i, j, k, xR, st);
    const int fa = AX == 0 ? i : (AX == 1 ? j : k);     // face coordinate along AX, in [-1, n+1]
    const long xL = xR - st;

    // adjoints of the midpoint flux and midpoint velocity of this face
    double Fmb[NEQ];
#pragma unroll
    for (int e = 0; e < NEQ; e++)
        Fmb[e] = VA.dt*(double(23)/double(15)*Fface_bar<DIM, MODEL, NSP, AX>(g, VA, i, j, k, fa, e) +
                        double(1)/double(30)*(Fface_bar<DIM, MODEL, NSP, AX>(g, VA, i, j, k, fa - 1, e) +
                                              Fface_bar<DIM, MODEL, NSP, AX>(g, VA, i, j, k, fa + 1, e)));
    double umb = 0.0;
    if constexpr (MODEL == FIVE_EQN_ALLAIRE) {
        umb = (double(3)/double(2)*(usrc_bar<DIM, MODEL, NSP, AX>(g, VA, i, j, k, fa - 1) -
                                    usrc_bar<DIM, MODEL, NSP, AX>(g, VA, i, j, k, fa)) +
               double(1)/double(30)*(usrc_bar<DIM, MODEL, NSP, AX>(g, VA, i, j, k, fa - 2) -
                                     usrc_bar<DIM, MODEL, NSP, AX>(g, VA, i, j, k, fa + 1)))/g.dx[AX];
    }

    // forward recompute (the exact form of face_item); the projection and the
    // reconstructed characteristic values come from face_proj_item / face_fwd_weno_item
    const double theta_avg = 0.5*(S.theta[xL] + S.theta[xR]);
    const double Omega_avg = 0.5*(S.Omega[xL] + S.Omega[xR]);
    const double sensor = -theta_avg/(fabs(theta_avg) + Omega_avg + HMR_EPS);
    const bool use_hll = sensor > 0.65;
    FaceProj<DIM, MODEL, NSP> F;
    load_proj<DIM, MODEL, NSP>(VA.Fp[AX], nf, t, F);
    double Wm[NEQ], Wp[NEQ];
#pragma unroll
    for (int e = 0; e < NEQ; e++) {
        Wm[e] = VA.Wv[AX][(long)(2 * e) * nf + t];
        Wp[e] = VA.Wv[AX][(long)(2 * e + 1) * nf + t];
    }
    double VL[NEQ], VR[NEQ];
    prim_from_char<true, DIM, MODEL, NSP, AX>(F, Wm, VL);
    prim_from_char<true, DIM, MODEL, NSP, AX>(F, Wp, VR);
    double mL, mR;
    const bool ok = face_bounded<DIM, MODEL, NSP>(P, VL, mL) & face_bounded<DIM, MODEL, NSP>(P, VR, mR);
    if (!ok) {
#pragma unroll
        for (int e = 0; e < NEQ; e++) { VL[e] = S.V[e * nc + xL]; VR[e] = S.V[e * nc + xR]; }
    }

    // reverse of the Riemann solve
    double VLb[NEQ], VRb[NEQ];
#pragma unroll
    for (int e = 0; e < NEQ; e++) { VLb[e] = 0.0; VRb[e] = 0.0; }
    double umid;
    riemann_bwd<DIM, MODEL, NSP, AX>(P, VL, VR, use_hll, Fmb, umb, VLb, VRb, umid);
    if constexpr (MODEL == FIVE_EQN_ALLAIRE) S.um[AX][t] = umid;
    VA.okf[AX][t] = ok ? 1 : 0;
    double* Cb = VA.Cb[AX];
    if (!ok) {
        // first order: the face states are the two cells' primitive variables
#pragma unroll
        for (int m = 0; m < 6; m++)
#pragma unroll
            for (int e = 0; e < NEQ; e++)
                Cb[(long)(m * NEQ + e) * nf + t] = m == 2 ? VLb[e] : (m == 3 ? VRb[e] : 0.0);
        Cb[(long)(6 * NEQ) * nf + t] = 0.0;
        Cb[(long)(6 * NEQ + 1) * nf + t] = 0.0;
        return;
    }
    double Wmb[NEQ], Wpb[NEQ];
#pragma unroll
    for (int e = 0; e < NEQ; e++) { Wmb[e] = 0.0; Wpb[e] = 0.0; }
    FaceProjBar<NSP> Fb;
    Fb.p_hrc = 0.0; Fb.ic2 = 0.0; Fb.irc = 0.0;
#pragma unroll
    for (int q = 0; q < NSP; q++) { Fb.zr[q] = 0.0; Fb.hz[q] = 0.0; }
    prim_from_char_bwd<DIM, MODEL, NSP, AX>(F, Wm, VLb, Wmb, Fb);
    prim_from_char_bwd<DIM, MODEL, NSP, AX>(F, Wp, VRb, Wpb, Fb);
    double* Wb = VA.Wb[AX];
#pragma unroll
    for (int e = 0; e < NEQ; e++) {
        Wb[(long)(2 * e) * nf + t] = Wmb[e];
        Wb[(long)(2 * e + 1) * nf + t] = Wpb[e];
    }
    double* Fp = VA.Fp[AX];
    Fp[(long)(FL::F + 0) * nf + t] = Fb.p_hrc;
    Fp[(long)(FL::F + 1) * nf + t] = Fb.ic2;
    Fp[(long)(FL::F + 2) * nf + t] = Fb.irc;
#pragma unroll
    for (int q = 0; q < NSP; q++) Fp[(long)(FL::F + 3 + q) * nf + t] = Fb.hz[q];
}

// Item u = e*nf + t: characteristic variable e of face t.
template <int DIM, int MODEL, int NSP, int SCHEME, int AX>
__device__ __forceinline__ void face_bwd_weno_item(const Params& P, const Geom& g, const Scratch& S,
                                                   const VjpArgs& VA, long u) {
    using M = Model<DIM, MODEL, NSP>;
    constexpr int NEQ = M::NEQ;
    const long nf = nface_of(g, AX);
    const long t = u % nf;
    const int e = (int)(u / nf);
    if (!VA.okf[AX][t]) return;
    const long nc = ncell_of(g);
    int i, j, k;
    long xR, st;
    face_coords<DIM, AX>(g, t, i, j, k, xR, st);
    FaceProj<DIM, MODEL, NSP> F;
    load_proj<DIM, MODEL, NSP>(VA.Fp[AX], nf, t, F);
    double U[6], Ub[6] = {0, 0, 0, 0, 0, 0};
    char_stencil<DIM, MODEL, NSP, AX>(g, S, F, xR, st, e, U);
    const double Wmb = VA.Wb[AX][(long)(2 * e) * nf + t];
    const double Wpb = VA.Wb[AX][(long)(2 * e + 1) * nf + t];
    constexpr int NB = weno_kept<SCHEME>();
    double b[NB];
#pragma unroll
    for (int q = 0; q < NB; q++) b[q] = VA.Kb[AX][(long)(NB * e + q) * nf + t];
    if constexpr (SCHEME == WCNS5_JS) js_pair_bwd(U, b, P.p, Wmb, Wpb, Ub);
    else if constexpr (SCHEME == WCNS6_LD) ld_pair_bwd(U, b, P, Wmb, Wpb, Ub);
    else if constexpr (SCHEME == WCNS5_Z) z_pair_bwd(U, b, P.p, Wmb, Wpb, Ub);
    else cu_pair_bwd<AX>(U, b, P, Wmb, Wpb, Ub);
    double* Cb = VA.Cb[AX];
#pragma unroll
    for (int m = 0; m < 6; m++) Cb[(long)(m * NEQ + e) * nf + t] = Ub[m];
}

template <int DIM, int MODEL, int NSP, int AX>
__device__ __forceinline__ void face_bwd_char_item(const Geom& g, const Scratch& S, const VjpArgs& VA, long t) {
    using M = Model<DIM, MODEL, NSP>;
    using FL = FaceLayout<NSP>;
    constexpr int NEQ = M::NEQ;
    const long nf = nface_of(g, AX);
    if (!VA.okf[AX][t]) return;
    const long nc = ncell_of(g);
    int i, j, k;
    long xR, st;
    face_coords<DIM, AX>(g, t, i, j, k, xR, st);
    const double* Fp = VA.Fp[AX];
    FaceProj<DIM, MODEL, NSP> F;
    load_proj<DIM, MODEL, NSP>(Fp, nf, t, F);
    FaceProjBar<NSP> Fb;
    Fb.p_hrc = Fp[(long)(FL::F + 0) * nf + t];
    Fb.ic2 = Fp[(long)(FL::F + 1) * nf + t];
    Fb.irc = Fp[(long)(FL::F + 2) * nf + t];
#pragma unroll
    for (int q = 0; q < NSP; q++) { Fb.hz[q] = Fp[(long)(FL::F + 3 + q) * nf + t]; Fb.zr[q] = 0.0; }
    double* Cb = VA.Cb[AX];
    double zbb[NSP];
#pragma unroll
    for (int q = 0; q < NSP; q++) zbb[q] = 0.0;
#pragma unroll
    for (int m = 0; m < 6; m++) {
        double Vm[NEQ], Vb[NEQ];
        const long x = xR + (m - 3) * st;
#pragma unroll
        for (int q = 0; q < NEQ; q++) { Vm[q] = S.V[q * nc + x]; Vb[q] = 0.0; }
#pragma unroll
        for (int e = 0; e < NEQ; e++)
            char_one_bwd<DIM, MODEL, NSP, AX>(F, Vm, e, Cb[(long)(m * NEQ + e) * nf + t], Vb, Fb);
        // row m held the WCNS adjoints of the stencil values; it now takes the primitive-variable ones
#pragma unroll
        for (int e = 0; e < NEQ; e++) Cb[(long)(m * NEQ + e) * nf + t] = Vb[e];
    }
    double rbb = 0.0, cbb = 0.0;
    face_proj_bwd<DIM, MODEL, NSP>(F, Fb, rbb, cbb, zbb);
    if constexpr (MODEL != SINGLE_SPECIES) {
#pragma unroll
        for (int q = 0; q < NSP; q++) {
            Cb[(long)(2 * NEQ + q) * nf + t] += 0.5*zbb[q];
            Cb[(long)(3 * NEQ + q) * nf + t] += 0.5*zbb[q];
        }
    }
    Cb[(long)(6 * NEQ) * nf + t] = rbb;
    Cb[(long)(6 * NEQ + 1) * nf + t] = cbb;
}

// ---------------------------------------------------------------------------
// Cell phase of the adjoint.
// ---------------------------------------------------------------------------
// Adjoint of the node (cell-centre) flux along AX at one cell.
template <int DIM, int MODEL, int NSP, int AX>
__device__ __forceinline__ void node_flux_bwd(const double* Q, const double* V, const double* Fnb, double* Vb,
                                              double* Qb) {
    using M = Model<DIM, MODEL, NSP>;
    const double un = V[M::IU + AX];
    const double p = V[M::IP];
    double unb = 0.0, pb = 0.0;
    if constexpr (MODEL == SINGLE_SPECIES) {
        Qb[1 + AX] += Fnb[0];
#pragma unroll
        for (int k = 0; k < DIM; k++) {
            unb += Fnb[1 + k]*Q[1 + k];
            Qb[1 + k] += un*Fnb[1 + k];
            if (k == AX) pb += Fnb[1 + k];
        }
        unb += Fnb[DIM + 1]*(Q[DIM + 1] + p);
        Qb[DIM + 1] += un*Fnb[DIM + 1];
        pb += un*Fnb[DIM + 1];
    } else {
#pragma unroll
        for (int e = 0; e < M::NEQ; e++) {
            if (e == NSP + DIM) {
                unb += Fnb[e]*(Q[e] + p);
                pb += un*Fnb[e];
            } else {
                unb += Fnb[e]*Q[e];
                if (e == NSP + AX) pb += Fnb[e];
            }
            Qb[e] += un*Fnb[e];
        }
    }
    Vb[M::IU + AX] += unb;
    Vb[M::IP] += pb;
}

// Contributions of axis AX to the adjoints of cell (i, j, k) (ghost-box coordinates).
template <int DIM, int MODEL, int NSP, int AX>
__device__ __forceinline__ void cell_axis_bwd(const Geom& g, const Scratch& S, const VjpArgs& VA, int i, int j,
                                              int k, long x, const double* Q, const double* V, double* Vb,
                                              double& rb, double& cb, double* Qb) {
    using M = Model<DIM, MODEL, NSP>;
    constexpr int NEQ = M::NEQ;
    const int c[3] = {i, j, k};
    // faces of axis AX span the interior along the other axes
#pragma unroll
    for (int d = 0; d < DIM; d++)
        if (d != AX && (c[d] < 0 || c[d] >= g.n[d])) return;
    const int ca = c[AX];
    const long nf = nface_of(g, AX);
    const double* Cb = VA.Cb[AX];
    auto fid = [&](int f) {
        return fidx<AX>(g, AX == 0 ? f : i, AX == 1 ? f : j, AX == 2 ? f : k);
    };
    // stencil contributions: this cell is offset m - 3 from the face with xR = ca + 3 - m
#pragma unroll
    for (int m = 0; m < 6; m++) {
        const int f = ca + 3 - m;
        if (f < -1 || f > g.n[AX] + 1) continue;
        const long ft = fid(f);
#pragma unroll
        for (int e = 0; e < NEQ; e++) Vb[e] += Cb[(long)(m * NEQ + e) * nf + ft];
    }
    // projection means: xR of face ca, xL of face ca + 1
    if (ca >= -1 && ca <= g.n[AX] + 1) {
        const long ft = fid(ca);
        rb += 0.5*Cb[(long)(6 * NEQ) * nf + ft];
        cb += 0.5*Cb[(long)(6 * NEQ + 1) * nf + ft];
    }
    if (ca + 1 >= -1 && ca + 1 <= g.n[AX] + 1) {
        const long ft = fid(ca + 1);
        rb += 0.5*Cb[(long)(6 * NEQ) * nf + ft];
        cb += 0.5*Cb[(long)(6 * NEQ + 1) * nf + ft];
    }
    // node flux of this cell enters the faces ca and ca + 1
    if (ca >= -1 && ca <= g.n[AX]) {
        double Fnb[NEQ];
        bool any = false;
#pragma unroll
        for (int e = 0; e < NEQ; e++) {
            Fnb[e] = -double(3)/double(10)*VA.dt*(Fface_bar<DIM, MODEL, NSP, AX>(g, VA, i, j, k, ca, e) +
                                                  Fface_bar<DIM, MODEL, NSP, AX>(g, VA, i, j, k, ca + 1, e));
            any = any || Fnb[e] != 0.0;
        }
        if (any) node_flux_bwd<DIM, MODEL, NSP, AX>(Q, V, Fnb, Vb, Qb);
        if constexpr (MODEL == FIVE_EQN_ALLAIRE) {
            // velocity at this cell in the source speed term of cells ca -/+ 1
            Vb[M::IU + AX] += (-double(3)/double(10)*usrc_bar<DIM, MODEL, NSP, AX>(g, VA, i, j, k, ca - 1) +
                               double(3)/double(10)*usrc_bar<DIM, MODEL, NSP, AX>(g, VA, i, j, k, ca + 1))/g.dx[AX];
        }
    }
    // advective source: d(dt Q_Z sum_a usrc_a)/dQ_Z for the interior cell itself
    if constexpr (MODEL == FIVE_EQN_ALLAIRE) {
        if (ca >= 0 && ca < g.n[AX]) {
            const long st = (AX == 0) ? 1 : (AX == 1 ? (long)g.G[0] : (long)g.G[0] * g.G[1]);
            const long f = fid(ca);
            const long fst = (AX == 0) ? 1 : (AX == 1 ? (long)g.n[0] : (long)g.n[0] * g.n[1]);
            const double* um = S.um[AX];
            const long ncl = ncell_of(g);
            const double* u = S.V + (M::IU + AX) * ncl;
            const double us = (double(3)/double(2)*(um[f + fst] - um[f]) -
                               double(3)/double(10)*(u[x + st] - u[x - st]) +
                               double(1)/double(30)*(um[f + 2 * fst] - um[f - fst]))/g.dx[AX];
#pragma unroll
            for (int q = 0; q < M::NZ; q++)
                Qb[M::IZ + q] += VA.beta*qbar_eff<DIM, MODEL, NSP>(VA, x, M::IZ + q)*VA.dt*us;
        }
    }
}

template <int DIM, int MODEL, int NSP>
__device__ __forceinline__ void cell_bwd_item(const Params& P, const Geom& g, const Scratch& S, const VjpArgs& VA,
                                              long x) {
    using M = Model<DIM, MODEL, NSP>;
    constexpr int NEQ = M::NEQ;
    constexpr int NCOMP = M::NCOMP;
    const long nc = ncell_of(g);
    {
        const int i = (int)(x % g.G[0]) - g.gh;
        const int j = (int)((x / g.G[0]) % g.G[1]) - g.gh;
        const int k = DIM == 3 ? (int)(x / ((long)g.G[0] * g.G[1])) - g.gh : 0;
        const bool interior = i >= 0 && i < g.n[0] && j >= 0 && j < g.n[1] && (DIM == 2 || (k >= 0 && k < g.n[2]));
        // alpha terms (interior; equations only: the stored last volume fraction is not an input of the update)
        if (interior) {
            for (int n = 0; n < VA.nst; n++) {
                if (VA.alpha[n] == 0.0) continue;
#pragma unroll
                for (int e = 0; e < NEQ; e++)
                    VA.Qbi[n].p[e][x] += VA.alpha[n]*qbar_eff<DIM, MODEL, NSP>(VA, x, e);
            }
        }
        if (VA.beta == 0.0) return;
        double Q[NCOMP], V[NEQ], Vb[NEQ], Qb[NCOMP];
#pragma unroll
        for (int e = 0; e < NCOMP; e++) { Q[e] = VA.Qs.p[e][x]; Qb[e] = 0.0; }
#pragma unroll
        for (int e = 0; e < NEQ; e++) { V[e] = S.V[e * nc + x]; Vb[e] = 0.0; }
        double rb = 0.0, cb = 0.0;
        if (VA.Dv != nullptr) {
#pragma unroll
            for (int e = 0; e < NEQ; e++) Vb[e] = VA.Dv[e * nc + x];
        }
        cell_axis_bwd<DIM, MODEL, NSP, 0>(g, S, VA, i, j, k, x, Q, V, Vb, rb, cb, Qb);
        cell_axis_bwd<DIM, MODEL, NSP, 1>(g, S, VA, i, j, k, x, Q, V, Vb, rb, cb, Qb);
        if constexpr (DIM == 3) cell_axis_bwd<DIM, MODEL, NSP, 2>(g, S, VA, i, j, k, x, Q, V, Vb, rb, cb, Qb);
        bool any = rb != 0.0 || cb != 0.0;
#pragma unroll
        for (int e = 0; e < NEQ; e++) any = any || Vb[e] != 0.0;
        if (any) cell_derived_bwd<DIM, MODEL, NSP>(P, Q, Vb, rb, cb, Qb);
        const int s = VA.nst - 1;
#pragma unroll
        for (int e = 0; e < NCOMP; e++)
            if (Qb[e] != 0.0) VA.Qbi[s].p[e][x] += Qb[e];
    }
}

}  // namespace hmr

#include "hmr_diffusive_vjp.cuh"
