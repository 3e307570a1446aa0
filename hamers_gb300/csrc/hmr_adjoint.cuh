// Reverse mode (vector-Jacobian products) of the face and cell computations
// of one RK substep.
//
// Every routine first recomputes its forward values with the reference's
// operation order (the X = true forms of hmr_physics.cuh), so that every
// discrete choice -- bounds check and first-order fallback, shock sensor,
// HLLC side, WCNS6-LD tau switch, min/max branches -- is the one the forward
// substep takes, and then propagates adjoints along that branch.  The one
// exception is the WCNS weighting of faces the HLLC (not HLLC-HLL) flux takes:
// it is recomputed in the regrouped form (X = false), within rounding of the
// reference's, from the reference's own smoothness indicators, so the WCNS
// decisions are the forward's and the Riemann decisions differ only where a
// reconstructed state sits within rounding of a threshold.
// Conventions at non-smooth points (shared with the CPU tangent of the oracle):
//   |x|        : sign(x), 0 at x = 0
//   fmin(a, b) : adjoint to a if a < b, else to b
//   fmax(a, b) : adjoint to a if a > b, else to b
//   sqrt(x)    : 0 at x = 0
// Where two expressions of the forward are equal as functions (the sound
// speed c^2 = Gamma p/rho + sum_i Y_i Psi_i equals gamma p/rho for both
// multi-species models because sum_i Y_i = 1 identically), the adjoint uses
// the simpler one; the derivative is the same.
#pragma once

#include "hmr_kernels.cuh"

namespace hmr {

__device__ __forceinline__ double sgn_(double x) { return x > 0.0 ? 1.0 : (x < 0.0 ? -1.0 : 0.0); }

// b^e for e >= 0 (1 for e = 0).
__device__ __forceinline__ double ipow0(double b, int e) {
    double r = 1.0;
    for (int i = 0; i < e; i++) r *= b;
    return r;
}

// Reciprocals 1/e_k of three or four positive values from one division,
// 1/e_k = (prod_{j!=k} e_j)/(prod_j e_j): the reverse sides take them for the
// derivative values only (e_k = beta_k + eps in [1e-15, 1e77) keeps the products in range).
__device__ __forceinline__ void recip3(double e0, double e1, double e2, double* r) {
    const double e12 = e1*e2;
    const double rp = double(1)/(e0*e12);
    r[0] = rp*e12; r[1] = rp*(e0*e2); r[2] = rp*(e0*e1);
}

__device__ __forceinline__ void recip4(double e0, double e1, double e2, double e3, double* r) {
    const double e01 = e0*e1, e23 = e2*e3;
    const double rp = double(1)/(e01*e23);
    r[0] = rp*(e1*e23); r[1] = rp*(e0*e23); r[2] = rp*(e01*e3); r[3] = rp*(e01*e2);
}

// ----------------------------------------------------------------------------
// Smoothness-indicator gradients.
// ----------------------------------------------------------------------------
// JS beta_0..2 of the stencil S0..S4 (upwind first): accumulates into Sb.
__device__ __forceinline__ void js_betas_bwd(const double* S, double bb0, double bb1, double bb2, double* Sb) {
    const double t = double(1)/double(3);
    Sb[0] += t*bb0*(8.0*S[0] - 19.0*S[1] + 11.0*S[2]);
    Sb[1] += t*bb0*(-19.0*S[0] + 50.0*S[1] - 31.0*S[2]);
    Sb[2] += t*bb0*(11.0*S[0] - 31.0*S[1] + 20.0*S[2]);
    Sb[1] += t*bb1*(8.0*S[1] - 13.0*S[2] + 5.0*S[3]);
    Sb[2] += t*bb1*(-13.0*S[1] + 26.0*S[2] - 13.0*S[3]);
    Sb[3] += t*bb1*(5.0*S[1] - 13.0*S[2] + 8.0*S[3]);
    Sb[2] += t*bb2*(20.0*S[2] - 31.0*S[3] + 11.0*S[4]);
    Sb[3] += t*bb2*(-31.0*S[2] + 50.0*S[3] - 19.0*S[4]);
    Sb[4] += t*bb2*(11.0*S[2] - 19.0*S[3] + 8.0*S[4]);
}

// WCNS6-LD beta_3 = Q(S)/232243200 with Q = sum_{i<=j} c_ij S_i S_j (the
// coefficients of ld_beta3): accumulates bb3 * dbeta_3/dS into Sb.
__device__ __forceinline__ void ld_beta3_bwd(const double* S, double bb3, double* Sb) {
    // upper triangle c_ij, i <= j
    constexpr double c00 = 525910327.0, c01 = -4562164630.0, c02 = 7799501420.0, c03 = -6610694540.0,
                     c04 = 2794296070.0, c05 = -472758974.0;
    constexpr double c11 = 5.0*2146987907.0, c12 = -5.0*7722406988.0, c13 = 5.0*6763559276.0,
                     c14 = -5.0*2926461814.0, c15 = 5.0*503766638.0;
    constexpr double c22 = 20.0*1833221603.0, c23 = -20.0*3358664662.0, c24 = 20.0*1495974539.0,
                     c25 = -20.0*263126407.0;
    constexpr double c33 = 20.0*1607794163.0, c34 = -20.0*1486026707.0, c35 = 20.0*268747951.0;
    constexpr double c44 = 5.0*1432381427.0, c45 = -5.0*536951582.0;
    constexpr double c55 = 263126407.0;
    const double f = bb3/232243200.0;
    Sb[0] += f*(2.0*c00*S[0] + c01*S[1] + c02*S[2] + c03*S[3] + c04*S[4] + c05*S[5]);
    Sb[1] += f*(c01*S[0] + 2.0*c11*S[1] + c12*S[2] + c13*S[3] + c14*S[4] + c15*S[5]);
    Sb[2] += f*(c02*S[0] + c12*S[1] + 2.0*c22*S[2] + c23*S[3] + c24*S[4] + c25*S[5]);
    Sb[3] += f*(c03*S[0] + c13*S[1] + c23*S[2] + 2.0*c33*S[3] + c34*S[4] + c35*S[5]);
    Sb[4] += f*(c04*S[0] + c14*S[1] + c24*S[2] + c34*S[3] + 2.0*c44*S[4] + c45*S[5]);
    Sb[5] += f*(c05*S[0] + c15*S[1] + c25*S[2] + c35*S[3] + c45*S[4] + 2.0*c55*S[5]);
}

// ----------------------------------------------------------------------------
// WCNS5-JS, one side: S[0..4] from the upwind side, obar = adjoint of the
// midpoint value; accumulates Sb[0..4].
// ----------------------------------------------------------------------------
__device__ __forceinline__ void js_side_bwd(int p, const double* S, double b0, double b1, double b2, double obar,
                                            double* Sb) {
    // alpha_k = d_k/(b_k + eps)^p, w_k = alpha_k/sum alpha (reciprocals: derivative values only)
    double rr[3];
    recip3(b0 + HMR_EPS, b1 + HMR_EPS, b2 + HMR_EPS, rr);
    const double r0 = rr[0], r1 = rr[1], r2 = rr[2];
    const double a0 = (double(1)/double(16))*ipow0(r0, p);
    const double a1 = (double(5)/double(8))*ipow0(r1, p);
    const double a2 = (double(5)/double(16))*ipow0(r2, p);
    const double iA = double(1)/(a0 + a1 + a2);
    const double w0 = a0*iA, w1 = a1*iA, w2 = a2*iA;
    const double q0 = 3.0/8.0*S[0] - 10.0/8.0*S[1] + 15.0/8.0*S[2];
    const double q1 = -1.0/8.0*S[1] + 6.0/8.0*S[2] + 3.0/8.0*S[3];
    const double q2 = 3.0/8.0*S[2] + 6.0/8.0*S[3] - 1.0/8.0*S[4];
    Sb[0] += obar*(3.0/8.0*w0);
    Sb[1] += obar*(-10.0/8.0*w0 - 1.0/8.0*w1);
    Sb[2] += obar*(15.0/8.0*w0 + 6.0/8.0*w1 + 3.0/8.0*w2);
    Sb[3] += obar*(3.0/8.0*w1 + 6.0/8.0*w2);
    Sb[4] += obar*(-1.0/8.0*w2);
    // d out/d b_k = sum_j q_j dw_j/db_k = -p r_k w_k (q_k - out)
    const double out = w0*q0 + w1*q1 + w2*q2;
    const double bb0 = -obar*p*r0*w0*(q0 - out);
    const double bb1 = -obar*p*r1*w1*(q1 - out);
    const double bb2 = -obar*p*r2*w2*(q2 - out);
    js_betas_bwd(S, bb0, bb1, bb2, Sb);
}

// The adjoint's forward recomputation of the smoothness indicators runs one (face, variable)
// item per thread at high occupancy, where integer-pipe multiplications (hmr_emu64.cuh) can run
// beside the native FP64 pipe; HMR_EMU_BETA_VJP takes the mask encoding of HMR_EMU_BETA.  The
// result bits are the same either way.
#ifndef HMR_EMU_BETA_VJP
#define HMR_EMU_BETA_VJP 0
#endif
constexpr int EMU_VJP_M = HMR_EMU_BETA_VJP & 3;
constexpr int EMU_VJP_P = (HMR_EMU_BETA_VJP >> 2) & 3;

// Forward of both sides (the operations of js_pair<X>) keeping the smoothness
// indicators: b[0..2] of the minus side, b[3..5] of the plus side.
template <bool X>
__device__ __forceinline__ void js_pair_keep(const double* U, int p, double& Um, double& Up, double* b) {
    js_betas_x<EMU_VJP_M>(U[0], U[1], U[2], U[3], U[4], b[0], b[1], b[2]);
    Um = js_interp<X>(b[0], b[1], b[2], p, U[0], U[1], U[2], U[3], U[4]);
    js_betas_x<EMU_VJP_P>(U[5], U[4], U[3], U[2], U[1], b[3], b[4], b[5]);
    Up = js_interp<X>(b[3], b[4], b[5], p, U[5], U[4], U[3], U[2], U[1]);
}

// Both sides of one characteristic variable: U[0..5] at cells face-3..face+2,
// b the indicators kept by js_pair_keep.
__device__ __forceinline__ void js_pair_bwd(const double* U, const double* b, int p, double Umb, double Upb,
                                            double* Ub) {
    double Sb[5] = {0, 0, 0, 0, 0};
    js_side_bwd(p, U, b[0], b[1], b[2], Umb, Sb);
#pragma unroll
    for (int j = 0; j < 5; j++) Ub[j] += Sb[j];
    const double R[5] = {U[5], U[4], U[3], U[2], U[1]};
    double Rb[5] = {0, 0, 0, 0, 0};
    js_side_bwd(p, R, b[3], b[4], b[5], Upb, Rb);
#pragma unroll
    for (int j = 0; j < 5; j++) Ub[5 - j] += Rb[j];
}

// ----------------------------------------------------------------------------
// WCNS6-LD.
// ----------------------------------------------------------------------------
// sigma = max(t1, t2), t = |a - b|/(|a| + |b| + eps): accumulates sigb*dsigma/dU.
__device__ __forceinline__ void ld_sigma_bwd(const double* U, double sigb, double* Ub) {
    const double a1 = sub_(U[2], U[1]);
    const double a2 = sub_(U[3], U[2]);
    const double a3 = sub_(U[4], U[3]);
    const double D1 = add_(add_(fabs(a1), fabs(a2)), HMR_EPS);
    const double D2 = add_(add_(fabs(a2), fabs(a3)), HMR_EPS);
    const double t1 = fabs(sub_(a1, a2))/D1;
    const double t2 = fabs(sub_(a2, a3))/D2;
    double ab1 = 0.0, ab2 = 0.0, ab3 = 0.0;
    if (t1 > t2) {
        const double s = sgn_(a1 - a2);
        ab1 += sigb*(s/D1 - t1*sgn_(a1)/D1);
        ab2 += sigb*(-s/D1 - t1*sgn_(a2)/D1);
    } else {
        const double s = sgn_(a2 - a3);
        ab2 += sigb*(s/D2 - t2*sgn_(a2)/D2);
        ab3 += sigb*(-s/D2 - t2*sgn_(a3)/D2);
    }
    Ub[2] += ab1; Ub[1] -= ab1;
    Ub[3] += ab2; Ub[2] -= ab2;
    Ub[4] += ab3; Ub[3] -= ab3;
}

// One side: S[0..5] from the upwind side.  Accumulates Sb and the adjoint of sigma.
__device__ __forceinline__ void ld_side_bwd(const Params& P, double sigma, const double* S, const double* b,
                                            double obar, double* Sb, double& sigb) {
    // decision inputs, exactly as in ld_interp
    const double tau_5 = fabs(sub_(b[0], b[2]));
    const double beta_avg = mul_(double(1)/double(8), add_(add_(b[0], b[2]), mul_(double(6), b[1])));
    const double tau_6 = fabs(sub_(b[3], beta_avg));
    const bool blend = ld_switch(tau_6, beta_avg, P.alpha_tau);
    // weights, with reciprocals (derivative values only)
    const double du[3] = {1.0/16.0, 5.0/8.0, 5.0/16.0};
    const double dc[4] = {1.0/32.0, 15.0/32.0, 15.0/32.0, 1.0/32.0};
    double r[4], xu[3] = {0, 0, 0}, xo[4], pu1[3] = {0, 0, 0}, po1[4], ur[3] = {0, 0, 0}, orw[4];
    recip4(b[0] + HMR_EPS, b[1] + HMR_EPS, b[2] + HMR_EPS, b[3] + HMR_EPS, r);
    double Us = 1.0, Os = 0.0;
    if (blend) {   // the upwind weights only enter where the switch blends
        Us = 0.0;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            xu[k] = tau_5*r[k];
            pu1[k] = ipow0(xu[k], P.p - 1);
            ur[k] = du[k]*(1.0 + pu1[k]*xu[k]);
            Us += ur[k];
        }
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
        xo[k] = tau_6*r[k];
        po1[k] = ipow0(xo[k], P.q - 1);
        orw[k] = dc[k]*(P.C + po1[k]*xo[k]);
        Os += orw[k];
    }
    const double iUs = blend ? double(1)/Us : 0.0, iOs = double(1)/Os;
    double u[3], o[4], of[4];
#pragma unroll
    for (int k = 0; k < 3; k++) u[k] = ur[k]*iUs;
#pragma unroll
    for (int k = 0; k < 4; k++) o[k] = orw[k]*iOs;
    if (blend) {
#pragma unroll
        for (int k = 0; k < 3; k++) of[k] = sigma*u[k] + (1.0 - sigma)*o[k];
        of[3] = (1.0 - sigma)*o[3];
    } else {
#pragma unroll
        for (int k = 0; k < 4; k++) of[k] = o[k];
    }
    const double q[4] = {3.0/8.0*S[0] - 10.0/8.0*S[1] + 15.0/8.0*S[2],
                         -1.0/8.0*S[1] + 6.0/8.0*S[2] + 3.0/8.0*S[3],
                         3.0/8.0*S[2] + 6.0/8.0*S[3] - 1.0/8.0*S[4],
                         15.0/8.0*S[3] - 10.0/8.0*S[4] + 3.0/8.0*S[5]};
    Sb[0] += obar*(3.0/8.0*of[0]);
    Sb[1] += obar*(-10.0/8.0*of[0] - 1.0/8.0*of[1]);
    Sb[2] += obar*(15.0/8.0*of[0] + 6.0/8.0*of[1] + 3.0/8.0*of[2]);
    Sb[3] += obar*(3.0/8.0*of[1] + 6.0/8.0*of[2] + 15.0/8.0*of[3]);
    Sb[4] += obar*(-1.0/8.0*of[2] - 10.0/8.0*of[3]);
    Sb[5] += obar*(3.0/8.0*of[3]);
    double ofb[4], ub[3] = {0, 0, 0}, ob[4];
#pragma unroll
    for (int k = 0; k < 4; k++) ofb[k] = obar*q[k];
    if (blend) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
            ub[k] = sigma*ofb[k];
            ob[k] = (1.0 - sigma)*ofb[k];
            sigb += ofb[k]*(u[k] - o[k]);
        }
        ob[3] = (1.0 - sigma)*ofb[3];
        sigb -= ofb[3]*o[3];
    } else {
#pragma unroll
        for (int k = 0; k < 4; k++) ob[k] = ofb[k];
    }
    const double dotu = ub[0]*u[0] + ub[1]*u[1] + ub[2]*u[2];
    const double doto = ob[0]*o[0] + ob[1]*o[1] + ob[2]*o[2] + ob[3]*o[3];
    double rb[4] = {0, 0, 0, 0}, bb[4];
    double tau5b = 0.0, tau6b = 0.0;
    if (blend) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const double xub = (ub[k] - dotu)*iUs*du[k]*P.p*pu1[k];
            tau5b += xub*r[k];
            rb[k] += xub*tau_5;
        }
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const double xob = (ob[k] - doto)*iOs*dc[k]*P.q*po1[k];
        tau6b += xob*r[k];
        rb[k] += xob*tau_6;
    }
#pragma unroll
    for (int k = 0; k < 4; k++) bb[k] = -rb[k]*r[k]*r[k];
    const double s6 = sgn_(b[3] - beta_avg);
    bb[3] += tau6b*s6;
    const double bavgb = -tau6b*s6;
    bb[0] += bavgb/8.0;
    bb[2] += bavgb/8.0;
    bb[1] += bavgb*6.0/8.0;
    const double s5 = sgn_(b[0] - b[2]);
    bb[0] += tau5b*s5;
    bb[2] -= tau5b*s5;
    js_betas_bwd(S, bb[0], bb[1], bb[2], Sb);
    ld_beta3_bwd(S, bb[3], Sb);
}

// Forward of both sides (the operations of ld_pair<X>) keeping the smoothness
// indicators b[0..3] (minus side), b[4..7] (plus side) and sigma (b[8]; negative
// where neither side blends, since sigma then enters nothing).
template <bool X>
__device__ __forceinline__ void ld_pair_keep(const double* U, const Params& P, double& Um, double& Up, double* b) {
    double sg = -1.0;
    js_betas_x<EMU_VJP_M>(U[0], U[1], U[2], U[3], U[4], b[0], b[1], b[2]);
    b[3] = ld_beta3<EMU_VJP_M>(U[0], U[1], U[2], U[3], U[4], U[5]);
    Um = ld_interp<X>(b, U, sg, P, U[0], U[1], U[2], U[3], U[4], U[5]);
    js_betas_x<EMU_VJP_P>(U[5], U[4], U[3], U[2], U[1], b[4], b[5], b[6]);
    b[7] = ld_beta3<EMU_VJP_P>(U[5], U[4], U[3], U[2], U[1], U[0]);
    Up = ld_interp<X>(b + 4, U, sg, P, U[5], U[4], U[3], U[2], U[1], U[0]);
    b[8] = sg;
}

__device__ __forceinline__ void ld_pair_bwd(const double* U, const double* b, const Params& P, double Umb,
                                            double Upb, double* Ub) {
    const double sigma = b[8];
    double sigb = 0.0;
    double Sb[6] = {0, 0, 0, 0, 0, 0};
    ld_side_bwd(P, sigma, U, b, Umb, Sb, sigb);
#pragma unroll
    for (int j = 0; j < 6; j++) Ub[j] += Sb[j];
    const double R[6] = {U[5], U[4], U[3], U[2], U[1], U[0]};
    double Rb[6] = {0, 0, 0, 0, 0, 0};
    ld_side_bwd(P, sigma, R, b + 4, Upb, Rb, sigb);
#pragma unroll
    for (int j = 0; j < 6; j++) Ub[5 - j] += Rb[j];
    if (sigma >= 0.0) ld_sigma_bwd(U, sigb, Ub);
}

// ----------------------------------------------------------------------------
// WCNS5-Z, one side: S[0..4] from the upwind side, b[0..2] its indicators.
// w_k = u_k/sum u, u_k = d_k (1 + x_k^p), x_k = tau_5/(b_k + eps), tau_5 = |b_0 - b_2|.
// ----------------------------------------------------------------------------
__device__ __forceinline__ void z_side_bwd(int p, const double* S, const double* b, double obar, double* Sb) {
    const double du[3] = {1.0/16.0, 5.0/8.0, 5.0/16.0};
    const double tau_5 = fabs(sub_(b[0], b[2]));
    double r[3], x[3], px1[3], ur[3], Us = 0.0;
    recip3(b[0] + HMR_EPS, b[1] + HMR_EPS, b[2] + HMR_EPS, r);
#pragma unroll
    for (int k = 0; k < 3; k++) {
        x[k] = tau_5*r[k];
        px1[k] = ipow0(x[k], p - 1);
        ur[k] = du[k]*(1.0 + px1[k]*x[k]);
        Us += ur[k];
    }
    const double iUs = double(1)/Us;
    const double w[3] = {ur[0]*iUs, ur[1]*iUs, ur[2]*iUs};
    const double q[3] = {3.0/8.0*S[0] - 10.0/8.0*S[1] + 15.0/8.0*S[2],
                         -1.0/8.0*S[1] + 6.0/8.0*S[2] + 3.0/8.0*S[3],
                         3.0/8.0*S[2] + 6.0/8.0*S[3] - 1.0/8.0*S[4]};
    Sb[0] += obar*(3.0/8.0*w[0]);
    Sb[1] += obar*(-10.0/8.0*w[0] - 1.0/8.0*w[1]);
    Sb[2] += obar*(15.0/8.0*w[0] + 6.0/8.0*w[1] + 3.0/8.0*w[2]);
    Sb[3] += obar*(3.0/8.0*w[1] + 6.0/8.0*w[2]);
    Sb[4] += obar*(-1.0/8.0*w[2]);
    const double out = w[0]*q[0] + w[1]*q[1] + w[2]*q[2];
    double bb[3], taub = 0.0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        // d out/d u_k = (q_k - out)/sum u
        const double xb = obar*(q[k] - out)*iUs*du[k]*p*px1[k];
        taub += xb*r[k];
        bb[k] = -xb*tau_5*r[k]*r[k];
    }
    const double s5 = sgn_(b[0] - b[2]);
    bb[0] += taub*s5;
    bb[2] -= taub*s5;
    js_betas_bwd(S, bb[0], bb[1], bb[2], Sb);
}

// Forward of both sides (the operations of z_pair<X>) keeping the indicators:
// b[0..2] minus side, b[3..5] plus side.
template <bool X>
__device__ __forceinline__ void z_pair_keep(const double* U, int p, double& Um, double& Up, double* b) {
    js_betas_x<EMU_VJP_M>(U[0], U[1], U[2], U[3], U[4], b[0], b[1], b[2]);
    Um = z_interp<X>(b[0], b[1], b[2], p, U[0], U[1], U[2], U[3], U[4]);
    js_betas_x<EMU_VJP_P>(U[5], U[4], U[3], U[2], U[1], b[3], b[4], b[5]);
    Up = z_interp<X>(b[3], b[4], b[5], p, U[5], U[4], U[3], U[2], U[1]);
}

__device__ __forceinline__ void z_pair_bwd(const double* U, const double* b, int p, double Umb, double Upb,
                                           double* Ub) {
    double Sb[5] = {0, 0, 0, 0, 0};
    z_side_bwd(p, U, b, Umb, Sb);
#pragma unroll
    for (int j = 0; j < 5; j++) Ub[j] += Sb[j];
    const double R[5] = {U[5], U[4], U[3], U[2], U[1]};
    double Rb[5] = {0, 0, 0, 0, 0};
    z_side_bwd(p, R, b + 3, Upb, Rb);
#pragma unroll
    for (int j = 0; j < 5; j++) Ub[5 - j] += Rb[j];
}

// ----------------------------------------------------------------------------
// WCNS6-CU-M2, one side: S[0..5] from the upwind side, b[0..3] its indicators,
// ce = eps dx^2 and cx = Chi dx^2 of the face's axis.
// w_k = o_k/sum o, o_k = dc_k y_k^q, y_k = C + tau_6 (beta_avg + cx)/((b_k + ce)(b_k + cx)),
// beta_avg = (b_0 + b_2 + 6 b_1)/8, tau_6 = |b_3 - beta_avg|.
// ----------------------------------------------------------------------------
__device__ __forceinline__ void cu_side_bwd(const Params& P, double ce, double cx, const double* S, const double* b,
                                            double obar, double* Sb) {
    const double dc[4] = {1.0/32.0, 15.0/32.0, 15.0/32.0, 1.0/32.0};
    const double beta_avg = mul_(double(1)/double(8), add_(add_(b[0], b[2]), mul_(double(6), b[1])));
    const double tau_6 = fabs(sub_(b[3], beta_avg));
    const double ax = beta_avg + cx;
    double ek[4], xk[4], g[4], py1[4], orw[4], Os = 0.0;
    recip4(b[0] + ce, b[1] + ce, b[2] + ce, b[3] + ce, ek);
    recip4(b[0] + cx, b[1] + cx, b[2] + cx, b[3] + cx, xk);
#pragma unroll
    for (int k = 0; k < 4; k++) {
        g[k] = tau_6*ax*ek[k]*xk[k];
        const double y = P.C + g[k];
        py1[k] = ipow0(y, P.q - 1);
        orw[k] = dc[k]*py1[k]*y;
        Os += orw[k];
    }
    const double iOs = double(1)/Os;
    double w[4];
#pragma unroll
    for (int k = 0; k < 4; k++) w[k] = orw[k]*iOs;
    const double q[4] = {3.0/8.0*S[0] - 10.0/8.0*S[1] + 15.0/8.0*S[2],
                         -1.0/8.0*S[1] + 6.0/8.0*S[2] + 3.0/8.0*S[3],
                         3.0/8.0*S[2] + 6.0/8.0*S[3] - 1.0/8.0*S[4],
                         15.0/8.0*S[3] - 10.0/8.0*S[4] + 3.0/8.0*S[5]};
    Sb[0] += obar*(3.0/8.0*w[0]);
    Sb[1] += obar*(-10.0/8.0*w[0] - 1.0/8.0*w[1]);
    Sb[2] += obar*(15.0/8.0*w[0] + 6.0/8.0*w[1] + 3.0/8.0*w[2]);
    Sb[3] += obar*(3.0/8.0*w[1] + 6.0/8.0*w[2] + 15.0/8.0*w[3]);
    Sb[4] += obar*(-1.0/8.0*w[2] - 10.0/8.0*w[3]);
    Sb[5] += obar*(3.0/8.0*w[3]);
    const double out = w[0]*q[0] + w[1]*q[1] + w[2]*q[2] + w[3]*q[3];
    double bb[4], tau6b = 0.0, axb = 0.0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const double yb = obar*(q[k] - out)*iOs*dc[k]*P.q*py1[k];
        const double ex = ek[k]*xk[k];
        tau6b += yb*ax*ex;
        axb += yb*tau_6*ex;
        bb[k] = -yb*g[k]*(ek[k] + xk[k]);
    }
    const double s6 = sgn_(b[3] - beta_avg);
    bb[3] += tau6b*s6;
    const double bavgb = axb - tau6b*s6;
    bb[0] += bavgb/8.0;
    bb[2] += bavgb/8.0;
    bb[1] += bavgb*6.0/8.0;
    js_betas_bwd(S, bb[0], bb[1], bb[2], Sb);
    ld_beta3_bwd(S, bb[3], Sb);
}

// Forward of both sides (the operations of cu_pair<X, A>) keeping the
// indicators: b[0..3] minus side, b[4..7] plus side.
template <bool X, int A>
__device__ __forceinline__ void cu_pair_keep(const double* U, const Params& P, double& Um, double& Up, double* b) {
    js_betas_x<EMU_VJP_M>(U[0], U[1], U[2], U[3], U[4], b[0], b[1], b[2]);
    b[3] = ld_beta3<EMU_VJP_M>(U[0], U[1], U[2], U[3], U[4], U[5]);
    Um = cu_interp<X>(b, P, P.cu_e[A], P.cu_x[A], U[0], U[1], U[2], U[3], U[4], U[5]);
    js_betas_x<EMU_VJP_P>(U[5], U[4], U[3], U[2], U[1], b[4], b[5], b[6]);
    b[7] = ld_beta3<EMU_VJP_P>(U[5], U[4], U[3], U[2], U[1], U[0]);
    Up = cu_interp<X>(b + 4, P, P.cu_e[A], P.cu_x[A], U[5], U[4], U[3], U[2], U[1], U[0]);
}

template <int A>
__device__ __forceinline__ void cu_pair_bwd(const double* U, const double* b, const Params& P, double Umb,
                                            double Upb, double* Ub) {
    double Sb[6] = {0, 0, 0, 0, 0, 0};
    cu_side_bwd(P, P.cu_e[A], P.cu_x[A], U, b, Umb, Sb);
#pragma unroll
    for (int j = 0; j < 6; j++) Ub[j] += Sb[j];
    const double R[6] = {U[5], U[4], U[3], U[2], U[1], U[0]};
    double Rb[6] = {0, 0, 0, 0, 0, 0};
    cu_side_bwd(P, P.cu_e[A], P.cu_x[A], R, b + 4, Upb, Rb);
#pragma unroll
    for (int j = 0; j < 6; j++) Ub[5 - j] += Rb[j];
}

// ----------------------------------------------------------------------------
// Thermodynamics.
// ----------------------------------------------------------------------------
// Mixture gamma of a face state or a cell and the adjoint of gamma pushed to
// its inputs (five-equation: the N-1 volume fractions of V, with the last
// one 1 - sum; four-equation: the partial densities).
template <int DIM, int MODEL, int NSP>
__device__ __forceinline__ void gamma_face_bwd(const Params& P, const double* V, double gamma, double gb,
                                               double* Vb) {
    using M = Model<DIM, MODEL, NSP>;
    if constexpr (MODEL == FIVE_EQN_ALLAIRE) {
        // gamma = 1 + 1/xi, xi = sum_k Z_k/(gamma_k - 1) + (1 - sum_k Z_k)/(gamma_N - 1)
        const double xib = -gb*(gamma - 1.0)*(gamma - 1.0);
#pragma unroll
        for (int k = 0; k < NSP - 1; k++) Vb[M::IZ + k] += xib*(P.inv_gm1[k] - P.inv_gm1[NSP - 1]);
    } else if constexpr (MODEL == FOUR_EQN_CONSERVATIVE) {
        // gamma = sum V_s c_p,s / sum V_s c_v,s
        double cvm = 0.0;
#pragma unroll
        for (int s = 0; s < NSP; s++) cvm += V[s]*P.cv[s];
#pragma unroll
        for (int s = 0; s < NSP; s++) Vb[s] += gb*(P.cp[s] - gamma*P.cv[s])/cvm;
    }
}

// Adjoint of face_thermo (rho, c, eps of one reconstructed face state).
template <int DIM, int MODEL, int NSP>
__device__ __forceinline__ void face_thermo_bwd(const Params& P, const double* V, double rho, double cs, double eps,
                                                double rhob, double csb, double epsb, double* Vb) {
    using M = Model<DIM, MODEL, NSP>;
    const double p = V[M::IP];
    if constexpr (MODEL == SINGLE_SPECIES) {
        const double gamma = P.gamma[0];
        double pb = csb*gamma/(2.0*cs*rho) + epsb/((gamma - 1.0)*rho);
        double rb = rhob - csb*cs/(2.0*rho) - epsb*eps/rho;
        Vb[0] += rb;
        Vb[M::IP] += pb;
    } else {
        // c = sqrt(gamma p/rho), eps = p/((gamma - 1) rho)
        double g;
        if constexpr (MODEL == FIVE_EQN_ALLAIRE) g = gamma_last<true, NSP>(P, V + M::IZ);
        else {
            double Y[NSP], cv;
#pragma unroll
            for (int s = 0; s < NSP; s++) Y[s] = V[s]/rho;
            g = mix_mass<true, NSP>(P, Y, cv);
        }
        const double pb = csb*g/(2.0*cs*rho) + epsb/((g - 1.0)*rho);
        const double rb = rhob - csb*cs/(2.0*rho) - epsb*eps/rho;
        const double gb = csb*p/(2.0*cs*rho) - epsb*eps/(g - 1.0);
#pragma unroll
        for (int s = 0; s < NSP; s++) Vb[s] += rb;
        Vb[M::IP] += pb;
        gamma_face_bwd<DIM, MODEL, NSP>(P, V, g, gb, Vb);
    }
}

// Adjoint of face_QF (conserved state Q and physical flux F of a face state).
template <int DIM, int MODEL, int NSP, int A>
__device__ __forceinline__ void face_QF_bwd(const double* V, double rho, double eps, const double* Q,
                                            const double* Qb_in, const double* Fb, double* Vb, double& rhob,
                                            double& epsb) {
    using M = Model<DIM, MODEL, NSP>;
    constexpr int NEQ = M::NEQ;
    double Qb[NEQ];
#pragma unroll
    for (int e = 0; e < NEQ; e++) Qb[e] = Qb_in[e];
    if constexpr (MODEL == SINGLE_SPECIES) {
        const double p = V[DIM + 1];
        // F0 = Q[1+A]; F[1+k] = Q[1+A] V[1+k] (+p); FE = V[1+A] (QE + p)
        Qb[1 + A] += Fb[0];
#pragma unroll
        for (int k = 0; k < DIM; k++) {
            Qb[1 + A] += Fb[1 + k]*V[1 + k];
            Vb[1 + k] += Fb[1 + k]*Q[1 + A];
            if (k == A) Vb[DIM + 1] += Fb[1 + k];
        }
        Vb[1 + A] += Fb[DIM + 1]*(Q[DIM + 1] + p);
        Qb[DIM + 1] += Fb[DIM + 1]*V[1 + A];
        Vb[DIM + 1] += Fb[DIM + 1]*V[1 + A];
        // Q0 = V0; Q[1+k] = V0 V[1+k]; QE = V0 (eps + ke/2)
        double ke = 0.0;
#pragma unroll
        for (int k = 0; k < DIM; k++) ke += V[1 + k]*V[1 + k];
        Vb[0] += Qb[0];
#pragma unroll
        for (int k = 0; k < DIM; k++) {
            Vb[0] += Qb[1 + k]*V[1 + k];
            Vb[1 + k] += Qb[1 + k]*V[0];
            Vb[1 + k] += Qb[DIM + 1]*V[0]*V[1 + k];
        }
        Vb[0] += Qb[DIM + 1]*(eps + 0.5*ke);
        epsb += Qb[DIM + 1]*V[0];
        (void)rho;
        (void)rhob;
    } else {
        const double p = V[NSP + DIM];
        const double un = V[NSP + A];
        double unb = 0.0;
#pragma unroll
        for (int s = 0; s < NSP; s++) {
            unb += Fb[s]*V[s];
            Vb[s] += un*Fb[s];
        }
#pragma unroll
        for (int k = 0; k < DIM; k++) {
            unb += Fb[NSP + k]*Q[NSP + k];
            Qb[NSP + k] += un*Fb[NSP + k];
            if (k == A) Vb[NSP + DIM] += Fb[NSP + k];
        }
        unb += Fb[NSP + DIM]*(Q[NSP + DIM] + p);
        Qb[NSP + DIM] += un*Fb[NSP + DIM];
        Vb[NSP + DIM] += un*Fb[NSP + DIM];
#pragma unroll
        for (int s = 0; s < M::NZ; s++) {
            unb += Fb[M::IZ + s]*V[M::IZ + s];
            Vb[M::IZ + s] += un*Fb[M::IZ + s];
        }
        Vb[NSP + A] += unb;
        double ke = 0.0;
#pragma unroll
        for (int k = 0; k < DIM; k++) ke += V[NSP + k]*V[NSP + k];
#pragma unroll
        for (int s = 0; s < NSP; s++) Vb[s] += Qb[s];
#pragma unroll
        for (int k = 0; k < DIM; k++) {
            rhob += Qb[NSP + k]*V[NSP + k];
            Vb[NSP + k] += rho*Qb[NSP + k];
            Vb[NSP + k] += rho*Qb[NSP + DIM]*V[NSP + k];
        }
        rhob += Qb[NSP + DIM]*(eps + 0.5*ke);
        epsb += rho*Qb[NSP + DIM];
#pragma unroll
        for (int s = 0; s < M::NZ; s++) Vb[M::IZ + s] += Qb[M::IZ + s];
    }
}

// ----------------------------------------------------------------------------
// Riemann solver: forward (reference order) and reverse in one call.
// Fb (NEQ) and umb are the adjoints of the midpoint flux and of the HLLC
// midpoint normal velocity; VLb, VRb receive the adjoints of the two states.
// u_mid_out receives the forward midpoint velocity.
// ----------------------------------------------------------------------------
template <int DIM, int MODEL, int NSP, int A>
__device__ void riemann_bwd(const Params& P, const double* VL, const double* VR, bool use_hll, const double* Fb,
                            double umb, double* VLb, double* VRb, double& u_mid_out) {
    using M = Model<DIM, MODEL, NSP>;
    constexpr int NEQ = M::NEQ;
    constexpr int IU = M::IU;
    constexpr int IP = M::IP;
    // ---- forward
    double rhoL, cL, epsL, rhoR, cR, epsR;
    face_thermo<true, DIM, MODEL, NSP>(P, VL, rhoL, cL, epsL);
    face_thermo<true, DIM, MODEL, NSP>(P, VR, rhoR, cR, epsR);
    const double uL = VL[IU + A], uR = VR[IU + A];
    const double pL = VL[IP], pR = VR[IP];
    const double ua = mul_(double(1)/double(2), add_(uL, uR));
    const double ca = mul_(double(1)/double(2), add_(cL, cR));
    const double sLa = sub_(ua, ca), sLb = sub_(uL, cL);
    const double sRa = add_(ua, ca), sRb = add_(uR, cR);
    const bool pickLa = sLa < sLb, pickRa = sRa > sRb;
    const double s_L = fmin(sLa, sLb), s_R = fmax(sRa, sRb);
    const double num = sub_(add_(sub_(pR, pL), mul_(mul_(rhoL, uL), sub_(s_L, uL))), mul_(mul_(rhoR, uR), sub_(s_R, uR)));
    const double den = sub_(mul_(rhoL, sub_(s_L, uL)), mul_(rhoR, sub_(s_R, uR)));
    const double s_star = num/den;
    const double s_minus = fmin(0.0, s_L);
    const double s_plus = fmax(0.0, s_R);
    const bool left = s_star > 0.0;
    double VK[NEQ];
#pragma unroll
    for (int e = 0; e < NEQ; e++) VK[e] = left ? VL[e] : VR[e];
    const double rhoK = left ? rhoL : rhoR;
    const double sK = left ? s_L : s_R;
    const double uK = left ? uL : uR;
    const double pK = left ? pL : pR;
    const double s_pm = left ? s_minus : s_plus;
    double QL[NEQ], FL[NEQ], QR[NEQ], FR[NEQ];
    face_QF<true, DIM, MODEL, NSP, A>(VL, rhoL, epsL, QL, FL);
    face_QF<true, DIM, MODEL, NSP, A>(VR, rhoR, epsR, QR, FR);
    double QK[NEQ], FK[NEQ];
#pragma unroll
    for (int e = 0; e < NEQ; e++) { QK[e] = left ? QL[e] : QR[e]; FK[e] = left ? FL[e] : FR[e]; }
    const double Chi = sub_(sK, uK)/sub_(sK, s_star);
    const double rK = (MODEL == SINGLE_SPECIES) ? VK[0] : rhoK;
    const double Tt = add_(mul_(rK, s_star), pK/sub_(sK, uK));
    const double QsE = mul_(Chi, add_(QK[M::IE], mul_(sub_(s_star, uK), Tt)));
    double Qs[NEQ], Fc[NEQ];
    if constexpr (MODEL == SINGLE_SPECIES) {
        Qs[0] = mul_(Chi, VK[0]);
#pragma unroll
        for (int k = 0; k < DIM; k++) Qs[1 + k] = (k == A) ? mul_(mul_(Chi, VK[0]), s_star) : mul_(Chi, QK[1 + k]);
        Qs[DIM + 1] = QsE;
    } else {
#pragma unroll
        for (int s = 0; s < NSP; s++) Qs[s] = mul_(Chi, VK[s]);
#pragma unroll
        for (int k = 0; k < DIM; k++) Qs[NSP + k] = (k == A) ? mul_(mul_(Chi, rhoK), s_star) : mul_(Chi, QK[NSP + k]);
        Qs[NSP + DIM] = QsE;
#pragma unroll
        for (int s = 0; s < M::NZ; s++) Qs[M::IZ + s] = mul_(Chi, VK[M::IZ + s]);
    }
#pragma unroll
    for (int e = 0; e < NEQ; e++) Fc[e] = add_(FK[e], mul_(s_pm, sub_(Qs[e], QK[e])));
    u_mid_out = add_(uK, mul_(s_pm, sub_(Chi, double(1))));

    // ---- reverse
    double QLb[NEQ], FLb[NEQ], QRb[NEQ], FRb[NEQ];
#pragma unroll
    for (int e = 0; e < NEQ; e++) { QLb[e] = 0.0; FLb[e] = 0.0; QRb[e] = 0.0; FRb[e] = 0.0; }
    double s_Lb = 0.0, s_Rb = 0.0, s_starb = 0.0;
    double rhoLb = 0.0, rhoRb = 0.0, cLb = 0.0, cRb = 0.0, epsLb = 0.0, epsRb = 0.0;
    double uLb = 0.0, uRb = 0.0, pLb = 0.0, pRb = 0.0;
    double Fcb[NEQ];
#pragma unroll
    for (int e = 0; e < NEQ; e++) Fcb[e] = Fb[e];

    if (use_hll) {
        double diff[DIM];
#pragma unroll
        for (int k = 0; k < DIM; k++) diff[k] = VR[IU + k] - VL[IU + k];
        double vsq = mul_(diff[0], diff[0]);
#pragma unroll
        for (int k = 1; k < DIM; k++) vsq = add_(vsq, mul_(diff[k], diff[k]));
        const double vm = sqrt(vsq);
        double a1, a2;
        const bool small = vm < HMR_EPS;
        if (small) { a1 = 1.0; a2 = 0.0; }
        else { a1 = fabs(diff[A])/vm; a2 = sqrt(sub_(double(1), mul_(a1, a1))); }
        const double b1 = mul_(double(1)/double(2), add_(double(1), a1/add_(a1, a2)));
        const double b2 = double(1) - b1;
        double b1b = 0.0;
#pragma unroll
        for (int e = 0; e < NEQ; e++) {
            if (!hll_comp<DIM, MODEL, NSP, A>(e)) continue;
            double Fh;
            const double Dh = s_R - s_L;
            if (s_L > 0.0) Fh = FL[e];
            else if (s_R < 0.0) Fh = FR[e];
            else Fh = add_(sub_(mul_(s_R, FL[e]), mul_(s_L, FR[e])), mul_(mul_(s_R, s_L), sub_(QR[e], QL[e])))/sub_(s_R, s_L);
            Fcb[e] = b1*Fb[e];
            const double Fhb = b2*Fb[e];
            b1b += Fb[e]*(Fc[e] - Fh);
            if (s_L > 0.0) FLb[e] += Fhb;
            else if (s_R < 0.0) FRb[e] += Fhb;
            else {
                const double dQ = QR[e] - QL[e];
                FLb[e] += s_R/Dh*Fhb;
                FRb[e] -= s_L/Dh*Fhb;
                QRb[e] += s_R*s_L/Dh*Fhb;
                QLb[e] -= s_R*s_L/Dh*Fhb;
                s_Rb += Fhb*(FL[e] + s_L*dQ - Fh)/Dh;
                s_Lb += Fhb*(-FR[e] + s_R*dQ + Fh)/Dh;
            }
        }
        if (!small) {
            const double sa = a1 + a2;
            const double a1b = b1b*0.5*a2/(sa*sa);
            const double a2b = -b1b*0.5*a1/(sa*sa);
            double rp2 = 0.0;
#pragma unroll
            for (int k = 0; k < DIM; k++) if (k != A) rp2 += diff[k]*diff[k];
            const double rp = sqrt(rp2);
            const double vm3 = vm*vm*vm;
            const double adA = fabs(diff[A]);
#pragma unroll
            for (int k = 0; k < DIM; k++) {
                double db;
                if (k == A) {
                    db = a1b*(sgn_(diff[A])/vm - adA*diff[A]/vm3) + a2b*(-rp*diff[A]/vm3);
                } else {
                    db = a1b*(-adA*diff[k]/vm3) + a2b*((rp > 0.0 ? diff[k]/(rp*vm) : 0.0) - rp*diff[k]/vm3);
                }
                VRb[IU + k] += db;
                VLb[IU + k] -= db;
            }
        }
    }

    // HLLC
    double s_pmb = umb*(Chi - 1.0);
    double Chib = umb*s_pm;
    double uKb = umb;
    double QKb[NEQ], Qsb[NEQ];
#pragma unroll
    for (int e = 0; e < NEQ; e++) {
        s_pmb += Fcb[e]*(Qs[e] - QK[e]);
        Qsb[e] = s_pm*Fcb[e];
        QKb[e] = -s_pm*Fcb[e];
    }
    double VKb[NEQ];
#pragma unroll
    for (int e = 0; e < NEQ; e++) {
        VKb[e] = 0.0;
        if (left) FLb[e] += Fcb[e];
        else FRb[e] += Fcb[e];
    }
    double rKb = 0.0, sKb = 0.0, pKb = 0.0;
    if constexpr (MODEL == SINGLE_SPECIES) {
        Chib += Qsb[0]*VK[0];
        VKb[0] += Chi*Qsb[0];
#pragma unroll
        for (int k = 0; k < DIM; k++) {
            if (k == A) {
                Chib += Qsb[1 + k]*VK[0]*s_star;
                VKb[0] += Chi*Qsb[1 + k]*s_star;
                s_starb += Chi*VK[0]*Qsb[1 + k];
            } else {
                Chib += Qsb[1 + k]*QK[1 + k];
                QKb[1 + k] += Chi*Qsb[1 + k];
            }
        }
    } else {
#pragma unroll
        for (int s = 0; s < NSP; s++) {
            Chib += Qsb[s]*VK[s];
            VKb[s] += Chi*Qsb[s];
        }
#pragma unroll
        for (int k = 0; k < DIM; k++) {
            if (k == A) {
                Chib += Qsb[NSP + k]*rhoK*s_star;
                rKb += Chi*Qsb[NSP + k]*s_star;
                s_starb += Chi*rhoK*Qsb[NSP + k];
            } else {
                Chib += Qsb[NSP + k]*QK[NSP + k];
                QKb[NSP + k] += Chi*Qsb[NSP + k];
            }
        }
#pragma unroll
        for (int s = 0; s < M::NZ; s++) {
            Chib += Qsb[M::IZ + s]*VK[M::IZ + s];
            VKb[M::IZ + s] += Chi*Qsb[M::IZ + s];
        }
    }
    {
        // QsE = Chi (QK[IE] + (s* - uK) T), T = rK s* + pK/(sK - uK)
        const double QsEb = Qsb[M::IE];
        const double w = sK - uK;
        Chib += QsEb*(QK[M::IE] + (s_star - uK)*Tt);
        QKb[M::IE] += Chi*QsEb;
        const double Tb = Chi*QsEb*(s_star - uK);
        s_starb += Chi*QsEb*Tt;
        uKb -= Chi*QsEb*Tt;
        if constexpr (MODEL == SINGLE_SPECIES) VKb[0] += Tb*s_star;
        else rKb += Tb*s_star;
        s_starb += Tb*rK;
        pKb += Tb/w;
        sKb -= Tb*pK/(w*w);
        uKb += Tb*pK/(w*w);
    }
    {
        // Chi = (sK - uK)/(sK - s*)
        const double Dc = sK - s_star, Nc = sK - uK;
        sKb += Chib*(1.0/Dc - Nc/(Dc*Dc));
        uKb -= Chib/Dc;
        s_starb += Chib*Nc/(Dc*Dc);
    }
    if (left) { if (!(0.0 < s_L)) s_Lb += s_pmb; }
    else { if (!(0.0 > s_R)) s_Rb += s_pmb; }
    if (left) { s_Lb += sKb; uLb += uKb; pLb += pKb; rhoLb += rKb; }
    else { s_Rb += sKb; uRb += uKb; pRb += pKb; rhoRb += rKb; }
#pragma unroll
    for (int e = 0; e < NEQ; e++) {
        if (left) { QLb[e] += QKb[e]; VLb[e] += VKb[e]; }
        else { QRb[e] += QKb[e]; VRb[e] += VKb[e]; }
    }
    // conserved states and physical fluxes of both sides
    face_QF_bwd<DIM, MODEL, NSP, A>(VL, rhoL, epsL, QL, QLb, FLb, VLb, rhoLb, epsLb);
    face_QF_bwd<DIM, MODEL, NSP, A>(VR, rhoR, epsR, QR, QRb, FRb, VRb, rhoRb, epsRb);
    {
        // s* = num/den
        const double numb = s_starb/den;
        const double denb = -s_starb*s_star/den;
        pRb += numb;
        pLb -= numb;
        rhoLb += numb*uL*(s_L - uL);
        uLb += numb*rhoL*(s_L - 2.0*uL);
        s_Lb += numb*rhoL*uL;
        rhoRb -= numb*uR*(s_R - uR);
        uRb -= numb*rhoR*(s_R - 2.0*uR);
        s_Rb -= numb*rhoR*uR;
        rhoLb += denb*(s_L - uL);
        s_Lb += denb*rhoL;
        uLb -= denb*rhoL;
        rhoRb -= denb*(s_R - uR);
        s_Rb -= denb*rhoR;
        uRb += denb*rhoR;
    }
    double uab = 0.0, cab = 0.0;
    if (pickLa) { uab += s_Lb; cab -= s_Lb; } else { uLb += s_Lb; cLb -= s_Lb; }
    if (pickRa) { uab += s_Rb; cab += s_Rb; } else { uRb += s_Rb; cRb += s_Rb; }
    uLb += 0.5*uab; uRb += 0.5*uab;
    cLb += 0.5*cab; cRb += 0.5*cab;
    VLb[IU + A] += uLb; VRb[IU + A] += uRb;
    VLb[IP] += pLb; VRb[IP] += pRb;
    if constexpr (MODEL == SINGLE_SPECIES) {
        // rho of a single-species face state is V[0]
        VLb[0] += rhoLb;
        VRb[0] += rhoRb;
        face_thermo_bwd<DIM, MODEL, NSP>(P, VL, rhoL, cL, epsL, 0.0, cLb, epsLb, VLb);
        face_thermo_bwd<DIM, MODEL, NSP>(P, VR, rhoR, cR, epsR, 0.0, cRb, epsRb, VRb);
    } else {
        face_thermo_bwd<DIM, MODEL, NSP>(P, VL, rhoL, cL, epsL, rhoLb, cLb, epsLb, VLb);
        face_thermo_bwd<DIM, MODEL, NSP>(P, VR, rhoR, cR, epsR, rhoRb, cRb, epsRb, VRb);
    }
}

// ----------------------------------------------------------------------------
// Characteristic projection.
// ----------------------------------------------------------------------------
// Adjoints of the per-face factors of FaceProj.
template <int NSP>
struct FaceProjBar {
    double p_hrc, ic2, irc;
    double zr[NSP], hz[NSP];
};

// One characteristic component e of char_from_prim (same operations).
template <int DIM, int MODEL, int NSP, int A>
__device__ __forceinline__ double char_one(const FaceProj<DIM, MODEL, NSP>& F, const double* V, int e) {
    using M = Model<DIM, MODEL, NSP>;
    if constexpr (MODEL == SINGLE_SPECIES) {
        const double un = V[1 + A];
        const double p = V[DIM + 1];
        if (e == 0) return add_(mul_(F.m_hrc, un), mul_(double(1)/double(2), p));
        if (e == 1) return sub_(V[0], mul_(F.ic2, p));
        if (e == DIM + 1) return add_(mul_(F.p_hrc, un), mul_(double(1)/double(2), p));
        int t = 2;
#pragma unroll
        for (int k = 0; k < DIM; k++) {
            if (k == A) continue;
            if (t == e) return V[1 + k];
            t++;
        }
        return 0.0;
    } else {
        const double un = V[NSP + A];
        const double p = V[NSP + DIM];
        if (e == 0) return sub_(un, mul_(F.irc, p));
        if (e == M::NEQ - 1) return add_(un, mul_(F.irc, p));
#pragma unroll
        for (int s = 0; s < NSP; s++)
            if (e == 1 + s) return sub_(V[s], mul_(F.zr[s], p));
#pragma unroll
        for (int s = 0; s < M::NZ; s++)
            if (e == NSP + DIM + s) return V[M::IZ + s];
        int t = NSP + 1;
#pragma unroll
        for (int k = 0; k < DIM; k++) {
            if (k == A) continue;
            if (t == e) return V[NSP + k];
            t++;
        }
        return 0.0;
    }
}

// Adjoint of component e of char_from_prim at one cell.
template <int DIM, int MODEL, int NSP, int A>
__device__ __forceinline__ void char_one_bwd(const FaceProj<DIM, MODEL, NSP>& F, const double* V, int e, double Wb,
                                             double* Vb, FaceProjBar<NSP>& Fb) {
    using M = Model<DIM, MODEL, NSP>;
    if constexpr (MODEL == SINGLE_SPECIES) {
        const double un = V[1 + A];
        const double p = V[DIM + 1];
        if (e == 0) { Vb[1 + A] -= F.p_hrc*Wb; Vb[DIM + 1] += 0.5*Wb; Fb.p_hrc -= Wb*un; return; }
        if (e == 1) { Vb[0] += Wb; Vb[DIM + 1] -= F.ic2*Wb; Fb.ic2 -= Wb*p; return; }
        if (e == DIM + 1) { Vb[1 + A] += F.p_hrc*Wb; Vb[DIM + 1] += 0.5*Wb; Fb.p_hrc += Wb*un; return; }
        int t = 2;
#pragma unroll
        for (int k = 0; k < DIM; k++) {
            if (k == A) continue;
            if (t == e) Vb[1 + k] += Wb;
            t++;
        }
    } else {
        const double p = V[NSP + DIM];
        if (e == 0) { Vb[NSP + A] += Wb; Vb[NSP + DIM] -= F.irc*Wb; Fb.irc -= Wb*p; return; }
        if (e == M::NEQ - 1) { Vb[NSP + A] += Wb; Vb[NSP + DIM] += F.irc*Wb; Fb.irc += Wb*p; return; }
#pragma unroll
        for (int s = 0; s < NSP; s++) {
            if (e == 1 + s) {
                Vb[s] += Wb;
                Vb[NSP + DIM] -= F.zr[s]*Wb;
                Fb.zr[s] -= Wb*p;
                return;
            }
        }
#pragma unroll
        for (int s = 0; s < M::NZ; s++) {
            if (e == NSP + DIM + s) { Vb[M::IZ + s] += Wb; return; }
        }
        int t = NSP + 1;
#pragma unroll
        for (int k = 0; k < DIM; k++) {
            if (k == A) continue;
            if (t == e) Vb[NSP + k] += Wb;
            t++;
        }
    }
}

// Adjoint of prim_from_char: Vb -> Wb (accumulated), factor adjoints.
template <int DIM, int MODEL, int NSP, int A>
__device__ __forceinline__ void prim_from_char_bwd(const FaceProj<DIM, MODEL, NSP>& F, const double* W,
                                                   const double* Vb, double* Wb, FaceProjBar<NSP>& Fb) {
    using M = Model<DIM, MODEL, NSP>;
    constexpr int L = M::NEQ - 1;
    if constexpr (MODEL == SINGLE_SPECIES) {
        Wb[0] += F.ic2*Vb[0]; Wb[L] += F.ic2*Vb[0]; Wb[1] += Vb[0];
        Fb.ic2 += Vb[0]*(W[0] + W[L]);
        Wb[0] -= F.irc*Vb[1 + A]; Wb[L] += F.irc*Vb[1 + A];
        Fb.irc += Vb[1 + A]*(W[L] - W[0]);
        Wb[0] += Vb[DIM + 1]; Wb[L] += Vb[DIM + 1];
        int t = 2;
#pragma unroll
        for (int k = 0; k < DIM; k++) if (k != A) Wb[t++] += Vb[1 + k];
    } else {
#pragma unroll
        for (int s = 0; s < NSP; s++) {
            Wb[s + 1] += Vb[s];
            Wb[L] += F.hz[s]*Vb[s];
            Wb[0] -= F.hz[s]*Vb[s];
            Fb.hz[s] += Vb[s]*(W[L] - W[0]);
        }
#pragma unroll
        for (int s = 0; s < M::NZ; s++) Wb[NSP + DIM + s] += Vb[M::IZ + s];
        int t = NSP + 1;
#pragma unroll
        for (int k = 0; k < DIM; k++) {
            if (k == A) { Wb[0] += 0.5*Vb[NSP + k]; Wb[L] += 0.5*Vb[NSP + k]; }
            else Wb[t++] += Vb[NSP + k];
        }
        Fb.p_hrc += Vb[NSP + DIM]*(W[L] - W[0]);
        Wb[L] += F.p_hrc*Vb[NSP + DIM];
        Wb[0] -= F.p_hrc*Vb[NSP + DIM];
    }
}

// Factor adjoints -> adjoints of the projection means rb, cb, zb.
template <int DIM, int MODEL, int NSP>
__device__ __forceinline__ void face_proj_bwd(const FaceProj<DIM, MODEL, NSP>& F, const FaceProjBar<NSP>& Fb,
                                              double& rbb, double& cbb, double* zbb) {
    rbb += 0.5*F.cb*Fb.p_hrc;
    cbb += 0.5*F.rb*Fb.p_hrc;
    cbb -= 2.0*F.ic2/F.cb*Fb.ic2;
    rbb -= F.irc/F.rb*Fb.irc;
    cbb -= F.irc/F.cb*Fb.irc;
    if constexpr (MODEL != SINGLE_SPECIES) {
        const double rcc = F.rb*F.cb*F.cb;
#pragma unroll
        for (int s = 0; s < NSP; s++) {
            zbb[s] += Fb.zr[s]/rcc;
            rbb -= Fb.zr[s]*F.zr[s]/F.rb;
            cbb -= 2.0*Fb.zr[s]*F.zr[s]/F.cb;
            zbb[s] += 0.5*Fb.hz[s]/F.cb;
            cbb -= Fb.hz[s]*F.hz[s]/F.cb;
        }
    }
}

// ----------------------------------------------------------------------------
// Cell data: adjoint of cell_derived (V, rho, cs from the conserved variables).
// Qb (NCOMP) is accumulated.
// ----------------------------------------------------------------------------
template <int DIM, int MODEL, int NSP>
__device__ __forceinline__ void cell_derived_bwd(const Params& P, const double* Q, const double* Vb, double rhob,
                                                 double csb, double* Qb) {
    using M = Model<DIM, MODEL, NSP>;
    double V[M::NEQ], rho, cs;
    cell_derived<DIM, MODEL, NSP>(P, Q, V, rho, cs);
    const double p = V[M::IP];
    double u[DIM], ke = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; k++) { u[k] = V[M::IU + k]; ke += u[k]*u[k]; }
    double gamma;
    if constexpr (MODEL == SINGLE_SPECIES) gamma = P.gamma[0];
    else gamma = cs*cs*rho/p;
    if constexpr (MODEL == FIVE_EQN_ALLAIRE) {
        double Z[NSP];
#pragma unroll
        for (int s = 0; s < NSP; s++) Z[s] = Q[M::IZ + s];
        gamma = gamma_all_x<NSP>(P, Z);
    } else if constexpr (MODEL == FOUR_EQN_CONSERVATIVE) {
        double Y[NSP], cv;
#pragma unroll
        for (int s = 0; s < NSP; s++) Y[s] = Q[s]/rho;
        gamma = mix_mass<true, NSP>(P, Y, cv);
    }
    // cs = sqrt(gamma p/rho)
    double pb = Vb[M::IP] + csb*gamma/(2.0*cs*rho);
    double rb = rhob - csb*cs/(2.0*rho);
    double gb = csb*p/(2.0*cs*rho);
    // p = (gamma - 1)(E - 1/2 sum m^2/rho)
    const double eps = p/((gamma - 1.0)*rho);
    double Eb = (gamma - 1.0)*pb;
    double mb[DIM];
#pragma unroll
    for (int k = 0; k < DIM; k++) mb[k] = -(gamma - 1.0)*pb*u[k];
    rb += (gamma - 1.0)*pb*0.5*ke;
    gb += pb*rho*eps;
    // u = m/rho
#pragma unroll
    for (int k = 0; k < DIM; k++) {
        mb[k] += Vb[M::IU + k]/rho;
        rb -= Vb[M::IU + k]*u[k]/rho;
    }
    if constexpr (MODEL == SINGLE_SPECIES) {
        Qb[0] += rb + Vb[0];
#pragma unroll
        for (int k = 0; k < DIM; k++) Qb[1 + k] += mb[k];
        Qb[DIM + 1] += Eb;
    } else {
#pragma unroll
        for (int s = 0; s < NSP; s++) Qb[s] += rb + Vb[s];
#pragma unroll
        for (int k = 0; k < DIM; k++) Qb[NSP + k] += mb[k];
        Qb[NSP + DIM] += Eb;
        if constexpr (MODEL == FIVE_EQN_ALLAIRE) {
            // gamma = 1 + 1/xi, xi = sum over all N stored volume fractions
            const double xib = -gb*(gamma - 1.0)*(gamma - 1.0);
#pragma unroll
            for (int s = 0; s < NSP; s++) Qb[M::IZ + s] += xib*P.inv_gm1[s];
#pragma unroll
            for (int s = 0; s < NSP - 1; s++) Qb[M::IZ + s] += Vb[M::IZ + s];
        } else {
            double cvm = 0.0;
#pragma unroll
            for (int s = 0; s < NSP; s++) cvm += Q[s]*P.cv[s];
#pragma unroll
            for (int s = 0; s < NSP; s++) Qb[s] += gb*(P.cp[s] - gamma*P.cv[s])/cvm;
        }
    }
}

}  // namespace hmr
