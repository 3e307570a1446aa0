// Device physics of the WCNS56 / HLLC-HLL convective path (FP64).
//
// Model and scheme are template parameters so every variant compiles to
// straight-line register code.  HMR_FAST selects the arithmetic form:
//   HMR_FAST == 0 : the reference's operation order, built with --fmad=false;
//                   results are bitwise equal to the CPU oracle.
//   HMR_FAST == 1 : algebraically regrouped (shared reciprocals, single
//                   normalisations) and FMA-contracted; agrees with the
//                   reference to rounding (<= 1e-12 relative).
// Formulas and the reference lines they follow:
//   WCNS5-JS  src/flow/convective_flux_reconstructors/WCNS56/ConvectiveFluxReconstructorWCNS5-JS-HLLC-HLL.cpp:24-164
//   WCNS6-LD  src/flow/convective_flux_reconstructors/WCNS56/ConvectiveFluxReconstructorWCNS6-LD-HLLC-HLL.cpp:24-319
//   WCNS5-Z   src/flow/convective_flux_reconstructors/WCNS56/ConvectiveFluxReconstructorWCNS5-Z-HLLC-HLL.cpp:78-168
//   WCNS6-CU-M2 src/flow/convective_flux_reconstructors/WCNS56/ConvectiveFluxReconstructorWCNS6-CU-M2-HLLC-HLL.cpp:112-228
//   projection / characteristic transforms / bounds
//             src/flow/flow_models/single-species/FlowModelBasicUtilitiesSingleSpecies.cpp:3013,4638,5882,7023
//             src/flow/flow_models/five-eqn_Allaire/FlowModelBasicUtilitiesFiveEqnAllaire.cpp:5446,7474,8232,9201
//   HLLC, HLLC-HLL
//             src/flow/flow_models/single-species/Riemann_solvers/FlowModelRiemannSolverSingleSpeciesHLLC-HLL.cpp:889-1027
//             src/flow/flow_models/five-eqn_Allaire/Riemann_solvers/FlowModelRiemannSolverFiveEqnAllaireHLLC-HLL.cpp:1283-1503
//             src/flow/flow_models/four-eqn_conservative/Riemann_solvers/FlowModelRiemannSolverFourEqnConservativeHLLC-HLL.cpp:1073-1245
//   ideal-gas EOS and volume-/mass-fraction mixing rules
//             src/util/mixing_rules/equations_of_state/ideal_gas/EquationOfStateIdealGas.cpp:29-43,561-575,1093-1107
//             src/util/mixing_rules/equations_of_state/ideal_gas/EquationOfStateMixingRulesIdealGas.cpp:107-120,6367-6420,6946-7150,7404-7800
#pragma once

#ifndef HMR_FAST
#define HMR_FAST 1
#endif

#define HMR_EPS 1.0e-15  // HAMERS_EPSILON

#include "hmr_emu64.cuh"

namespace hmr {

enum { SINGLE_SPECIES = 0, FOUR_EQN_CONSERVATIVE = 1, FIVE_EQN_ALLAIRE = 2 };
enum { WCNS5_JS = 0, WCNS6_LD = 1, WCNS5_Z = 2, WCNS6_CU_M2 = 3 };

constexpr int MAX_SPECIES = 4;
constexpr int MAX_COMP = 12;

// Scheme and species constants shared by every kernel of a context.
struct Params {
    double gamma[MAX_SPECIES];         // species_gamma
    double inv_gm1[MAX_SPECIES];       // 1/(gamma_i - 1)
    double cp[MAX_SPECIES];            // species c_p = gamma_i/(gamma_i - 1)*R_i (four-equation model)
    double cv[MAX_SPECIES];            // species c_v = 1/(gamma_i - 1)*R_i
    int p, q;                          // WCNS constants
    double C, alpha_tau;
    double cu_e[3];                    // WCNS6-CU-M2 epsilon*dx*dx per axis (dx: the grid geometry's spacing)
    double cu_x[3];                    // WCNS6-CU-M2 Chi*dx*dx per axis
    // Navier-Stokes (single species): side values of 4/3 mu + mu_v, 2/3 mu - mu_v, mu, kappa
    // (constant cell values interpolated to the midpoints), and (gamma - 1) c_v for T.
    int dorder;                        // 0 Euler; 2, 4 midpoint diffusive flux of that order
    double dS43, dS23, dmu, dkappa, dTc;
    double cmu, cmu_v, ckappa;         // the cell values of mu, mu_v, kappa (stable time step)
};

template <int DIM, int MODEL, int NSP>
struct Model {
    static constexpr int NEQ = MODEL == SINGLE_SPECIES ? DIM + 2
                             : (MODEL == FIVE_EQN_ALLAIRE ? DIM + 2 * NSP : NSP + DIM + 1);
    static constexpr int NCOMP = NEQ + (MODEL == FIVE_EQN_ALLAIRE ? 1 : 0);
    static constexpr int IU = MODEL == SINGLE_SPECIES ? 1 : NSP;            // first velocity in V
    static constexpr int IP = MODEL == SINGLE_SPECIES ? DIM + 1 : NSP + DIM; // pressure in V
    static constexpr int IZ = NSP + DIM + 1;                                  // first volume fraction in V (five)
    static constexpr int NZ = MODEL == FIVE_EQN_ALLAIRE ? NSP - 1 : 0;       // volume fractions in the equations
    static constexpr int NPROJ = MODEL == SINGLE_SPECIES ? 2 : NSP + 2;
    static constexpr int IE = MODEL == SINGLE_SPECIES ? DIM + 1 : NSP + DIM; // total energy in Q
};

__device__ __forceinline__ double ipow_d(double b, int e) {
    double r = b;
    for (int i = 1; i < e; i++) r *= b;
    return r;
}

// ----------------------------------------------------------------------------
// Cell derived data: primitive variables V, density, sound speed.
// single: FlowModelSingleSpecies.cpp:2649-3180; five: FlowModelFiveEqnAllaire.cpp:3734-4877.
// Always evaluated in the reference's operation order with explicitly
// rounded products (never contracted into FMAs), in both arithmetic forms:
// the shock sensor is built from these values, and identical inputs keep
// its HLLC / HLLC-HLL choice identical between the exact and fast forms.
// ----------------------------------------------------------------------------
__device__ __forceinline__ double mul_(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add_(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub_(double a, double b) { return __dsub_rn(a, b); }

// The same explicitly rounded operations on the native FP64 pipe or emulated on the integer
// pipes (hmr_emu64.cuh): identical result bits, different hardware.  E is a mask: bit 0
// emulates the multiplications, bit 1 the additions and subtractions.  An emulated
// multiplication costs about 24 ALU and 20 IMAD warp instructions, less pipe time than the 64
// cycles a native one holds the FP64 pipe; an emulated addition costs about 49 ALU
// instructions, more.  The smoothness indicators -- about half of a face's FP64 operations --
// take E per side from HMR_EMU_BETA (bits 0-1 the minus side, bits 2-3 the plus side), so that
// the integer pipes carry part of the work the narrow FP64 pipe would otherwise serialise.
template <int E>
__device__ __forceinline__ double mulx(double a, double b) {
    if constexpr ((E & 1) != 0) return emu_dmul(a, b);
    else return __dmul_rn(a, b);
}
template <int E>
__device__ __forceinline__ double addx(double a, double b) {
    if constexpr ((E & 2) != 0) return emu_dadd(a, b);
    else return __dadd_rn(a, b);
}
template <int E>
__device__ __forceinline__ double subx(double a, double b) {
    if constexpr ((E & 2) != 0) return emu_dsub(a, b);
    else return __dsub_rn(a, b);
}

#ifndef HMR_EMU_BETA
#define HMR_EMU_BETA 0
#endif
constexpr int EMU_BETA_M = HMR_EMU_BETA & 3;         // minus-side indicators
constexpr int EMU_BETA_P = (HMR_EMU_BETA >> 2) & 3;  // plus-side indicators

template <int NSP>
__device__ __forceinline__ double gamma_all_x(const Params& P, const double* Z) {
    double xi = 0.0;
#pragma unroll
    for (int s = 0; s < NSP; s++) xi = add_(xi, mul_(Z[s], P.inv_gm1[s]));
    return add_(double(1)/xi, double(1));
}

// Four-equation model: mass-fraction mixture c_p, c_v and gamma = c_p/c_v
// (EquationOfStateMixingRulesIdealGas.cpp:6946-7150).
template <bool X, int NSP>
__device__ __forceinline__ double mix_mass(const Params& P, const double* Y, double& cv) {
    double cp = 0.0;
    cv = 0.0;
#pragma unroll
    for (int s = 0; s < NSP; s++) {
        cp = X ? add_(cp, mul_(Y[s], P.cp[s])) : cp + Y[s]*P.cp[s];
        cv = X ? add_(cv, mul_(Y[s], P.cv[s])) : cv + Y[s]*P.cv[s];
    }
    return cp/cv;
}

// Four-equation model, reference order: squared sound speed
// Gamma p/rho + sum Y_i Psi_i with Psi_i = ((c_p,i - gamma c_v,i)/c_v + gamma - 1) eps
// and eps = p/((gamma - 1) rho) (EquationOfStateMixingRulesIdealGas.cpp:6367-6420,
// FlowModelFourEqnConservative.cpp:5087-5445).  Returns c^2; eps is the
// internal energy from (rho, p, Y) (EquationOfStateIdealGas.cpp:6291).
template <int NSP>
__device__ __forceinline__ double four_c2_x(const Params& P, double rho, double p, const double* Y, double& eps) {
    double cv;
    const double gamma = mix_mass<true, NSP>(P, Y, cv);
    const double Gamma = sub_(gamma, double(1));
    eps = p/mul_(sub_(gamma, double(1)), rho);
    double c2 = mul_(Gamma, p)/rho;
#pragma unroll
    for (int s = 0; s < NSP; s++) {
        const double Psi = mul_(sub_(add_(sub_(P.cp[s], mul_(gamma, P.cv[s]))/cv, gamma), double(1)), eps);
        c2 = add_(c2, mul_(Y[s], Psi));
    }
    return c2;
}

template <int DIM, int MODEL, int NSP>
__device__ __forceinline__ void cell_derived(const Params& P, const double* Q, double* V,
                                             double& rho, double& cs) {
    using M = Model<DIM, MODEL, NSP>;
    if constexpr (MODEL == SINGLE_SPECIES) {
        const double gamma = P.gamma[0];
        rho = Q[0];
        double u[DIM];
#pragma unroll
        for (int k = 0; k < DIM; k++) u[k] = Q[1 + k]/rho;
        double ke = mul_(u[0], u[0]);
#pragma unroll
        for (int k = 1; k < DIM; k++) ke = add_(ke, mul_(u[k], u[k]));
        const double eps = sub_(Q[DIM + 1]/rho, mul_(double(1)/double(2), ke));
        const double p = mul_(mul_(sub_(gamma, double(1)), rho), eps);
        cs = sqrt(mul_(gamma, p)/rho);
        V[0] = rho;
#pragma unroll
        for (int k = 0; k < DIM; k++) V[1 + k] = u[k];
        V[DIM + 1] = p;
    } else if constexpr (MODEL == FOUR_EQN_CONSERVATIVE) {
        // FlowModelFourEqnConservative.cpp:3877-5445
        double r = 0.0;
#pragma unroll
        for (int s = 0; s < NSP; s++) r = add_(r, Q[s]);
        rho = r;
        double Y[NSP];
        double u[DIM];
#pragma unroll
        for (int s = 0; s < NSP; s++) Y[s] = Q[s]/r;
#pragma unroll
        for (int k = 0; k < DIM; k++) u[k] = Q[NSP + k]/r;
        double ke = mul_(u[0], u[0]);
#pragma unroll
        for (int k = 1; k < DIM; k++) ke = add_(ke, mul_(u[k], u[k]));
        double cv;
        const double gamma = mix_mass<true, NSP>(P, Y, cv);
        const double eps = sub_(Q[NSP + DIM]/r, mul_(double(1)/double(2), ke));
        const double p = mul_(mul_(sub_(gamma, double(1)), r), eps);
        double eps_p;
        cs = sqrt(four_c2_x<NSP>(P, r, p, Y, eps_p));
#pragma unroll
        for (int s = 0; s < NSP; s++) V[s] = Q[s];
#pragma unroll
        for (int k = 0; k < DIM; k++) V[NSP + k] = u[k];
        V[NSP + DIM] = p;
    } else {
        double r = 0.0;
#pragma unroll
        for (int s = 0; s < NSP; s++) r = add_(r, Q[s]);
        rho = r;
        double Y[NSP];
        double u[DIM];
#pragma unroll
        for (int s = 0; s < NSP; s++) Y[s] = Q[s]/r;
#pragma unroll
        for (int k = 0; k < DIM; k++) u[k] = Q[NSP + k]/r;
        double ke = mul_(u[0], u[0]);
#pragma unroll
        for (int k = 1; k < DIM; k++) ke = add_(ke, mul_(u[k], u[k]));
        double Z[NSP];
#pragma unroll
        for (int s = 0; s < NSP; s++) Z[s] = Q[M::IZ + s];
        const double gamma = gamma_all_x<NSP>(P, Z);
        const double eps = sub_(Q[NSP + DIM]/r, mul_(double(1)/double(2), ke));
        const double p = mul_(mul_(sub_(gamma, double(1)), r), eps);
        const double Gamma = sub_(gamma, double(1));
        const double Psi = p/r;
        double c2 = mul_(Gamma, p)/r;
#pragma unroll
        for (int s = 0; s < NSP; s++) c2 = add_(c2, mul_(Y[s], Psi));
        cs = sqrt(c2);
#pragma unroll
        for (int s = 0; s < NSP; s++) V[s] = Q[s];
#pragma unroll
        for (int k = 0; k < DIM; k++) V[NSP + k] = u[k];
        V[NSP + DIM] = p;
#pragma unroll
        for (int s = 0; s < NSP - 1; s++) V[M::IZ + s] = Z[s];
    }
}

// ----------------------------------------------------------------------------
// Characteristic projection at a face normal to A.
//
// Everything from the cell primitives to the smoothness indicators is
// evaluated in the reference's operation order with explicitly rounded
// products, in both arithmetic forms.  Smoothness indicators cancel heavily
// on smooth data and the eps-regularised weights amplify their rounding near
// discontinuities, so the reference's own rounding in W and beta is part of
// its result at the 1e-12 level; reproducing it bit for bit keeps the fast
// form within tolerance and keeps every discrete decision (the WCNS6-LD
// tau-switch) identical.  The per-face factors below are the reference's
// subexpressions, computed once per face instead of once per offset (same
// bits).
// ----------------------------------------------------------------------------
template <int DIM, int MODEL, int NSP>
struct FaceProj {
    double rb, cb;          // projection means
    double zb[NSP];         // partial-density means (five-equation model)
    double m_hrc, p_hrc;    // (-1/2*rb)*cb, (1/2*rb)*cb
    double ic2;             // 1/(cb*cb)
    double irc;             // 1/(rb*cb)
    double zr[NSP];         // zb/((rb*cb)*cb)
    double hz[NSP];         // (1/2*zb)/cb
};

template <int DIM, int MODEL, int NSP>
__device__ __forceinline__ void face_proj_setup(FaceProj<DIM, MODEL, NSP>& F) {
    F.m_hrc = mul_(mul_(-double(1)/double(2), F.rb), F.cb);
    F.p_hrc = mul_(mul_(double(1)/double(2), F.rb), F.cb);
    F.ic2 = double(1)/mul_(F.cb, F.cb);
    F.irc = double(1)/mul_(F.rb, F.cb);
    if constexpr (MODEL != SINGLE_SPECIES) {
        const double rcc = mul_(mul_(F.rb, F.cb), F.cb);
#pragma unroll
        for (int s = 0; s < NSP; s++) {
            F.zr[s] = F.zb[s]/rcc;
            F.hz[s] = mul_(double(1)/double(2), F.zb[s])/F.cb;
        }
    }
}

// single: FlowModelBasicUtilitiesSingleSpecies.cpp:6135-6246 (2D), 3D block after it;
// five:   FlowModelBasicUtilitiesFiveEqnAllaire.cpp:8540-8760 (2D), 3D block after it.
template <int DIM, int MODEL, int NSP, int A>
__device__ __forceinline__ void char_from_prim(const FaceProj<DIM, MODEL, NSP>& F, const double* V, double* W) {
    using M = Model<DIM, MODEL, NSP>;
    if constexpr (MODEL == SINGLE_SPECIES) {
        const double un = V[1 + A];
        const double p = V[DIM + 1];
        const double hp = mul_(double(1)/double(2), p);
        W[0] = add_(mul_(F.m_hrc, un), hp);
        W[1] = sub_(V[0], mul_(F.ic2, p));
        W[DIM + 1] = add_(mul_(F.p_hrc, un), hp);
        int t = 2;
#pragma unroll
        for (int k = 0; k < DIM; k++) if (k != A) W[t++] = V[1 + k];
    } else {
        const double un = V[NSP + A];
        const double p = V[NSP + DIM];
#pragma unroll
        for (int s = 0; s < NSP; s++) W[1 + s] = sub_(V[s], mul_(F.zr[s], p));
#pragma unroll
        for (int s = 0; s < M::NZ; s++) W[NSP + DIM + s] = V[M::IZ + s];
        W[0] = sub_(un, mul_(F.irc, p));
        W[M::NEQ - 1] = add_(un, mul_(F.irc, p));
        int t = NSP + 1;
#pragma unroll
        for (int k = 0; k < DIM; k++) if (k != A) W[t++] = V[NSP + k];
    }
}

// ----------------------------------------------------------------------------
// From here on every routine has two forms selected by the template flag X:
//   X = true : the reference's operation order with every product explicitly
//              rounded (__dmul_rn / __dadd_rn / __dsub_rn, never contracted),
//              bitwise equal to the reference in either translation unit;
//   X = false: regrouped for fewer FP64 instructions (shared reciprocals,
//              one normalisation per weight set, FMA contraction).
// The fast kernels run X = false and recompute a face with X = true where the
// reference's own result is ill-conditioned (see face_item).
// ----------------------------------------------------------------------------
template <bool X>
__device__ __forceinline__ double ipow_(double b, int e) {
    if constexpr (!X) {   // the reconstructors' default exponents, by squaring
        if (e == 2) return b*b;
        if (e == 4) {
            const double b2 = b*b;
            return b2*b2;
        }
    }
    double r = b;
    for (int i = 1; i < e; i++) r = X ? mul_(r, b) : r*b;
    return r;
}

// Mixture gamma from N-1 volume fractions (side data of the Riemann drivers),
// EquationOfStateMixingRulesIdealGas.cpp:7599-7800.
template <bool X, int NSP>
__device__ __forceinline__ double gamma_last(const Params& P, const double* Z) {
    double xi = 0.0;
    double Zl = 1.0;
#pragma unroll
    for (int s = 0; s < NSP - 1; s++) {
        xi = X ? add_(xi, mul_(Z[s], P.inv_gm1[s])) : xi + Z[s]*P.inv_gm1[s];
        Zl = X ? sub_(Zl, Z[s]) : Zl - Z[s];
    }
    xi = X ? add_(xi, Zl/sub_(P.gamma[NSP - 1], double(1))) : xi + Zl*P.inv_gm1[NSP - 1];
    return X ? add_(double(1)/xi, double(1)) : double(1)/xi + double(1);
}

// single: FlowModelBasicUtilitiesSingleSpecies.cpp:7279-7330 (2D) and the 3D block;
// five:   FlowModelBasicUtilitiesFiveEqnAllaire.cpp:9201-... (2D block).
template <bool X, int DIM, int MODEL, int NSP, int A>
__device__ __forceinline__ void prim_from_char(const FaceProj<DIM, MODEL, NSP>& F, const double* W, double* V) {
    using M = Model<DIM, MODEL, NSP>;
    constexpr int L = M::NEQ - 1;
    if constexpr (MODEL == SINGLE_SPECIES) {
        if constexpr (X) {
            V[0] = add_(add_(mul_(F.ic2, W[0]), W[1]), mul_(F.ic2, W[L]));
            V[1 + A] = add_(mul_(-F.irc, W[0]), mul_(F.irc, W[L]));
            V[DIM + 1] = add_(W[0], W[L]);
        } else {
            V[0] = F.ic2*(W[0] + W[L]) + W[1];
            V[1 + A] = F.irc*(W[L] - W[0]);
            V[DIM + 1] = W[0] + W[L];
        }
        int t = 2;
#pragma unroll
        for (int k = 0; k < DIM; k++) if (k != A) V[1 + k] = W[t++];
    } else {
#pragma unroll
        for (int s = 0; s < NSP; s++) {
            if constexpr (X) V[s] = add_(add_(mul_(-F.hz[s], W[0]), W[s + 1]), mul_(F.hz[s], W[L]));
            else V[s] = F.hz[s]*(W[L] - W[0]) + W[s + 1];
        }
#pragma unroll
        for (int s = 0; s < M::NZ; s++) V[M::IZ + s] = W[NSP + DIM + s];
        int t = NSP + 1;
#pragma unroll
        for (int k = 0; k < DIM; k++) {
            if (k == A) {
                if constexpr (X) V[NSP + k] = add_(mul_(double(1)/double(2), W[0]), mul_(double(1)/double(2), W[L]));
                else V[NSP + k] = double(1)/double(2)*(W[0] + W[L]);
            } else {
                V[NSP + k] = W[t++];
            }
        }
        if constexpr (X) V[NSP + DIM] = add_(mul_(F.m_hrc, W[0]), mul_(F.p_hrc, W[L]));
        else V[NSP + DIM] = F.p_hrc*(W[L] - W[0]);
    }
}

// ----------------------------------------------------------------------------
// WCNS5-JS (U[m] = characteristic variable at cell face-3+m).
// ----------------------------------------------------------------------------
// Smoothness indicators of the 3-point sub-stencils, S0..S4 ordered from the
// upwind side (U[0..4] for the minus side, U[5..1] for the plus side), every
// product explicitly rounded: see the note above char_from_prim.  WCNS6-LD's
// tau-switch (R_tau > alpha_tau) is a discrete decision on these values.
template <int E = 0>
__device__ __forceinline__ double lin3x(double c0, double a0, double c1, double a1, double c2, double a2) {
    return addx<E>(subx<E>(mulx<E>(c0, a0), mulx<E>(c1, a1)), mulx<E>(c2, a2));
}

template <int E = 0>
__device__ __forceinline__ void js_betas_x(double S0, double S1, double S2, double S3, double S4,
                                           double& b0, double& b1, double& b2) {
    // b0 = 1/3*(S0*(4*S0 - 19*S1 + 11*S2) + S1*(25*S1 - 31*S2) + 10*S2*S2)
    b0 = mulx<E>(double(1)/double(3), addx<E>(addx<E>(mulx<E>(S0, lin3x<E>(4.0, S0, 19.0, S1, 11.0, S2)),
                                            mulx<E>(S1, subx<E>(mulx<E>(25.0, S1), mulx<E>(31.0, S2)))),
                                       mulx<E>(mulx<E>(10.0, S2), S2)));
    // b1 = 1/3*(S1*(4*S1 - 13*S2 + 5*S3) + 13*S2*(S2 - S3) + 4*S3*S3)
    b1 = mulx<E>(double(1)/double(3), addx<E>(addx<E>(mulx<E>(S1, lin3x<E>(4.0, S1, 13.0, S2, 5.0, S3)),
                                            mulx<E>(mulx<E>(13.0, S2), subx<E>(S2, S3))),
                                       mulx<E>(mulx<E>(4.0, S3), S3)));
    // b2 = 1/3*(S2*(10*S2 - 31*S3 + 11*S4) + S3*(25*S3 - 19*S4) + 4*S4*S4)
    b2 = mulx<E>(double(1)/double(3), addx<E>(addx<E>(mulx<E>(S2, lin3x<E>(10.0, S2, 31.0, S3, 11.0, S4)),
                                            mulx<E>(S3, subx<E>(mulx<E>(25.0, S3), mulx<E>(19.0, S4)))),
                                       mulx<E>(mulx<E>(4.0, S4), S4)));
}

// Weighted 5-point midpoint value from the stencil S0..S4 (upwind first).
template <bool X>
__device__ __forceinline__ double js_interp(double b0, double b1, double b2, int p,
                                            double S0, double S1, double S2, double S3, double S4) {
    double w0, w1, w2;
    if constexpr (X) {
        // ConvectiveFluxReconstructorWCNS5-JS-HLLC-HLL.cpp:96-117
        w0 = double(1.0)/double(16)/ipow_<true>(add_(b0, HMR_EPS), p);
        w1 = double(5.0)/double(8)/ipow_<true>(add_(b1, HMR_EPS), p);
        w2 = double(5.0)/double(16)/ipow_<true>(add_(b2, HMR_EPS), p);
        const double ws = add_(add_(w0, w1), w2);
        w0 = w0/ws; w1 = w1/ws; w2 = w2/ws;
        const double t0 = mul_(mul_(double(3)/double(8), w0), S0);
        const double t1 = mul_(sub_(mul_(-double(10)/double(8), w0), mul_(double(1)/double(8), w1)), S1);
        const double t2 = mul_(add_(add_(mul_(double(15)/double(8), w0), mul_(double(6)/double(8), w1)),
                                    mul_(double(3)/double(8), w2)), S2);
        const double t3 = mul_(add_(mul_(double(3)/double(8), w1), mul_(double(6)/double(8), w2)), S3);
        const double t4 = mul_(mul_(double(1)/double(8), w2), S4);
        return sub_(add_(add_(add_(t0, t1), t2), t3), t4);
    } else {
        // w_k = d_k/(b_k+eps)^p / sum_j d_j/(b_j+eps)^p with a single reciprocal:
        // w_k = d_k prod_{j!=k} e_j / sum_m d_m prod_{j!=m} e_j.
        const double e0 = ipow_<false>(b0 + HMR_EPS, p), e1 = ipow_<false>(b1 + HMR_EPS, p),
                     e2 = ipow_<false>(b2 + HMR_EPS, p);
        const double a0 = double(1)/double(16)*(e1*e2);
        const double a1 = double(5)/double(8)*(e0*e2);
        const double a2 = double(5)/double(16)*(e0*e1);
        const double r = double(1)/(a0 + a1 + a2);
        w0 = a0*r; w1 = a1*r; w2 = a2*r;
        return double(3)/double(8)*w0*S0 +
            (-double(10)/double(8)*w0 - double(1)/double(8)*w1)*S1 +
            (double(15)/double(8)*w0 + double(6)/double(8)*w1 + double(3)/double(8)*w2)*S2 +
            (double(3)/double(8)*w1 + double(6)/double(8)*w2)*S3 -
            double(1)/double(8)*w2*S4;
    }
}

template <bool X>
__device__ __forceinline__ void js_pair(const double* U, int p, double& Um, double& Up) {
    double b0, b1, b2;
    js_betas_x<EMU_BETA_M>(U[0], U[1], U[2], U[3], U[4], b0, b1, b2);
    Um = js_interp<X>(b0, b1, b2, p, U[0], U[1], U[2], U[3], U[4]);
    js_betas_x<EMU_BETA_P>(U[5], U[4], U[3], U[2], U[1], b0, b1, b2);
    Up = js_interp<X>(b0, b1, b2, p, U[5], U[4], U[3], U[2], U[1]);
}

// ----------------------------------------------------------------------------
// WCNS6-LD.
// ----------------------------------------------------------------------------
__device__ __forceinline__ double ld_sigma(const double* U) {  // WCNS6-LD-HLLC-HLL.cpp:24-41
    const double a1 = sub_(U[2], U[1]);
    const double a2 = sub_(U[3], U[2]);
    const double a3 = sub_(U[4], U[3]);
    const double t1 = fabs(sub_(a1, a2))/add_(add_(fabs(a1), fabs(a2)), HMR_EPS);
    const double t2 = fabs(sub_(a2, a3))/add_(add_(fabs(a2), fabs(a3)), HMR_EPS);
    return fmax(t1, t2);
}

// beta_3 with the stencil ordered from the upwind side (S0..S5), every
// product explicitly rounded (see js_betas_x).  WCNS6-LD-HLLC-HLL.cpp:70-83.
template <int E = 0>
__device__ __forceinline__ double ld_beta3(double S0, double S1, double S2, double S3, double S4, double S5) {
    // S0*(525910327*S0 - 4562164630*S1 + 7799501420*S2 - 6610694540*S3 + 2794296070*S4 - 472758974*S5)
    const double t0 = mulx<E>(S0, subx<E>(addx<E>(subx<E>(addx<E>(subx<E>(mulx<E>(525910327.0, S0), mulx<E>(4562164630.0, S1)),
                                                  mulx<E>(7799501420.0, S2)), mulx<E>(6610694540.0, S3)),
                                        mulx<E>(2794296070.0, S4)), mulx<E>(472758974.0, S5)));
    // 5*S1*(2146987907*S1 - 7722406988*S2 + 6763559276*S3 - 2926461814*S4 + 503766638*S5)
    const double t1 = mulx<E>(mulx<E>(5.0, S1), addx<E>(subx<E>(addx<E>(subx<E>(mulx<E>(2146987907.0, S1), mulx<E>(7722406988.0, S2)),
                                                        mulx<E>(6763559276.0, S3)), mulx<E>(2926461814.0, S4)),
                                              mulx<E>(503766638.0, S5)));
    // 20*S2*(1833221603*S2 - 3358664662*S3 + 1495974539*S4 - 263126407*S5)
    const double t2 = mulx<E>(mulx<E>(20.0, S2), subx<E>(addx<E>(subx<E>(mulx<E>(1833221603.0, S2), mulx<E>(3358664662.0, S3)),
                                                    mulx<E>(1495974539.0, S4)), mulx<E>(263126407.0, S5)));
    // 20*S3*(1607794163*S3 - 1486026707*S4 + 268747951*S5)
    const double t3 = mulx<E>(mulx<E>(20.0, S3), addx<E>(subx<E>(mulx<E>(1607794163.0, S3), mulx<E>(1486026707.0, S4)),
                                               mulx<E>(268747951.0, S5)));
    // 5*S4*(1432381427*S4 - 536951582*S5)
    const double t4 = mulx<E>(mulx<E>(5.0, S4), subx<E>(mulx<E>(1432381427.0, S4), mulx<E>(536951582.0, S5)));
    // 263126407*S5*S5
    const double t5 = mulx<E>(mulx<E>(263126407.0, S5), S5);
    return mulx<E>(double(1)/double(232243200), addx<E>(addx<E>(addx<E>(addx<E>(addx<E>(t0, t1), t2), t3), t4), t5));
}

// WCNS6-LD's tau switch, R_tau = tau_6/(beta_avg + eps) > alpha_tau, decided without
// the division where the product m = alpha_tau (beta_avg + eps) is far from tau_6.  With
// u = 2^-53: tau_6 > m (1 + 1e-14) puts the exact quotient above alpha_tau (1 + 4u), so its
// rounding exceeds alpha_tau; tau_6 < m (1 - 1e-14) puts it below alpha_tau, so its rounding
// does not exceed it.  Between the two, for NaN, and outside the normal range the quotient
// is formed as the reference forms it.  The decision is the reference's bit for bit.
__device__ __forceinline__ bool ld_switch(double tau_6, double beta_avg, double alpha) {
    const double d = add_(beta_avg, HMR_EPS);
    const double m = mul_(alpha, d);
    if (alpha > 1.0e-280 && m > 1.0e-280 && m < 1.0e280) {
        if (tau_6 > mul_(m, 1.0 + 1.0e-14)) return true;
        if (tau_6 < mul_(m, 1.0 - 1.0e-14)) return false;
    }
    return tau_6/d > alpha;
}

// WCNS6-LD weights and midpoint value (WCNS6-LD-HLLC-HLL.cpp:158-222), stencil S0..S5 from
// the upwind side; b[0..3] are that side's smoothness indicators.
template <bool X>
// sigma: the pair's ld_sigma(U), or negative until a side needs it (computed on first use:
// it only enters where the switch blends).
__device__ __forceinline__ double ld_interp(const double* b, const double* U, double& sigma, const Params& P,
                                            double S0, double S1, double S2, double S3, double S4, double S5) {
    // Decision inputs are always exact (tau_5, tau_6, beta_avg), and the tau switch is the
    // reference's decision in both forms.
    const double tau_5 = fabs(sub_(b[0], b[2]));
    const double beta_avg = mul_(double(1)/double(8), add_(add_(b[0], b[2]), mul_(double(6), b[1])));
    const double tau_6 = fabs(sub_(b[3], beta_avg));
    const bool blend = X ? tau_6/add_(beta_avg, HMR_EPS) > P.alpha_tau : ld_switch(tau_6, beta_avg, P.alpha_tau);
    double u0 = 0.0, u1 = 0.0, u2 = 0.0, o0, o1, o2, o3;
    // The upwind weights u_k only enter when the switch blends (their value is not used
    // otherwise, so skipping them changes no result).
    if constexpr (X) {
        if (blend) {
            u0 = mul_(double(1)/double(16), add_(double(1), ipow_<true>(tau_5/add_(b[0], HMR_EPS), P.p)));
            u1 = mul_(double(5)/double(8), add_(double(1), ipow_<true>(tau_5/add_(b[1], HMR_EPS), P.p)));
            u2 = mul_(double(5)/double(16), add_(double(1), ipow_<true>(tau_5/add_(b[2], HMR_EPS), P.p)));
            const double us = add_(add_(u0, u1), u2);
            u0 = u0/us; u1 = u1/us; u2 = u2/us;
        }
        o0 = mul_(double(1)/double(32), add_(P.C, ipow_<true>(tau_6/add_(b[0], HMR_EPS), P.q)));
        o1 = mul_(double(15)/double(32), add_(P.C, ipow_<true>(tau_6/add_(b[1], HMR_EPS), P.q)));
        o2 = mul_(double(15)/double(32), add_(P.C, ipow_<true>(tau_6/add_(b[2], HMR_EPS), P.q)));
        o3 = mul_(double(1)/double(32), add_(P.C, ipow_<true>(tau_6/add_(b[3], HMR_EPS), P.q)));
        const double os = add_(add_(add_(o0, o1), o2), o3);
        o0 = o0/os; o1 = o1/os; o2 = o2/os; o3 = o3/os;
        if (blend) {
            if (sigma < 0.0) sigma = ld_sigma(U);
            const double ms = sub_(double(1), sigma);
            o0 = add_(mul_(sigma, u0), mul_(ms, o0));
            o1 = add_(mul_(sigma, u1), mul_(ms, o1));
            o2 = add_(mul_(sigma, u2), mul_(ms, o2));
            o3 = mul_(ms, o3);
        }
        const double t0 = mul_(mul_(double(3)/double(8), o0), S0);
        const double t1 = mul_(sub_(mul_(-double(10)/double(8), o0), mul_(double(1)/double(8), o1)), S1);
        const double t2 = mul_(add_(add_(mul_(double(15)/double(8), o0), mul_(double(6)/double(8), o1)),
                                    mul_(double(3)/double(8), o2)), S2);
        const double t3 = mul_(add_(add_(mul_(double(3)/double(8), o1), mul_(double(6)/double(8), o2)),
                                    mul_(double(15)/double(8), o3)), S3);
        const double t4 = mul_(sub_(mul_(-double(1)/double(8), o2), mul_(double(10)/double(8), o3)), S4);
        const double t5 = mul_(mul_(double(3)/double(8), o3), S5);
        return add_(add_(add_(add_(add_(t0, t1), t2), t3), t4), t5);
    } else {
        // the four 1/(beta_k + eps) from one division: 1/e_k = (prod_{j!=k} e_j)/(prod_j e_j)
        // (e_k in [1e-15, 1e77) keeps the product of four in range)
        const double e0 = b[0] + HMR_EPS, e1 = b[1] + HMR_EPS, e2 = b[2] + HMR_EPS, e3 = b[3] + HMR_EPS;
        const double e01 = e0*e1, e23 = e2*e3;
        const double rp = double(1)/(e01*e23);
        const double r0 = rp*(e1*e23), r1 = rp*(e0*e23), r2 = rp*(e01*e3), r3 = rp*(e01*e2);
        if (blend) {
            u0 = double(1)/double(16)*(double(1) + ipow_<false>(tau_5*r0, P.p));
            u1 = double(5)/double(8)*(double(1) + ipow_<false>(tau_5*r1, P.p));
            u2 = double(5)/double(16)*(double(1) + ipow_<false>(tau_5*r2, P.p));
            const double ru = double(1)/(u0 + u1 + u2);
            u0 *= ru; u1 *= ru; u2 *= ru;
        }
        o0 = double(1)/double(32)*(P.C + ipow_<false>(tau_6*r0, P.q));
        o1 = double(15)/double(32)*(P.C + ipow_<false>(tau_6*r1, P.q));
        o2 = double(15)/double(32)*(P.C + ipow_<false>(tau_6*r2, P.q));
        o3 = double(1)/double(32)*(P.C + ipow_<false>(tau_6*r3, P.q));
        const double ro = double(1)/(o0 + o1 + o2 + o3);
        o0 *= ro; o1 *= ro; o2 *= ro; o3 *= ro;
        if (blend) {
            if (sigma < 0.0) sigma = ld_sigma(U);
            o0 = sigma*u0 + (double(1) - sigma)*o0;
            o1 = sigma*u1 + (double(1) - sigma)*o1;
            o2 = sigma*u2 + (double(1) - sigma)*o2;
            o3 = (double(1) - sigma)*o3;
        }
        return double(3)/double(8)*o0*S0 +
            (-double(10)/double(8)*o0 - double(1)/double(8)*o1)*S1 +
            (double(15)/double(8)*o0 + double(6)/double(8)*o1 + double(3)/double(8)*o2)*S2 +
            (double(3)/double(8)*o1 + double(6)/double(8)*o2 + double(15)/double(8)*o3)*S3 +
            (-double(1)/double(8)*o2 - double(10)/double(8)*o3)*S4 +
            double(3)/double(8)*o3*S5;
    }
}

template <bool X>
__device__ __forceinline__ void ld_pair(const double* U, const Params& P, double& Um, double& Up) {
    double sigma = -1.0;   // ld_sigma(U), computed if a side blends
    double b[4];
    js_betas_x<EMU_BETA_M>(U[0], U[1], U[2], U[3], U[4], b[0], b[1], b[2]);
    b[3] = ld_beta3<EMU_BETA_M>(U[0], U[1], U[2], U[3], U[4], U[5]);
    Um = ld_interp<X>(b, U, sigma, P, U[0], U[1], U[2], U[3], U[4], U[5]);
    js_betas_x<EMU_BETA_P>(U[5], U[4], U[3], U[2], U[1], b[0], b[1], b[2]);
    b[3] = ld_beta3<EMU_BETA_P>(U[5], U[4], U[3], U[2], U[1], U[0]);
    Up = ld_interp<X>(b, U, sigma, P, U[5], U[4], U[3], U[2], U[1], U[0]);
}

// ----------------------------------------------------------------------------
// WCNS5-Z (WCNS5-Z-HLLC-HLL.cpp:78-168): the WCNS5-JS indicators and stencil,
// weights d_k (1 + (tau_5/(beta_k + eps))^p) with tau_5 = |beta_0 - beta_2|.
// ----------------------------------------------------------------------------
template <bool X>
__device__ __forceinline__ double z_interp(double b0, double b1, double b2, int p,
                                           double S0, double S1, double S2, double S3, double S4) {
    const double tau_5 = fabs(sub_(b0, b2));
    double w0, w1, w2;
    if constexpr (X) {
        w0 = mul_(double(1)/double(16), add_(double(1), ipow_<true>(tau_5/add_(b0, HMR_EPS), p)));
        w1 = mul_(double(5)/double(8), add_(double(1), ipow_<true>(tau_5/add_(b1, HMR_EPS), p)));
        w2 = mul_(double(5)/double(16), add_(double(1), ipow_<true>(tau_5/add_(b2, HMR_EPS), p)));
        const double ws = add_(add_(w0, w1), w2);
        w0 = w0/ws; w1 = w1/ws; w2 = w2/ws;
        const double t0 = mul_(mul_(double(3)/double(8), w0), S0);
        const double t1 = mul_(sub_(mul_(-double(10)/double(8), w0), mul_(double(1)/double(8), w1)), S1);
        const double t2 = mul_(add_(add_(mul_(double(15)/double(8), w0), mul_(double(6)/double(8), w1)),
                                    mul_(double(3)/double(8), w2)), S2);
        const double t3 = mul_(add_(mul_(double(3)/double(8), w1), mul_(double(6)/double(8), w2)), S3);
        const double t4 = mul_(mul_(double(1)/double(8), w2), S4);
        return sub_(add_(add_(add_(t0, t1), t2), t3), t4);
    } else {
        // d_k (1 + T/E_k) with E_k = (beta_k + eps)^p, T = tau_5^p, over one common
        // denominator: w_k = d_k (E_k + T) prod_{j!=k} E_j / sum_m (...).
        const double T = ipow_<false>(tau_5, p);
        const double e0 = ipow_<false>(b0 + HMR_EPS, p), e1 = ipow_<false>(b1 + HMR_EPS, p),
                     e2 = ipow_<false>(b2 + HMR_EPS, p);
        const double a0 = double(1)/double(16)*((e0 + T)*(e1*e2));
        const double a1 = double(5)/double(8)*((e1 + T)*(e0*e2));
        const double a2 = double(5)/double(16)*((e2 + T)*(e0*e1));
        const double r = double(1)/(a0 + a1 + a2);
        w0 = a0*r; w1 = a1*r; w2 = a2*r;
        return double(3)/double(8)*w0*S0 +
            (-double(10)/double(8)*w0 - double(1)/double(8)*w1)*S1 +
            (double(15)/double(8)*w0 + double(6)/double(8)*w1 + double(3)/double(8)*w2)*S2 +
            (double(3)/double(8)*w1 + double(6)/double(8)*w2)*S3 -
            double(1)/double(8)*w2*S4;
    }
}

template <bool X>
__device__ __forceinline__ void z_pair(const double* U, int p, double& Um, double& Up) {
    double b0, b1, b2;
    js_betas_x<EMU_BETA_M>(U[0], U[1], U[2], U[3], U[4], b0, b1, b2);
    Um = z_interp<X>(b0, b1, b2, p, U[0], U[1], U[2], U[3], U[4]);
    js_betas_x<EMU_BETA_P>(U[5], U[4], U[3], U[2], U[1], b0, b1, b2);
    Up = z_interp<X>(b0, b1, b2, p, U[5], U[4], U[3], U[2], U[1]);
}

// ----------------------------------------------------------------------------
// WCNS6-CU-M2 (WCNS6-CU-M2-HLLC-HLL.cpp:112-228): the WCNS6-LD indicators and
// stencil, weights d_k (C + tau_6/(beta_k + eps dx^2) (beta_avg + Chi dx^2)/(beta_k + Chi dx^2))^q
// with beta_avg = (beta_0 + beta_2 + 6 beta_1)/8, tau_6 = |beta_3 - beta_avg|.
// ce = eps dx^2 and cx = Chi dx^2 of the face's axis.
// ----------------------------------------------------------------------------
template <bool X>
__device__ __forceinline__ double cu_interp(const double* b, const Params& P, double ce, double cx,
                                            double S0, double S1, double S2, double S3, double S4, double S5) {
    const double beta_avg = mul_(double(1)/double(8), add_(add_(b[0], b[2]), mul_(double(6), b[1])));
    const double tau_6 = fabs(sub_(b[3], beta_avg));
    double o0, o1, o2, o3;
    if constexpr (X) {
        const double ax = add_(beta_avg, cx);
        o0 = mul_(double(1)/double(32), ipow_<true>(add_(P.C, mul_(tau_6/add_(b[0], ce), ax)/add_(b[0], cx)), P.q));
        o1 = mul_(double(15)/double(32), ipow_<true>(add_(P.C, mul_(tau_6/add_(b[1], ce), ax)/add_(b[1], cx)), P.q));
        o2 = mul_(double(15)/double(32), ipow_<true>(add_(P.C, mul_(tau_6/add_(b[2], ce), ax)/add_(b[2], cx)), P.q));
        o3 = mul_(double(1)/double(32), ipow_<true>(add_(P.C, mul_(tau_6/add_(b[3], ce), ax)/add_(b[3], cx)), P.q));
        const double os = add_(add_(add_(o0, o1), o2), o3);
        o0 = o0/os; o1 = o1/os; o2 = o2/os; o3 = o3/os;
        const double t0 = mul_(mul_(double(3)/double(8), o0), S0);
        const double t1 = mul_(sub_(mul_(-double(10)/double(8), o0), mul_(double(1)/double(8), o1)), S1);
        const double t2 = mul_(add_(add_(mul_(double(15)/double(8), o0), mul_(double(6)/double(8), o1)),
                                    mul_(double(3)/double(8), o2)), S2);
        const double t3 = mul_(add_(add_(mul_(double(3)/double(8), o1), mul_(double(6)/double(8), o2)),
                                    mul_(double(15)/double(8), o3)), S3);
        const double t4 = mul_(sub_(mul_(-double(1)/double(8), o2), mul_(double(10)/double(8), o3)), S4);
        const double t5 = mul_(mul_(double(3)/double(8), o3), S5);
        return add_(add_(add_(add_(add_(t0, t1), t2), t3), t4), t5);
    } else {
        // g/d_k with d_k = (beta_k + eps dx^2)(beta_k + Chi dx^2), the four from one division
        const double g = tau_6*(beta_avg + cx);
        const double d0 = (b[0] + ce)*(b[0] + cx), d1 = (b[1] + ce)*(b[1] + cx);
        const double d2 = (b[2] + ce)*(b[2] + cx), d3 = (b[3] + ce)*(b[3] + cx);
        const double d01 = d0*d1, d23 = d2*d3;
        const double gp = g/(d01*d23);
        o0 = double(1)/double(32)*ipow_<false>(P.C + gp*(d1*d23), P.q);
        o1 = double(15)/double(32)*ipow_<false>(P.C + gp*(d0*d23), P.q);
        o2 = double(15)/double(32)*ipow_<false>(P.C + gp*(d01*d3), P.q);
        o3 = double(1)/double(32)*ipow_<false>(P.C + gp*(d01*d2), P.q);
        const double ro = double(1)/(o0 + o1 + o2 + o3);
        o0 *= ro; o1 *= ro; o2 *= ro; o3 *= ro;
        return double(3)/double(8)*o0*S0 +
            (-double(10)/double(8)*o0 - double(1)/double(8)*o1)*S1 +
            (double(15)/double(8)*o0 + double(6)/double(8)*o1 + double(3)/double(8)*o2)*S2 +
            (double(3)/double(8)*o1 + double(6)/double(8)*o2 + double(15)/double(8)*o3)*S3 +
            (-double(1)/double(8)*o2 - double(10)/double(8)*o3)*S4 +
            double(3)/double(8)*o3*S5;
    }
}

template <bool X, int A>
__device__ __forceinline__ void cu_pair(const double* U, const Params& P, double& Um, double& Up) {
    double b[4];
    js_betas_x<EMU_BETA_M>(U[0], U[1], U[2], U[3], U[4], b[0], b[1], b[2]);
    b[3] = ld_beta3<EMU_BETA_M>(U[0], U[1], U[2], U[3], U[4], U[5]);
    Um = cu_interp<X>(b, P, P.cu_e[A], P.cu_x[A], U[0], U[1], U[2], U[3], U[4], U[5]);
    js_betas_x<EMU_BETA_P>(U[5], U[4], U[3], U[2], U[1], b[0], b[1], b[2]);
    b[3] = ld_beta3<EMU_BETA_P>(U[5], U[4], U[3], U[2], U[1], U[0]);
    Up = cu_interp<X>(b, P, P.cu_e[A], P.cu_x[A], U[5], U[4], U[3], U[2], U[1], U[0]);
}

// ----------------------------------------------------------------------------
// Bounds check of a reconstructed face state.  Always exact (a discrete
// decision).  `margin` receives how far the state is from the nearest bound,
// relative to its scale, so that the fast kernels can recompute faces whose
// decision could depend on rounding.
// single: FlowModelBasicUtilitiesSingleSpecies.cpp:3013-3440;
// five:   FlowModelBasicUtilitiesFiveEqnAllaire.cpp:5446-7347, bounds
//         FlowModelBasicUtilitiesFiveEqnAllaire.hpp:24-27.
// ----------------------------------------------------------------------------
template <int DIM, int MODEL, int NSP>
__device__ __forceinline__ bool face_bounded(const Params& P, const double* V, double& margin) {
    using M = Model<DIM, MODEL, NSP>;
    if constexpr (MODEL == SINGLE_SPECIES) {
        margin = fmin(fabs(V[0]), fabs(V[DIM + 1]));
        return (V[0] > 0.0) && (V[DIM + 1] > 0.0);
    } else if constexpr (MODEL == FOUR_EQN_CONSERVATIVE) {
        // FlowModelBasicUtilitiesFourEqnConservative.cpp:3737-4510, bounds
        // FlowModelBasicUtilitiesFourEqnConservative.hpp:24-25: Y in (-0.001, 1.001), rho > 0, p > 0.
        // margin covers the mass fractions; the caller adds density and pressure.
        double rho = 0.0;
#pragma unroll
        for (int s = 0; s < NSP; s++) rho = add_(rho, V[s]);
        bool ok = true;
        double m = 1.0e300;
#pragma unroll
        for (int s = 0; s < NSP; s++) {
            const double Y = V[s]/rho;
            ok = ok && (Y > -0.001 && Y < 1.001);
            m = fmin(m, fmin(fabs(Y + 0.001), fabs(1.001 - Y)));
        }
        ok = ok && (rho > 0.0) && (V[NSP + DIM] > 0.0);
        margin = m;
        return ok;
    } else {
        bool ok = true;
        double Z[NSP];
        Z[NSP - 1] = 1.0;
#pragma unroll
        for (int s = 0; s < NSP - 1; s++) {
            Z[s] = V[M::IZ + s];
            Z[NSP - 1] = sub_(Z[NSP - 1], Z[s]);
            ok = ok && (Z[s] > -1000.0 && Z[s] < 1000.0);
        }
        ok = ok && (Z[NSP - 1] > -1000.0 && Z[NSP - 1] < 1000.0);
        double rho = 0.0;
#pragma unroll
        for (int s = 0; s < NSP; s++) rho = add_(rho, V[s]);
        double Y[NSP];
        double m = 1.0e300;
#pragma unroll
        for (int s = 0; s < NSP; s++) {
            Y[s] = V[s]/rho;
            ok = ok && (Y[s] > -0.001 && Y[s] < 1.001);
            m = fmin(m, fmin(fabs(Y[s] + 0.001), fabs(1.001 - Y[s])));
        }
#pragma unroll
        for (int s = 0; s < NSP; s++) {
            ok = ok && (V[s] > 0.0);
            m = fmin(m, fabs(Y[s]));
        }
        const double p = V[NSP + DIM];
        const double gamma = gamma_all_x<NSP>(P, Z);
        const double Gamma = sub_(gamma, double(1));
        const double Psi = p/rho;
        double c2 = mul_(Gamma, p)/rho;
#pragma unroll
        for (int s = 0; s < NSP; s++) c2 = add_(c2, mul_(Y[s], Psi));
        ok = ok && (c2 > 0.0);
        margin = fmin(m, fabs(c2)/fmax(fabs(mul_(Gamma, p)/rho), 1e-300));
        return ok;
    }
}

// ----------------------------------------------------------------------------
// Face thermodynamics of one reconstructed state (Riemann drivers).
// single: EquationOfStateIdealGas.cpp:5806 (c), :6135 (eps)
// five:   FlowModelRiemannSolverFiveEqnAllaireHLLC.cpp:4824-6097 (rho, Y, Gamma, c, eps)
// ----------------------------------------------------------------------------
template <bool X, int DIM, int MODEL, int NSP>
__device__ __forceinline__ void face_thermo(const Params& P, const double* V, double& rho, double& cs,
                                            double& eps) {
    using M = Model<DIM, MODEL, NSP>;
    if constexpr (MODEL == SINGLE_SPECIES) {
        const double gamma = P.gamma[0];
        rho = V[0];
        const double p = V[DIM + 1];
        if constexpr (X) {
            cs = sqrt(mul_(gamma, p)/rho);
            eps = p/mul_(sub_(gamma, double(1)), rho);
        } else {
            const double ri = double(1)/rho;
            cs = sqrt(gamma*p*ri);
            eps = p*ri*P.inv_gm1[0];
        }
    } else if constexpr (MODEL == FOUR_EQN_CONSERVATIVE) {
        // FlowModelRiemannSolverFourEqnConservativeHLLC-HLL.cpp:5530-5680 (2D x block)
        double r = 0.0;
#pragma unroll
        for (int s = 0; s < NSP; s++) r = X ? add_(r, V[s]) : r + V[s];
        rho = r;
        const double p = V[NSP + DIM];
        double Y[NSP];
        if constexpr (X) {
#pragma unroll
            for (int s = 0; s < NSP; s++) Y[s] = V[s]/r;
            cs = sqrt(four_c2_x<NSP>(P, r, p, Y, eps));
        } else {
            const double ri = double(1)/r;
#pragma unroll
            for (int s = 0; s < NSP; s++) Y[s] = V[s]*ri;
            double cv;
            const double gamma = mix_mass<false, NSP>(P, Y, cv);
            const double icv = double(1)/cv;
            const double gm1 = gamma - double(1);
            const double pr = p*ri;
            eps = pr/gm1;
            double c2 = gm1*pr;
#pragma unroll
            for (int s = 0; s < NSP; s++) c2 += Y[s]*(((P.cp[s] - gamma*P.cv[s])*icv + gm1)*eps);
            cs = sqrt(c2);
        }
    } else {
        double r = 0.0;
#pragma unroll
        for (int s = 0; s < NSP; s++) r = X ? add_(r, V[s]) : r + V[s];
        rho = r;
        const double p = V[NSP + DIM];
        const double gamma = gamma_last<X, NSP>(P, V + M::IZ);
        if constexpr (X) {
            double Y[NSP];
#pragma unroll
            for (int s = 0; s < NSP; s++) Y[s] = V[s]/r;
            const double Gamma = sub_(gamma, double(1));
            const double Psi = p/r;
            double c2 = mul_(Gamma, p)/r;
#pragma unroll
            for (int s = 0; s < NSP; s++) c2 = add_(c2, mul_(Y[s], Psi));
            cs = sqrt(c2);
            eps = p/mul_(sub_(gamma, double(1)), r);
        } else {
            const double ri = double(1)/r;
            const double Psi = p*ri;
            double c2 = (gamma - double(1))*Psi;
#pragma unroll
            for (int s = 0; s < NSP; s++) c2 += (V[s]*ri)*Psi;
            cs = sqrt(c2);
            eps = Psi/(gamma - double(1));
        }
    }
}

// Conserved state and physical flux of one face state.
template <bool X, int DIM, int MODEL, int NSP, int A>
__device__ __forceinline__ void face_QF(const double* V, double rho, double eps, double* Q, double* F) {
    using M = Model<DIM, MODEL, NSP>;
    if constexpr (MODEL == SINGLE_SPECIES) {
        const double p = V[DIM + 1];
        Q[0] = V[0];
#pragma unroll
        for (int k = 0; k < DIM; k++) Q[1 + k] = X ? mul_(V[0], V[1 + k]) : V[0]*V[1 + k];
        double ke = X ? mul_(V[1], V[1]) : V[1]*V[1];
#pragma unroll
        for (int k = 1; k < DIM; k++) ke = X ? add_(ke, mul_(V[1 + k], V[1 + k])) : ke + V[1 + k]*V[1 + k];
        Q[DIM + 1] = X ? mul_(V[0], add_(eps, mul_(double(1)/double(2), ke)))
                       : V[0]*(eps + double(1)/double(2)*ke);
        F[0] = Q[1 + A];
#pragma unroll
        for (int k = 0; k < DIM; k++) {
            if (k == A) F[1 + k] = X ? add_(mul_(Q[1 + A], V[1 + k]), p) : Q[1 + A]*V[1 + k] + p;
            else F[1 + k] = X ? mul_(Q[1 + A], V[1 + k]) : Q[1 + A]*V[1 + k];
        }
        F[DIM + 1] = X ? mul_(V[1 + A], add_(Q[DIM + 1], p)) : V[1 + A]*(Q[DIM + 1] + p);
    } else {
        const double p = V[NSP + DIM];
        const double un = V[NSP + A];
#pragma unroll
        for (int s = 0; s < NSP; s++) Q[s] = V[s];
#pragma unroll
        for (int k = 0; k < DIM; k++) Q[NSP + k] = X ? mul_(rho, V[NSP + k]) : rho*V[NSP + k];
        double ke = X ? mul_(V[NSP], V[NSP]) : V[NSP]*V[NSP];
#pragma unroll
        for (int k = 1; k < DIM; k++)
            ke = X ? add_(ke, mul_(V[NSP + k], V[NSP + k])) : ke + V[NSP + k]*V[NSP + k];
        Q[NSP + DIM] = X ? mul_(rho, add_(eps, mul_(double(1)/double(2), ke)))
                         : rho*(eps + double(1)/double(2)*ke);
#pragma unroll
        for (int s = 0; s < M::NZ; s++) Q[M::IZ + s] = V[M::IZ + s];
#pragma unroll
        for (int s = 0; s < NSP; s++) F[s] = X ? mul_(un, V[s]) : un*V[s];
#pragma unroll
        for (int k = 0; k < DIM; k++) {
            if (k == A) F[NSP + k] = X ? add_(mul_(un, Q[NSP + k]), p) : un*Q[NSP + k] + p;
            else F[NSP + k] = X ? mul_(un, Q[NSP + k]) : un*Q[NSP + k];
        }
        F[NSP + DIM] = X ? mul_(un, add_(Q[NSP + DIM], p)) : un*(Q[NSP + DIM] + p);
#pragma unroll
        for (int s = 0; s < M::NZ; s++) F[M::IZ + s] = X ? mul_(un, V[M::IZ + s]) : un*V[M::IZ + s];
    }
}

template <int DIM, int MODEL, int NSP, int A>
__device__ __forceinline__ constexpr bool hll_comp(int e) {
    if constexpr (MODEL == SINGLE_SPECIES) {
        return e == 0 || (e >= 1 && e <= DIM && (e - 1) != A);
    } else {
        return e < NSP || (e >= NSP && e < NSP + DIM && (e - NSP) != A) || e > NSP + DIM;
    }
}

// Midpoint flux of one face: HLLC, or HLLC-HLL when use_hll is set (the
// shock sensor's choice, WCNS56-HLLC-HLL.cpp:1090-1113), and the HLLC
// midpoint normal velocity.
//  HLLC:     FlowModelRiemannSolverSingleSpeciesHLLC.cpp:604-692 (five: ...FiveEqnAllaireHLLC.cpp:848-990)
//  HLLC-HLL: FlowModelRiemannSolverSingleSpeciesHLLC-HLL.cpp:889-1027 (five: ...FiveEqnAllaireHLLC-HLL.cpp:1283-1503)
template <bool X, int DIM, int MODEL, int NSP, int A>
__device__ __forceinline__ void riemann(const Params& P, const double* VL, const double* VR, bool use_hll,
                                        double* Fout, double& u_mid) {
    using M = Model<DIM, MODEL, NSP>;
    constexpr int NEQ = M::NEQ;
    constexpr int IU = M::IU;
    constexpr int IP = M::IP;
    double rhoL, cL, epsL, rhoR, cR, epsR;
    face_thermo<X, DIM, MODEL, NSP>(P, VL, rhoL, cL, epsL);
    face_thermo<X, DIM, MODEL, NSP>(P, VR, rhoR, cR, epsR);
    const double uL = VL[IU + A], uR = VR[IU + A];
    const double pL = VL[IP], pR = VR[IP];
    double s_L, s_R, s_star;
    if constexpr (X) {
        const double u_average = mul_(double(1)/double(2), add_(uL, uR));
        const double c_average = mul_(double(1)/double(2), add_(cL, cR));
        s_L = fmin(sub_(u_average, c_average), sub_(uL, cL));
        s_R = fmax(add_(u_average, c_average), add_(uR, cR));
        const double num = sub_(add_(sub_(pR, pL), mul_(mul_(rhoL, uL), sub_(s_L, uL))),
                                mul_(mul_(rhoR, uR), sub_(s_R, uR)));
        const double den = sub_(mul_(rhoL, sub_(s_L, uL)), mul_(rhoR, sub_(s_R, uR)));
        s_star = num/den;
    } else {
        const double u_average = double(1)/double(2)*(uL + uR);
        const double c_average = double(1)/double(2)*(cL + cR);
        s_L = fmin(u_average - c_average, uL - cL);
        s_R = fmax(u_average + c_average, uR + cR);
        s_star = (pR - pL + rhoL*uL*(s_L - uL) - rhoR*uR*(s_R - uR))/(rhoL*(s_L - uL) - rhoR*(s_R - uR));
    }
    const double s_minus = fmin(0.0, s_L);
    const double s_plus = fmax(0.0, s_R);

    const bool left = s_star > 0.0;
    const double* VK = left ? VL : VR;
    const double rhoK = left ? rhoL : rhoR;
    const double epsK = left ? epsL : epsR;
    const double sK = left ? s_L : s_R;
    const double uK = left ? uL : uR;
    const double pK = left ? pL : pR;
    const double s_pm = left ? s_minus : s_plus;
    double QK[NEQ], FK[NEQ], Qs[NEQ];
    face_QF<X, DIM, MODEL, NSP, A>(VK, rhoK, epsK, QK, FK);
    const double Chi = X ? sub_(sK, uK)/sub_(sK, s_star) : (sK - uK)/(sK - s_star);
    // Energy of the star state: Chi*(E_K + (s* - u_K)*(rho_K s* + p_K/(s_K - u_K)))
    const double rK = (MODEL == SINGLE_SPECIES) ? VK[0] : rhoK;
    double QsE;
    if constexpr (X) QsE = mul_(Chi, add_(QK[M::IE], mul_(sub_(s_star, uK), add_(mul_(rK, s_star), pK/sub_(sK, uK)))));
    else QsE = Chi*(QK[M::IE] + (s_star - uK)*(rK*s_star + pK/(sK - uK)));
    if constexpr (MODEL == SINGLE_SPECIES) {
        Qs[0] = X ? mul_(Chi, VK[0]) : Chi*VK[0];
#pragma unroll
        for (int k = 0; k < DIM; k++) {
            if (k == A) Qs[1 + k] = X ? mul_(mul_(Chi, VK[0]), s_star) : Chi*VK[0]*s_star;
            else Qs[1 + k] = X ? mul_(Chi, QK[1 + k]) : Chi*QK[1 + k];
        }
        Qs[DIM + 1] = QsE;
    } else {
#pragma unroll
        for (int s = 0; s < NSP; s++) Qs[s] = X ? mul_(Chi, VK[s]) : Chi*VK[s];
#pragma unroll
        for (int k = 0; k < DIM; k++) {
            if (k == A) Qs[NSP + k] = X ? mul_(mul_(Chi, rhoK), s_star) : Chi*rhoK*s_star;
            else Qs[NSP + k] = X ? mul_(Chi, QK[NSP + k]) : Chi*QK[NSP + k];
        }
        Qs[NSP + DIM] = QsE;
#pragma unroll
        for (int s = 0; s < M::NZ; s++) Qs[M::IZ + s] = X ? mul_(Chi, VK[M::IZ + s]) : Chi*VK[M::IZ + s];
    }
#pragma unroll
    for (int e = 0; e < NEQ; e++) Fout[e] = X ? add_(FK[e], mul_(s_pm, sub_(Qs[e], QK[e]))) : FK[e] + s_pm*(Qs[e] - QK[e]);
    u_mid = X ? add_(uK, mul_(s_pm, sub_(Chi, double(1)))) : uK + s_pm*(Chi - double(1));

    if (use_hll) {
        // HLL for mass/partial densities, transverse momenta and volume
        // fractions, blended with HLLC by the direction of the velocity jump.
        double QL[NEQ], FL[NEQ], QR[NEQ], FR[NEQ];
        face_QF<X, DIM, MODEL, NSP, A>(VL, rhoL, epsL, QL, FL);
        face_QF<X, DIM, MODEL, NSP, A>(VR, rhoR, epsR, QR, FR);
        double diff[DIM];
#pragma unroll
        for (int k = 0; k < DIM; k++) diff[k] = VR[IU + k] - VL[IU + k];
        double vsq = X ? mul_(diff[0], diff[0]) : diff[0]*diff[0];
#pragma unroll
        for (int k = 1; k < DIM; k++) vsq = X ? add_(vsq, mul_(diff[k], diff[k])) : vsq + diff[k]*diff[k];
        const double vel_mag = sqrt(vsq);
        double alpha_1, alpha_2;
        if (vel_mag < HMR_EPS) {
            alpha_1 = 1.0;
            alpha_2 = 0.0;
        } else {
            alpha_1 = fabs(diff[A])/vel_mag;
            alpha_2 = sqrt(X ? sub_(double(1), mul_(alpha_1, alpha_1)) : double(1) - alpha_1*alpha_1);
        }
        const double beta_1 = X ? mul_(double(1)/double(2), add_(double(1), alpha_1/add_(alpha_1, alpha_2)))
                                : double(1)/double(2)*(double(1) + alpha_1/(alpha_1 + alpha_2));
        const double beta_2 = double(1) - beta_1;
#pragma unroll
        for (int e = 0; e < NEQ; e++) {
            if (hll_comp<DIM, MODEL, NSP, A>(e)) {
                double Fh;
                if (s_L > 0.0) Fh = FL[e];
                else if (s_R < 0.0) Fh = FR[e];
                else if constexpr (X)
                    Fh = add_(sub_(mul_(s_R, FL[e]), mul_(s_L, FR[e])), mul_(mul_(s_R, s_L), sub_(QR[e], QL[e])))/
                         sub_(s_R, s_L);
                else Fh = (s_R*FL[e] - s_L*FR[e] + s_R*s_L*(QR[e] - QL[e]))/(s_R - s_L);
                Fout[e] = X ? add_(mul_(beta_1, Fout[e]), mul_(beta_2, Fh)) : beta_1*Fout[e] + beta_2*Fh;
            }
        }
    }
}

}  // namespace hmr
