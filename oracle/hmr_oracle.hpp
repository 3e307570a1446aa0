// CPU oracle for the HAMeRS per-patch convective hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker that the GPU path is
// compared against; nothing in the product (the hamers_gb300 package or its
// CUDA library) includes, links or calls it.  Only tests/, the smoke check and
// the CPU-baseline leg of bench.py load the compiled oracle.
//
// It restates, sweep by sweep, the reference's FP64 algorithm for one patch:
//
//   ConvectiveFluxReconstructorWCNS56::computeConvectiveFluxAndSourceOnPatch
//     src/flow/convective_flux_reconstructors/WCNS56/ConvectiveFluxReconstructorWCNS56-HLLC-HLL.cpp:40-2656
//   Euler::advanceSingleStepOnPatch                       src/apps/Euler/Euler.cpp:1003-1680
//
// Every arithmetic expression keeps the reference's operation order (it is
// compiled with -ffp-contract=off), so that a GPU build without FMA
// contraction can be compared bit for bit.  Each function cites the reference
// lines it follows.  The scalar type is a template parameter so that a dual
// number can produce the FP64 tangent of the same code path.
//
// Parity pins: the reference ships no golden flux vectors; its own tests pin
// only the order of accuracy (tests/2D_convergence_test_*/convergence_test.py:8-16,
// L2 rate > 4.8 for WCNS5-JS and > 5.8 for WCNS6-LD).  tests/test_oracle_convergence.py
// reruns those problems through this oracle and checks the same rates.

#pragma once

#include <cmath>
#include <cstring>
#include <vector>
#include <algorithm>

namespace hmro {

// HAMERS_EPSILON, include/HAMeRS_config.hpp.in:16
constexpr double EPS = 1.0e-15;

// ---------------------------------------------------------------------------
// Scalar helpers.  Overloaded for the dual-number type in hmr_dual.hpp.
// ---------------------------------------------------------------------------
inline double s_sqrt(double a) { return std::sqrt(a); }
inline double s_fabs(double a) { return std::fabs(a); }
inline double s_fmin(double a, double b) { return std::fmin(a, b); }
inline double s_fmax(double a, double b) { return std::fmax(a, b); }
inline double s_val(double a) { return a; }

// Sub-phase markers for the operation counter (hmr_opcount.cpp defines HMRO_PHASE to attribute
// every counted operation to the current sub-phase); no-ops otherwise.
enum { HMRO_PH_CELLS = 0, HMRO_PH_SENSOR, HMRO_PH_PROJ, HMRO_PH_CHAR, HMRO_PH_BETA, HMRO_PH_WEIGHTS,
       HMRO_PH_INV, HMRO_PH_BOUNDS, HMRO_PH_RIEMANN, HMRO_PH_FLUX, HMRO_PH_SOURCE, HMRO_PH_STAGE, HMRO_NPH };
#ifndef HMRO_PHASE
#define HMRO_PHASE(k) ((void)0)
#endif

enum { MODEL_SINGLE_SPECIES = 0, MODEL_FOUR_EQN_CONSERVATIVE = 1, MODEL_FIVE_EQN_ALLAIRE = 2 };
// ConvectiveFluxReconstructorManager.cpp:40-91: WCNS5_JS_HLLC_HLL, WCNS6_LD_HLLC_HLL,
// WCNS5_Z_HLLC_HLL, WCNS6_CU_M2_HLLC_HLL (all on the WCNS56 driver).
enum { SCHEME_WCNS5_JS = 0, SCHEME_WCNS6_LD = 1, SCHEME_WCNS5_Z = 2, SCHEME_WCNS6_CU_M2 = 3 };

struct Config {
    int model;
    int dim;
    int num_species;
    int scheme;
    double gamma[8];     // species_gamma
    double R[8];         // species_R (four-equation model: species heat capacities)
    int p;               // constant_p  (JS, Z default 2, WCNS5-JS-HLLC-HLL.cpp:188-191; LD default 2)
    int q;               // constant_q  (LD, CU-M2 default 4, WCNS6-LD-HLLC-HLL.cpp:343-361)
    double C;            // constant_C  (LD default 1e9; CU-M2 default 1000, WCNS6-CU-M2-HLLC-HLL.cpp:252-270)
    double alpha_tau;    // constant_alpha_tau (LD default 35)
    double Chi;          // constant_Chi (CU-M2 default 1e8)
    double epsilon;      // constant_epsilon (CU-M2 default 1e-8)
    double grid_dx[3];   // CartesianGridGeometry::getDx(): the coarsest level's spacing, which
                         // WCNS6-CU-M2 uses on every level (WCNS6-CU-M2-HLLC-HLL.cpp:367-368)
    int ghosts = 4;      // ghost width of the patch arrays: 4 (WCNS56-HLLC-HLL.cpp:22), or 5 with
                         // the sixth-order diffusive flux (DiffusiveFluxReconstructorMidpointSixthOrder.cpp:22)
};

// Number of equations.  single: 2+dim (FlowModelSingleSpecies.cpp:29);
// four-eqn: N+dim+1; five-eqn: dim+2N (FlowModelFiveEqnAllaire.cpp:29).
inline int num_eqn(const Config& c) {
    if (c.model == MODEL_SINGLE_SPECIES) return c.dim + 2;
    if (c.model == MODEL_FOUR_EQN_CONSERVATIVE) return c.num_species + c.dim + 1;
    return c.dim + 2 * c.num_species;
}
// Number of volume fractions in the equations (five-equation model only).
inline int num_vf(const Config& c) { return c.model == MODEL_FIVE_EQN_ALLAIRE ? c.num_species - 1 : 0; }
// Number of stored conserved components: the five-equation model also keeps
// the last volume fraction (CellVariable of depth N, FlowModelFiveEqnAllaire.cpp:130-140).
inline int num_comp(const Config& c) {
    return num_eqn(c) + (c.model == MODEL_FIVE_EQN_ALLAIRE ? 1 : 0);
}

// Patch geometry: interior n[3] (n[2]=1 in 2D), ghost width g (4 for WCNS56,
// ConvectiveFluxReconstructorWCNS56-HLLC-HLL.cpp:22).
struct Box {
    int dim;
    int n[3];
    int g[3];   // ghost width per axis (0 on the unused z axis in 2D)
    int G[3];   // ghost-box extents
    long cell(int i, int j, int k) const {
        return (long)(i + g[0]) + (long)(j + g[1]) * G[0] + (long)(k + g[2]) * G[0] * G[1];
    }
    long ncell() const { return (long)G[0] * G[1] * G[2]; }
};

inline Box make_box(int dim, const int* n, int ghost) {
    Box b;
    b.dim = dim;
    for (int d = 0; d < 3; d++) {
        b.n[d] = (d < dim) ? n[d] : 1;
        b.g[d] = (d < dim) ? ghost : 0;
        b.G[d] = b.n[d] + 2 * b.g[d];
    }
    return b;
}

// Faces normal to axis a used by the reconstruction: index along a in
// [-1, n_a+1], interior along the other axes (the loops of
// WCNS56-HLLC-HLL.cpp:966-1031 and WCNS5-JS-HLLC-HLL.cpp:489-505).
struct FaceSet {
    int a;
    int lo[3], ext[3];
    long idx(int i, int j, int k) const {
        return (long)(i - lo[0]) + (long)(j - lo[1]) * ext[0] + (long)(k - lo[2]) * ext[0] * ext[1];
    }
    long count() const { return (long)ext[0] * ext[1] * ext[2]; }
};

inline FaceSet make_faces(const Box& b, int a) {
    FaceSet f;
    f.a = a;
    for (int d = 0; d < 3; d++) {
        if (d == a) { f.lo[d] = -1; f.ext[d] = b.n[d] + 3; }
        else { f.lo[d] = 0; f.ext[d] = b.n[d]; }
    }
    return f;
}

// Output side layout (SAMRAI SideData with 0 ghosts): axis a has n_a+1 faces.
inline long side_index(const Box& b, int a, int i, int j, int k) {
    int e0 = b.n[0] + (a == 0 ? 1 : 0);
    int e1 = b.n[1] + (a == 1 ? 1 : 0);
    return (long)i + (long)j * e0 + (long)k * e0 * e1;
}

inline long interior_index(const Box& b, int i, int j, int k) {
    return (long)i + (long)j * b.n[0] + (long)k * b.n[0] * b.n[1];
}

// ---------------------------------------------------------------------------
// WCNS5-JS local interpolation, ConvectiveFluxReconstructorWCNS5-JS-HLLC-HLL.cpp:9-164.
// U[m] is the characteristic variable at cell (face - 3 + m), m = 0..5.
// ---------------------------------------------------------------------------
template <class T>
inline T ipow_(T base, int e) {  // WCNS5-JS-HLLC-HLL.cpp:9-18
    T r = base;
    for (int i = 1; i < e; i++) r *= base;
    return r;
}

template <class T>
inline void js_beta(T& b0, T& b1, T& b2, const T* U) {  // :24-45
    b0 = double(1)/double(3)*(U[0]*(double(4)*U[0] - double(19)*U[1] + double(11)*U[2]) +
         U[1]*(double(25)*U[1] - double(31)*U[2]) + double(10)*U[2]*U[2]);
    b1 = double(1)/double(3)*(U[1]*(double(4)*U[1] - double(13)*U[2] + double(5)*U[3]) +
         double(13)*U[2]*(U[2] - U[3]) + double(4)*U[3]*U[3]);
    b2 = double(1)/double(3)*(U[2]*(double(10)*U[2] - double(31)*U[3] + double(11)*U[4]) +
         U[3]*(double(25)*U[3] - double(19)*U[4]) + double(4)*U[4]*U[4]);
}

template <class T>
inline void js_beta_tilde(T& b0, T& b1, T& b2, const T* U) {  // :51-72
    b0 = double(1)/double(3)*(U[5]*(double(4)*U[5] - double(19)*U[4] + double(11)*U[3]) +
         U[4]*(double(25)*U[4] - double(31)*U[3]) + double(10)*U[3]*U[3]);
    b1 = double(1)/double(3)*(U[4]*(double(4)*U[4] - double(13)*U[3] + double(5)*U[2]) +
         double(13)*U[3]*(U[3] - U[2]) + double(4)*U[2]*U[2]);
    b2 = double(1)/double(3)*(U[3]*(double(10)*U[3] - double(31)*U[2] + double(11)*U[1]) +
         U[2]*(double(25)*U[2] - double(19)*U[1]) + double(4)*U[1]*U[1]);
}

template <class T>
inline T js_minus(const T* U, int p) {  // :78-117
    T b0, b1, b2;
    HMRO_PHASE(HMRO_PH_BETA);
    js_beta(b0, b1, b2, U);
    HMRO_PHASE(HMRO_PH_WEIGHTS);
    T w0 = double(1.0)/double(16)/ipow_(b0 + EPS, p);
    T w1 = double(5.0)/double(8)/ipow_(b1 + EPS, p);
    T w2 = double(5.0)/double(16)/ipow_(b2 + EPS, p);
    T ws = w0 + w1 + w2;
    w0 = w0/ws; w1 = w1/ws; w2 = w2/ws;
    return double(3)/double(8)*w0*U[0] +
        (-double(10)/double(8)*w0 - double(1)/double(8)*w1)*U[1] +
        (double(15)/double(8)*w0 + double(6)/double(8)*w1 + double(3)/double(8)*w2)*U[2] +
        (double(3)/double(8)*w1 + double(6)/double(8)*w2)*U[3] -
        double(1)/double(8)*w2*U[4];
}

template <class T>
inline T js_plus(const T* U, int p) {  // :123-164
    T b0, b1, b2;
    HMRO_PHASE(HMRO_PH_BETA);
    js_beta_tilde(b0, b1, b2, U);
    HMRO_PHASE(HMRO_PH_WEIGHTS);
    T w0 = double(1)/double(16)/ipow_(b0 + EPS, p);
    T w1 = double(5)/double(8)/ipow_(b1 + EPS, p);
    T w2 = double(5)/double(16)/ipow_(b2 + EPS, p);
    T ws = w0 + w1 + w2;
    w0 = w0/ws; w1 = w1/ws; w2 = w2/ws;
    return double(3)/double(8)*w0*U[5] +
        (-double(10)/double(8)*w0 - double(1)/double(8)*w1)*U[4] +
        (double(15)/double(8)*w0 + double(6)/double(8)*w1 + double(3)/double(8)*w2)*U[3] +
        (double(3)/double(8)*w1 + double(6)/double(8)*w2)*U[2] -
        double(1)/double(8)*w2*U[1];
}

// ---------------------------------------------------------------------------
// WCNS6-LD local interpolation, ConvectiveFluxReconstructorWCNS6-LD-HLLC-HLL.cpp:24-319.
// ---------------------------------------------------------------------------
template <class T>
inline T ld_sigma(const T* U) {  // :24-41
    const T a1 = U[2] - U[1];
    const T a2 = U[3] - U[2];
    const T a3 = U[4] - U[3];
    const T t1 = s_fabs(a1 - a2)/(s_fabs(a1) + s_fabs(a2) + EPS);
    const T t2 = s_fabs(a2 - a3)/(s_fabs(a2) + s_fabs(a3) + EPS);
    return s_fmax(t1, t2);
}

template <class T>
inline T ld_beta3(const T* U) {  // :70-83 (6-point smoothness indicator)
    return double(1)/double(232243200)*(U[0]*(double(525910327)*U[0] -
         double(4562164630)*U[1] + double(7799501420)*U[2] -
         double(6610694540)*U[3] + double(2794296070)*U[4] -
         double(472758974)*U[5]) + double(5)*U[1]*
        (double(2146987907)*U[1] - double(7722406988)*U[2] +
         double(6763559276)*U[3] - double(2926461814)*U[4] +
         double(503766638)*U[5]) + double(20)*U[2]*
        (double(1833221603)*U[2] - double(3358664662)*U[3] +
         double(1495974539)*U[4] - double(263126407)*U[5]) +
        double(20)*U[3]*(double(1607794163)*U[3] -
         double(1486026707)*U[4] + double(268747951)*U[5]) +
        double(5)*U[4]*(double(1432381427)*U[4] -
         double(536951582)*U[5]) +
        double(263126407)*U[5]*U[5]);
}

template <class T>
inline T ld_beta3_tilde(const T* U) {  // :119-132
    return double(1)/double(232243200)*(U[5]*(double(525910327)*U[5] -
         double(4562164630)*U[4] + double(7799501420)*U[3] -
         double(6610694540)*U[2] + double(2794296070)*U[1] -
         double(472758974)*U[0]) + double(5)*U[4]*
        (double(2146987907)*U[4] - double(7722406988)*U[3] +
         double(6763559276)*U[2] - double(2926461814)*U[1] +
         double(503766638)*U[0]) + double(20)*U[3]*
        (double(1833221603)*U[3] - double(3358664662)*U[2] +
         double(1495974539)*U[1] - double(263126407)*U[0]) +
        double(20)*U[2]*(double(1607794163)*U[2] -
         double(1486026707)*U[1] + double(268747951)*U[0]) +
        double(5)*U[1]*(double(1432381427)*U[1] -
         double(536951582)*U[0]) +
        double(263126407)*U[0]*U[0]);
}

// Shared weight logic of performLocalWENOInterpolationMinus/Plus (:139-222, :238-319).
// beta[0..3] are beta_k (minus side) or beta_tilde_k (plus side).
template <class T>
inline void ld_weights(T& o0, T& o1, T& o2, T& o3, const T* beta, const T& sigma,
                       int p, int q, double C, double alpha_tau) {
    T tau_5 = s_fabs(beta[0] - beta[2]);
    T u0 = double(1)/double(16)*(double(1) + ipow_(tau_5/(beta[0] + EPS), p));
    T u1 = double(5)/double(8)*(double(1) + ipow_(tau_5/(beta[1] + EPS), p));
    T u2 = double(5)/double(16)*(double(1) + ipow_(tau_5/(beta[2] + EPS), p));
    T us = u0 + u1 + u2;
    u0 = u0/us; u1 = u1/us; u2 = u2/us;

    T beta_avg = double(1)/double(8)*(beta[0] + beta[2] + double(6)*beta[1]);
    T tau_6 = s_fabs(beta[3] - beta_avg);
    o0 = double(1)/double(32)*(C + ipow_(tau_6/(beta[0] + EPS), q));
    o1 = double(15)/double(32)*(C + ipow_(tau_6/(beta[1] + EPS), q));
    o2 = double(15)/double(32)*(C + ipow_(tau_6/(beta[2] + EPS), q));
    o3 = double(1)/double(32)*(C + ipow_(tau_6/(beta[3] + EPS), q));
    T os = o0 + o1 + o2 + o3;
    o0 = o0/os; o1 = o1/os; o2 = o2/os; o3 = o3/os;

    T R_tau = tau_6/(beta_avg + EPS);
    if (s_val(R_tau) > alpha_tau) {
        o0 = sigma*u0 + (double(1) - sigma)*o0;
        o1 = sigma*u1 + (double(1) - sigma)*o1;
        o2 = sigma*u2 + (double(1) - sigma)*o2;
        o3 = (double(1) - sigma)*o3;
    }
}

template <class T>
inline T ld_minus(const T* U, int p, int q, double C, double alpha_tau) {  // :139-222
    HMRO_PHASE(HMRO_PH_WEIGHTS);
    T sigma = ld_sigma(U);
    T beta[4];
    HMRO_PHASE(HMRO_PH_BETA);
    js_beta(beta[0], beta[1], beta[2], U);
    beta[3] = ld_beta3(U);
    HMRO_PHASE(HMRO_PH_WEIGHTS);
    T o0, o1, o2, o3;
    ld_weights(o0, o1, o2, o3, beta, sigma, p, q, C, alpha_tau);
    return double(3)/double(8)*o0*U[0] +
        (-double(10)/double(8)*o0 - double(1)/double(8)*o1)*U[1] +
        (double(15)/double(8)*o0 + double(6)/double(8)*o1 + double(3)/double(8)*o2)*U[2] +
        (double(3)/double(8)*o1 + double(6)/double(8)*o2 + double(15)/double(8)*o3)*U[3] +
        (-double(1)/double(8)*o2 - double(10)/double(8)*o3)*U[4] +
        double(3)/double(8)*o3*U[5];
}

template <class T>
inline T ld_plus(const T* U, int p, int q, double C, double alpha_tau) {  // :238-319
    HMRO_PHASE(HMRO_PH_WEIGHTS);
    T sigma = ld_sigma(U);
    T beta[4];
    HMRO_PHASE(HMRO_PH_BETA);
    js_beta_tilde(beta[0], beta[1], beta[2], U);
    beta[3] = ld_beta3_tilde(U);
    HMRO_PHASE(HMRO_PH_WEIGHTS);
    T o0, o1, o2, o3;
    ld_weights(o0, o1, o2, o3, beta, sigma, p, q, C, alpha_tau);
    return double(3)/double(8)*o0*U[5] +
        (-double(10)/double(8)*o0 - double(1)/double(8)*o1)*U[4] +
        (double(15)/double(8)*o0 + double(6)/double(8)*o1 + double(3)/double(8)*o2)*U[3] +
        (double(3)/double(8)*o1 + double(6)/double(8)*o2 + double(15)/double(8)*o3)*U[2] +
        (-double(1)/double(8)*o2 - double(10)/double(8)*o3)*U[1] +
        double(3)/double(8)*o3*U[0];
}

// ---------------------------------------------------------------------------
// WCNS5-Z local interpolation, ConvectiveFluxReconstructorWCNS5-Z-HLLC-HLL.cpp:78-168:
// the WCNS5-JS indicators and 5-point stencil with the weights
// d_k (1 + (tau_5/(beta_k + eps))^p), tau_5 = |beta_0 - beta_2|.
// ---------------------------------------------------------------------------
template <class T>
inline void z_weights(T& w0, T& w1, T& w2, const T& b0, const T& b1, const T& b2, int p) {
    T tau_5 = s_fabs(b0 - b2);
    w0 = double(1)/double(16)*(double(1) + ipow_(tau_5/(b0 + EPS), p));
    w1 = double(5)/double(8)*(double(1) + ipow_(tau_5/(b1 + EPS), p));
    w2 = double(5)/double(16)*(double(1) + ipow_(tau_5/(b2 + EPS), p));
    T ws = w0 + w1 + w2;
    w0 = w0/ws; w1 = w1/ws; w2 = w2/ws;
}

template <class T>
inline T z_minus(const T* U, int p) {  // :78-120
    T b0, b1, b2, w0, w1, w2;
    HMRO_PHASE(HMRO_PH_BETA);
    js_beta(b0, b1, b2, U);
    HMRO_PHASE(HMRO_PH_WEIGHTS);
    z_weights(w0, w1, w2, b0, b1, b2, p);
    return double(3)/double(8)*w0*U[0] +
        (-double(10)/double(8)*w0 - double(1)/double(8)*w1)*U[1] +
        (double(15)/double(8)*w0 + double(6)/double(8)*w1 +
        double(3)/double(8)*w2)*U[2] +
        (double(3)/double(8)*w1 + double(6)/double(8)*w2)*U[3] -
        double(1)/double(8)*w2*U[4];
}

template <class T>
inline T z_plus(const T* U, int p) {  // :126-168
    T b0, b1, b2, w0, w1, w2;
    HMRO_PHASE(HMRO_PH_BETA);
    js_beta_tilde(b0, b1, b2, U);
    HMRO_PHASE(HMRO_PH_WEIGHTS);
    z_weights(w0, w1, w2, b0, b1, b2, p);
    return double(3)/double(8)*w0*U[5] +
        (-double(10)/double(8)*w0 - double(1)/double(8)*w1)*U[4] +
        (double(15)/double(8)*w0 + double(6)/double(8)*w1 +
        double(3)/double(8)*w2)*U[3] +
        (double(3)/double(8)*w1 + double(6)/double(8)*w2)*U[2] -
        double(1)/double(8)*w2*U[1];
}

// ---------------------------------------------------------------------------
// WCNS6-CU-M2 local interpolation, ConvectiveFluxReconstructorWCNS6-CU-M2-HLLC-HLL.cpp:112-228:
// the WCNS6-LD indicators and 6-point stencil with the weights
//   d_k (C + tau_6/(beta_k + eps dx^2) (beta_avg + Chi dx^2)/(beta_k + Chi dx^2))^q,
// beta_avg = (beta_0 + beta_2 + 6 beta_1)/8, tau_6 = |beta_3 - beta_avg|, and no
// central-upwind switch.  dx is the grid geometry's spacing along the face normal.
// ---------------------------------------------------------------------------
template <class T>
inline void cu_weights(T& o0, T& o1, T& o2, T& o3, const T* beta, int q, double C, double Chi,
                       double epsilon, double dx) {
    T beta_avg = double(1)/double(8)*(beta[0] + beta[2] + double(6)*beta[1]);  // 6*beta_1 in the reference: the same value
    T tau_6 = s_fabs(beta[3] - beta_avg);
    o0 = double(1)/double(32)*ipow_(C + tau_6/(beta[0] + epsilon*dx*dx)*
        (beta_avg + Chi*dx*dx)/(beta[0] + Chi*dx*dx), q);
    o1 = double(15)/double(32)*ipow_(C + tau_6/(beta[1] + epsilon*dx*dx)*
        (beta_avg + Chi*dx*dx)/(beta[1] + Chi*dx*dx), q);
    o2 = double(15)/double(32)*ipow_(C + tau_6/(beta[2] + epsilon*dx*dx)*
        (beta_avg + Chi*dx*dx)/(beta[2] + Chi*dx*dx), q);
    o3 = double(1)/double(32)*ipow_(C + tau_6/(beta[3] + epsilon*dx*dx)*
        (beta_avg + Chi*dx*dx)/(beta[3] + Chi*dx*dx), q);
    T os = o0 + o1 + o2 + o3;
    o0 = o0/os; o1 = o1/os; o2 = o2/os; o3 = o3/os;
}

template <class T>
inline T cu_minus(const T* U, int q, double C, double Chi, double epsilon, double dx) {  // :112-167
    T beta[4];
    HMRO_PHASE(HMRO_PH_BETA);
    js_beta(beta[0], beta[1], beta[2], U);
    beta[3] = ld_beta3(U);
    HMRO_PHASE(HMRO_PH_WEIGHTS);
    T o0, o1, o2, o3;
    cu_weights(o0, o1, o2, o3, beta, q, C, Chi, epsilon, dx);
    return double(3)/double(8)*o0*U[0] +
        (-double(10)/double(8)*o0 - double(1)/double(8)*o1)*U[1] +
        (double(15)/double(8)*o0 + double(6)/double(8)*o1 + double(3)/double(8)*o2)*U[2] +
        (double(3)/double(8)*o1 + double(6)/double(8)*o2 + double(15)/double(8)*o3)*U[3] +
        (-double(1)/double(8)*o2 - double(10)/double(8)*o3)*U[4] +
        double(3)/double(8)*o3*U[5];
}

template <class T>
inline T cu_plus(const T* U, int q, double C, double Chi, double epsilon, double dx) {  // :173-228
    T beta[4];
    HMRO_PHASE(HMRO_PH_BETA);
    js_beta_tilde(beta[0], beta[1], beta[2], U);
    beta[3] = ld_beta3_tilde(U);
    HMRO_PHASE(HMRO_PH_WEIGHTS);
    T o0, o1, o2, o3;
    cu_weights(o0, o1, o2, o3, beta, q, C, Chi, epsilon, dx);
    return double(3)/double(8)*o0*U[5] +
        (-double(10)/double(8)*o0 - double(1)/double(8)*o1)*U[4] +
        (double(15)/double(8)*o0 + double(6)/double(8)*o1 + double(3)/double(8)*o2)*U[3] +
        (double(3)/double(8)*o1 + double(6)/double(8)*o2 + double(15)/double(8)*o3)*U[2] +
        (-double(1)/double(8)*o2 - double(10)/double(8)*o3)*U[1] +
        double(3)/double(8)*o3*U[0];
}

}  // namespace hmro

namespace hmro {

// ---------------------------------------------------------------------------
// Mixture ratio of specific heats from volume fractions (ideal gas, isobaric).
// All N fractions given (cell data):        EquationOfStateMixingRulesIdealGas.cpp:7404-7598
//   xi = 0; xi += Z_i * (1/(gamma_i - 1)); gamma = 1/xi + 1
// N-1 fractions given (side data in the Riemann drivers): :7599-7800
//   xi = 0; xi += Z_i * (1/(gamma_i - 1)), i < N-1; Z_last = 1 - sum Z_i;
//   xi += Z_last/(gamma_N - 1); gamma = 1/xi + 1
// ---------------------------------------------------------------------------
template <class T>
inline T gamma_mix_all(const Config& c, const T* Z) {
    T xi = T(0.0);
    for (int si = 0; si < c.num_species; si++) {
        const double one_over_denominator = double(1)/(c.gamma[si] - double(1));
        xi += Z[si]*one_over_denominator;
    }
    return double(1)/xi + double(1);
}

template <class T>
inline T gamma_mix_last(const Config& c, const T* Z /* N-1 */) {
    T xi = T(0.0);
    T Z_last = T(1.0);
    for (int si = 0; si < c.num_species - 1; si++) {
        const double one_over_denominator = double(1)/(c.gamma[si] - double(1));
        xi += Z[si]*one_over_denominator;
        Z_last -= Z[si];
    }
    xi += Z_last/(c.gamma[c.num_species - 1] - double(1));
    return double(1)/xi + double(1);
}

// Four-equation (conservative) model, ideal-gas mixture with mass fractions,
// EquationOfStateMixingRulesIdealGas.cpp:4677-5143 (c_p, c_v weighted by Y,
// gamma = c_p/c_v), species c_p = gamma/(gamma-1)*R, c_v = 1/(gamma-1)*R
// (:113-119), and the partial-density derivative of pressure
// Psi_i = ((c_p,i - gamma c_v,i)/c_v + gamma - 1) eps, eps = p/((gamma-1) rho)
// (:3102-3157, array form :6367-6420).
inline double species_cp(const Config& c, int s) { return c.gamma[s]/(c.gamma[s] - double(1))*c.R[s]; }
inline double species_cv(const Config& c, int s) { return double(1)/(c.gamma[s] - double(1))*c.R[s]; }

template <class T>
inline void mix_mass(const Config& c, const T* Y, T& gamma, T& cv) {
    T cp = T(0.0);
    cv = T(0.0);
    for (int si = 0; si < c.num_species; si++) {
        cp += Y[si]*species_cp(c, si);
        cv += Y[si]*species_cv(c, si);
    }
    gamma = cp/cv;
}

// Sound speed of the four-equation model from rho, p and the mass fractions.
template <class T>
inline T four_sound_speed(const Config& c, const T& rho, const T& p, const T* Y) {
    T gamma, cv;
    mix_mass(c, Y, gamma, cv);
    const T Gamma = gamma - double(1);
    const T eps = p/((gamma - double(1))*rho);
    T c2 = Gamma*p/rho;
    for (int si = 0; si < c.num_species; si++) {
        const T Psi = ((species_cp(c, si) - gamma*species_cv(c, si))/cv + gamma - double(1))*eps;
        c2 += Y[si]*Psi;
    }
    return s_sqrt(c2);
}

// Face thermodynamics used by the Riemann drivers (density, sound speed,
// specific internal energy of one reconstructed state V).
//  single: EquationOfStateIdealGas.cpp:5806 (c = sqrt(gamma*p/rho)), :6135 (eps = p/((gamma-1)*rho))
//  five:   FlowModelRiemannSolverFiveEqnAllaireHLLC.cpp:4824-6097 (2D block): rho = sum Z_rho,
//          Y = Z_rho/rho, Gamma = gamma-1, c^2 = Gamma*p/rho + sum Y*(p/rho), eps = p/((gamma-1)*rho)
template <class T>
inline void face_thermo(const Config& c, const T* V, T& rho, T& cs, T& eps) {
    const int dim = c.dim;
    if (c.model == MODEL_SINGLE_SPECIES) {
        const double gamma = c.gamma[0];
        rho = V[0];
        const T& p = V[dim + 1];
        cs = s_sqrt(gamma*p/rho);
        eps = p/((gamma - double(1))*rho);
    } else if (c.model == MODEL_FOUR_EQN_CONSERVATIVE) {
        // FlowModelRiemannSolverFourEqnConservativeHLLC-HLL.cpp:5013-6180 (2D block)
        const int N = c.num_species;
        rho = T(0.0);
        for (int si = 0; si < N; si++) rho += V[si];
        const T& p = V[N + dim];
        T Y[8];
        for (int si = 0; si < N; si++) Y[si] = V[si]/rho;
        cs = four_sound_speed(c, rho, p, Y);
        T gamma, cv;
        mix_mass(c, Y, gamma, cv);
        eps = p/((gamma - double(1))*rho);
    } else {
        const int N = c.num_species;
        rho = T(0.0);
        for (int si = 0; si < N; si++) rho += V[si];
        const T& p = V[N + dim];
        T Y[8];
        for (int si = 0; si < N; si++) Y[si] = V[si]/rho;
        const T gamma = gamma_mix_last(c, V + N + dim + 1);
        const T Gamma = gamma - double(1);
        const T Psi = p/rho;
        T c2 = Gamma*p/rho;
        for (int si = 0; si < N; si++) c2 += Y[si]*Psi;
        cs = s_sqrt(c2);
        const T gamma_e = gamma_mix_last(c, V + N + dim + 1);
        eps = p/((gamma_e - double(1))*rho);
    }
}

// Bounds check of a reconstructed face state.
//  single: FlowModelBasicUtilitiesSingleSpecies.cpp:3013-3440 (rho > 0 and p > 0)
//  five:   FlowModelBasicUtilitiesFiveEqnAllaire.cpp:5446-7347 with the bounds of
//          FlowModelBasicUtilitiesFiveEqnAllaire.hpp:24-27 (Y in (-0.001, 1.001),
//          Z in (-1000, 1000)), partial densities > 0 and c^2 > 0.
template <class T>
inline int face_bounded(const Config& c, const T* V) {
    const int dim = c.dim;
    int ok = 1;
    if (c.model == MODEL_SINGLE_SPECIES) {
        ok &= (s_val(V[0]) > 0.0) ? 1 : 0;
        ok &= (s_val(V[dim + 1]) > 0.0) ? 1 : 0;
        return ok;
    }
    if (c.model == MODEL_FOUR_EQN_CONSERVATIVE) {
        // FlowModelBasicUtilitiesFourEqnConservative.cpp:3737-4540, bounds
        // FlowModelBasicUtilitiesFourEqnConservative.hpp:24-25: Y in (-0.001, 1.001), rho > 0, p > 0.
        const int N = c.num_species;
        T rho = T(0.0);
        for (int si = 0; si < N; si++) rho += V[si];
        for (int si = 0; si < N; si++) {
            const T Y = V[si]/rho;
            ok &= (s_val(Y) > -0.001 && s_val(Y) < 1.001) ? 1 : 0;
        }
        ok &= (s_val(rho) > 0.0) ? 1 : 0;
        ok &= (s_val(V[N + dim]) > 0.0) ? 1 : 0;
        return ok;
    }
    const int N = c.num_species;
    const double Y_lo = -0.001, Y_up = 1.001, Z_lo = -1000.0, Z_up = 1000.0;
    T Z[8];
    Z[N - 1] = T(1.0);
    for (int si = 0; si < N - 1; si++) {
        Z[si] = V[N + dim + 1 + si];
        Z[N - 1] -= Z[si];
        ok &= (s_val(Z[si]) > Z_lo && s_val(Z[si]) < Z_up) ? 1 : 0;
    }
    ok &= (s_val(Z[N - 1]) > Z_lo && s_val(Z[N - 1]) < Z_up) ? 1 : 0;
    T rho = T(0.0);
    for (int si = 0; si < N; si++) rho += V[si];
    T Y[8];
    for (int si = 0; si < N; si++) {
        Y[si] = V[si]/rho;
        ok &= (s_val(Y[si]) > Y_lo && s_val(Y[si]) < Y_up) ? 1 : 0;
    }
    for (int si = 0; si < N; si++) ok &= (s_val(V[si]) > 0.0) ? 1 : 0;
    const T& p = V[N + dim];
    const T gamma = gamma_mix_all(c, Z);
    const T Gamma = gamma - double(1);
    const T Psi = p/rho;
    T c2 = Gamma*p/rho;
    for (int si = 0; si < N; si++) c2 += Y[si]*Psi;
    ok &= (s_val(c2) > 0.0) ? 1 : 0;
    return ok;
}

// Conserved state, physical flux of one face state (direction a) in the
// component order of the model.
//  single: FlowModelRiemannSolverSingleSpeciesHLLC-HLL.cpp:889-1027 (2D x), :1183 (2D y), :1030 (3D x)
//  five:   FlowModelRiemannSolverFiveEqnAllaireHLLC-HLL.cpp:1283-1503 (2D x) and siblings
template <class T>
inline void face_QF(const Config& c, int a, const T* V, const T& rho, const T& eps, T* Q, T* F) {
    const int dim = c.dim;
    if (c.model == MODEL_SINGLE_SPECIES) {
        const T& p = V[dim + 1];
        Q[0] = V[0];
        for (int k = 0; k < dim; k++) Q[1 + k] = V[0]*V[1 + k];
        T ke = V[1]*V[1];
        for (int k = 1; k < dim; k++) ke = ke + V[1 + k]*V[1 + k];
        Q[dim + 1] = V[0]*(eps + double(1)/double(2)*ke);
        const T& un = V[1 + a];
        F[0] = Q[1 + a];
        for (int k = 0; k < dim; k++) {
            if (k == a) F[1 + k] = Q[1 + a]*V[1 + k] + p;
            else F[1 + k] = Q[1 + a]*V[1 + k];
        }
        F[dim + 1] = un*(Q[dim + 1] + p);
        return;
    }
    const int N = c.num_species;
    const T& p = V[N + dim];
    const T& un = V[N + a];
    for (int si = 0; si < N; si++) Q[si] = V[si];
    for (int k = 0; k < dim; k++) Q[N + k] = rho*V[N + k];
    T ke = V[N]*V[N];
    for (int k = 1; k < dim; k++) ke = ke + V[N + k]*V[N + k];
    Q[N + dim] = rho*(eps + double(1)/double(2)*ke);
    for (int si = 0; si < num_vf(c); si++) Q[N + dim + 1 + si] = V[N + dim + 1 + si];
    for (int si = 0; si < N; si++) F[si] = un*V[si];
    for (int k = 0; k < dim; k++) {
        if (k == a) F[N + k] = un*Q[N + k] + p;
        else F[N + k] = un*Q[N + k];
    }
    F[N + dim] = un*(Q[N + dim] + p);
    for (int si = 0; si < num_vf(c); si++) F[N + dim + 1 + si] = un*V[N + dim + 1 + si];
}

// Is component e advected with the HLL flux inside HLLC-HLL (mass/partial
// densities, transverse momenta, volume fractions)?
inline bool hll_component(const Config& c, int a, int e) {
    const int dim = c.dim;
    if (c.model == MODEL_SINGLE_SPECIES) {
        if (e == 0) return true;
        if (e >= 1 && e <= dim) return (e - 1) != a;
        return false;
    }
    const int N = c.num_species;
    if (e < N) return true;
    if (e < N + dim) return (e - N) != a;
    if (e == N + dim) return false;
    return true;
}

// HLLC and HLLC-HLL midpoint fluxes of one face, plus the HLLC midpoint
// normal velocity (FlowModelRiemannSolverFiveEqnAllaireHLLC.cpp:2084-2088 /
// single-species HLLC.cpp:3060-3070 pattern).
template <class T>
inline void riemann_face(const Config& c, int a, const T* VL, const T* VR,
                         T* F_hllc, T* F_hllc_hll, T& u_mid, bool need_hll = true) {
    const int dim = c.dim;
    const int neq = num_eqn(c);
    const int ip = (c.model == MODEL_SINGLE_SPECIES) ? dim + 1 : c.num_species + dim;
    const int iu = (c.model == MODEL_SINGLE_SPECIES) ? 1 : c.num_species;
    T rhoL, cL, epsL, rhoR, cR, epsR;
    face_thermo(c, VL, rhoL, cL, epsL);
    face_thermo(c, VR, rhoR, cR, epsR);
    const T& uL = VL[iu + a];
    const T& uR = VR[iu + a];
    const T& pL = VL[ip];
    const T& pR = VR[ip];

    const T u_average = double(1)/double(2)*(uL + uR);
    const T c_average = double(1)/double(2)*(cL + cR);
    const T s_L = s_fmin(u_average - c_average, uL - cL);
    const T s_R = s_fmax(u_average + c_average, uR + cR);
    const T s_minus = s_fmin(T(0.0), s_L);
    const T s_plus = s_fmax(T(0.0), s_R);
    const T s_star = (pR - pL + rhoL*uL*(s_L - uL) - rhoR*uR*(s_R - uR))/
        (rhoL*(s_L - uL) - rhoR*(s_R - uR));

    T QL[16], QR[16], FL[16], FR[16], Qs[16];
    face_QF(c, a, VL, rhoL, epsL, QL, FL);
    face_QF(c, a, VR, rhoR, epsR, QR, FR);

    // HLL part (HLLC-HLL only): HLLC-HLL.cpp:949-970
    T F_hll[16];
    for (int e = 0; e < neq && need_hll; e++) {
        if (!hll_component(c, a, e)) continue;
        F_hll[e] = (s_R*FL[e] - s_L*FR[e] + s_R*s_L*(QR[e] - QL[e]))/(s_R - s_L);
        if (s_val(s_L) > 0.0) F_hll[e] = FL[e];
    }
    if (need_hll && s_val(s_R) < 0.0) {
        for (int e = 0; e < neq; e++) if (hll_component(c, a, e)) F_hll[e] = FR[e];
    }

    // HLLC star state: HLLC.cpp:636-691
    const bool left = s_val(s_star) > 0.0;
    const T* VK = left ? VL : VR;
    const T* QK = left ? QL : QR;
    const T* FK = left ? FL : FR;
    const T& rhoK = left ? rhoL : rhoR;
    const T& sK = left ? s_L : s_R;
    const T& uK = left ? uL : uR;
    const T& pK = left ? pL : pR;
    const T& s_pm = left ? s_minus : s_plus;
    const T Chi = (sK - uK)/(sK - s_star);
    if (c.model == MODEL_SINGLE_SPECIES) {
        Qs[0] = Chi*VK[0];
        for (int k = 0; k < dim; k++) {
            if (k == a) Qs[1 + k] = Chi*VK[0]*s_star;
            else Qs[1 + k] = Chi*QK[1 + k];
        }
        Qs[dim + 1] = Chi*(QK[dim + 1] + (s_star - uK)*(VK[0]*s_star + pK/(sK - uK)));
    } else {
        const int N = c.num_species;
        for (int si = 0; si < N; si++) Qs[si] = Chi*VK[si];
        for (int k = 0; k < dim; k++) {
            if (k == a) Qs[N + k] = Chi*rhoK*s_star;
            else Qs[N + k] = Chi*QK[N + k];
        }
        Qs[N + dim] = Chi*(QK[N + dim] + (s_star - uK)*(rhoK*s_star + pK/(sK - uK)));
        for (int si = 0; si < num_vf(c); si++) Qs[N + dim + 1 + si] = Chi*VK[N + dim + 1 + si];
    }
    for (int e = 0; e < neq; e++) F_hllc[e] = FK[e] + s_pm*(Qs[e] - QK[e]);
    u_mid = uK + s_pm*(Chi - double(1));

    if (!need_hll) {
        for (int e = 0; e < neq; e++) F_hllc_hll[e] = F_hllc[e];
        return;
    }
    // Hybridization weights: HLLC-HLL.cpp:998-1026
    T diff[3];
    for (int k = 0; k < dim; k++) diff[k] = VR[iu + k] - VL[iu + k];
    T vsq = diff[0]*diff[0];
    for (int k = 1; k < dim; k++) vsq = vsq + diff[k]*diff[k];
    const T vel_mag = s_sqrt(vsq);
    T alpha_1, alpha_2;
    if (s_val(vel_mag) < EPS) {
        alpha_1 = T(1.0);
        alpha_2 = T(0.0);
    } else {
        alpha_1 = s_fabs(diff[a])/vel_mag;
        alpha_2 = s_sqrt(double(1) - alpha_1*alpha_1);
    }
    const T beta_1 = double(1)/double(2)*(double(1) + alpha_1/(alpha_1 + alpha_2));
    const T beta_2 = double(1) - beta_1;
    for (int e = 0; e < neq; e++) {
        if (hll_component(c, a, e)) F_hllc_hll[e] = beta_1*F_hllc[e] + beta_2*F_hll[e];
        else F_hllc_hll[e] = F_hllc[e];
    }
}

// Characteristic projection of primitive variables at one face and offset.
//  single: FlowModelBasicUtilitiesSingleSpecies.cpp:5882-6451 (2D x :6135-6165, y :6167-6205)
//  five:   FlowModelBasicUtilitiesFiveEqnAllaire.cpp:8232-9178 (2D block)
// proj = {rho_bar, c_bar} (single) or {Zrho_bar_0..N-1, rho_bar, c_bar} (five).
template <class T>
inline void char_from_prim(const Config& c, int a, const T* proj, const T* V, T* W) {
    const int dim = c.dim;
    if (c.model == MODEL_SINGLE_SPECIES) {
        const T& rb = proj[0];
        const T& cb = proj[1];
        const T& un = V[1 + a];
        const T& p = V[dim + 1];
        W[0] = -double(1)/double(2)*rb*cb*un + double(1)/double(2)*p;
        W[1] = V[0] - double(1)/(cb*cb)*p;
        int t = 2;
        for (int k = 0; k < dim; k++) if (k != a) W[t++] = V[1 + k];
        W[dim + 1] = double(1)/double(2)*rb*cb*un + double(1)/double(2)*p;
        return;
    }
    const int N = c.num_species;
    const T& rb = proj[N];
    const T& cb = proj[N + 1];
    const T& un = V[N + a];
    const T& p = V[N + dim];
    for (int si = 0; si < N; si++) {
        W[1 + si] = V[si] - proj[si]/(rb*cb*cb)*p;
    }
    for (int si = 0; si < num_vf(c); si++) W[N + dim + si] = V[N + dim + 1 + si];
    W[0] = un - double(1)/(rb*cb)*p;
    int t = N + 1;
    for (int k = 0; k < dim; k++) if (k != a) W[t++] = V[N + k];
    W[num_eqn(c) - 1] = un + double(1)/(rb*cb)*p;
}

//  single: FlowModelBasicUtilitiesSingleSpecies.cpp:7023-7474 (2D :7279-7330)
//  five:   FlowModelBasicUtilitiesFiveEqnAllaire.cpp:9201-… (2D block)
template <class T>
inline void prim_from_char(const Config& c, int a, const T* proj, const T* W, T* V) {
    const int dim = c.dim;
    if (c.model == MODEL_SINGLE_SPECIES) {
        const T& rb = proj[0];
        const T& cb = proj[1];
        const int last = dim + 1;
        V[0] = double(1)/(cb*cb)*W[0] + W[1] + double(1)/(cb*cb)*W[last];
        int t = 2;
        for (int k = 0; k < dim; k++) {
            if (k == a) V[1 + k] = -double(1)/(rb*cb)*W[0] + double(1)/(rb*cb)*W[last];
            else V[1 + k] = W[t++];
        }
        V[dim + 1] = W[0] + W[last];
        return;
    }
    const int N = c.num_species;
    const int last = num_eqn(c) - 1;
    const T& rb = proj[N];
    const T& cb = proj[N + 1];
    for (int si = 0; si < N; si++) {
        V[si] = -double(1)/double(2)*proj[si]/cb*W[0] + W[si + 1] +
            double(1)/double(2)*proj[si]/cb*W[last];
    }
    for (int si = 0; si < num_vf(c); si++) V[N + dim + 1 + si] = W[N + dim + si];
    int t = N + 1;
    for (int k = 0; k < dim; k++) {
        if (k == a) V[N + k] = double(1)/double(2)*W[0] + double(1)/double(2)*W[last];
        else V[N + k] = W[t++];
    }
    V[N + dim] = -double(1)/double(2)*rb*cb*W[0] + double(1)/double(2)*rb*cb*W[last];
}

}  // namespace hmro

namespace hmro {

// ---------------------------------------------------------------------------
// Derived cell data on the whole ghost box (FlowModel::computeDerivedCellData).
//  single: FlowModelSingleSpecies.cpp:1240-1390 -> velocity :2649, internal energy :2849,
//          pressure :3074 (EquationOfStateIdealGas.cpp:5477), sound speed :3127 (:5806),
//          convective flux :3233-3884.
//  five:   FlowModelFiveEqnAllaire.cpp:1267-1450 -> density (EquationOfStateMixingRules.cpp:735-871),
//          mass fractions :3772, velocity :3989, internal energy :4214, pressure :4454,
//          sound speed :4512-4877, convective flux :4877-5902.
// V holds the primitive variables (FlowModel*::getCellDataOfPrimitiveVariables),
// Fn the node fluxes per direction, vel the velocity field.
// ---------------------------------------------------------------------------
template <class T>
struct Derived {
    std::vector<T> V;        // neq x ncell
    std::vector<T> rho;      // mixture density (five) / density (single)
    std::vector<T> cs;       // sound speed
    std::vector<T> Fn;       // dim x neq x ncell
    long ncell;
};

template <class T>
void compute_derived(const Config& c, const Box& b, const T* const* Q, Derived<T>& D) {
    const int dim = c.dim;
    const int neq = num_eqn(c);
    const long nc = b.ncell();
    D.ncell = nc;
    D.V.assign((size_t)neq * nc, T(0.0));
    D.rho.assign(nc, T(0.0));
    D.cs.assign(nc, T(0.0));
    D.Fn.assign((size_t)dim * neq * nc, T(0.0));
    for (long x = 0; x < nc; x++) {
        if (c.model == MODEL_SINGLE_SPECIES) {
            const double gamma = c.gamma[0];
            const T& rho = Q[0][x];
            T u[3];
            for (int k = 0; k < dim; k++) u[k] = Q[1 + k][x]/rho;
            const T& E = Q[dim + 1][x];
            T ke = u[0]*u[0];
            for (int k = 1; k < dim; k++) ke = ke + u[k]*u[k];
            const T eps = E/rho - double(1)/double(2)*ke;
            const T p = (gamma - double(1))*rho*eps;
            const T cs = s_sqrt(gamma*p/rho);
            D.rho[x] = rho;
            D.cs[x] = cs;
            D.V[x] = rho;
            for (int k = 0; k < dim; k++) D.V[(size_t)(1 + k) * nc + x] = u[k];
            D.V[(size_t)(dim + 1) * nc + x] = p;
            for (int a = 0; a < dim; a++) {
                T* F = &D.Fn[(size_t)a * neq * nc];
                F[x] = Q[1 + a][x];
                for (int k = 0; k < dim; k++) {
                    if (k == a) F[(size_t)(1 + k) * nc + x] = u[a]*Q[1 + k][x] + p;
                    else F[(size_t)(1 + k) * nc + x] = u[a]*Q[1 + k][x];
                }
                F[(size_t)(dim + 1) * nc + x] = u[a]*(E + p);
            }
        } else if (c.model == MODEL_FOUR_EQN_CONSERVATIVE) {
            // FlowModelFourEqnConservative.cpp:3877-5499: density, mass fractions,
            // velocity, internal energy, pressure (mass-fraction mixture), sound speed.
            const int N = c.num_species;
            T rho = T(0.0);
            for (int si = 0; si < N; si++) rho += Q[si][x];
            T Y[8];
            for (int si = 0; si < N; si++) Y[si] = Q[si][x]/rho;
            T u[3];
            for (int k = 0; k < dim; k++) u[k] = Q[N + k][x]/rho;
            const T& E = Q[N + dim][x];
            T ke = u[0]*u[0];
            for (int k = 1; k < dim; k++) ke = ke + u[k]*u[k];
            const T eps = E/rho - double(1)/double(2)*ke;
            T gamma, cv;
            mix_mass(c, Y, gamma, cv);
            const T p = (gamma - double(1))*rho*eps;
            const T cs = four_sound_speed(c, rho, p, Y);
            D.rho[x] = rho;
            D.cs[x] = cs;
            for (int si = 0; si < N; si++) D.V[(size_t)si * nc + x] = Q[si][x];
            for (int k = 0; k < dim; k++) D.V[(size_t)(N + k) * nc + x] = u[k];
            D.V[(size_t)(N + dim) * nc + x] = p;
            for (int a = 0; a < dim; a++) {
                T* F = &D.Fn[(size_t)a * neq * nc];
                for (int si = 0; si < N; si++) F[(size_t)si * nc + x] = u[a]*Q[si][x];
                for (int k = 0; k < dim; k++) {
                    if (k == a) F[(size_t)(N + k) * nc + x] = u[a]*Q[N + k][x] + p;
                    else F[(size_t)(N + k) * nc + x] = u[a]*Q[N + k][x];
                }
                F[(size_t)(N + dim) * nc + x] = u[a]*(E + p);
            }
        } else {
            const int N = c.num_species;
            T rho = T(0.0);
            for (int si = 0; si < N; si++) rho += Q[si][x];
            T Y[8];
            for (int si = 0; si < N; si++) Y[si] = Q[si][x]/rho;
            T u[3];
            for (int k = 0; k < dim; k++) u[k] = Q[N + k][x]/rho;
            const T& E = Q[N + dim][x];
            T ke = u[0]*u[0];
            for (int k = 1; k < dim; k++) ke = ke + u[k]*u[k];
            const T eps = E/rho - double(1)/double(2)*ke;
            T Z[8];
            for (int si = 0; si < N; si++) Z[si] = Q[N + dim + 1 + si][x];
            const T gamma = gamma_mix_all(c, Z);
            const T p = (gamma - double(1))*rho*eps;
            const T gamma_g = gamma_mix_all(c, Z);
            const T Gamma = gamma_g - double(1);
            const T Psi = p/rho;
            T c2 = Gamma*p/rho;
            for (int si = 0; si < N; si++) c2 += Y[si]*Psi;
            const T cs = s_sqrt(c2);
            D.rho[x] = rho;
            D.cs[x] = cs;
            for (int si = 0; si < N; si++) D.V[(size_t)si * nc + x] = Q[si][x];
            for (int k = 0; k < dim; k++) D.V[(size_t)(N + k) * nc + x] = u[k];
            D.V[(size_t)(N + dim) * nc + x] = p;
            for (int si = 0; si < N - 1; si++) D.V[(size_t)(N + dim + 1 + si) * nc + x] = Z[si];
            for (int a = 0; a < dim; a++) {
                T* F = &D.Fn[(size_t)a * neq * nc];
                for (int si = 0; si < N; si++) F[(size_t)si * nc + x] = u[a]*Q[si][x];
                for (int k = 0; k < dim; k++) {
                    if (k == a) F[(size_t)(N + k) * nc + x] = u[a]*Q[N + k][x] + p;
                    else F[(size_t)(N + k) * nc + x] = u[a]*Q[N + k][x];
                }
                F[(size_t)(N + dim) * nc + x] = u[a]*(E + p);
                for (int si = 0; si < N - 1; si++)
                    F[(size_t)(N + dim + 1 + si) * nc + x] = u[a]*Z[si];
            }
        }
    }
}

// Velocity component index inside V.
inline int vel_index(const Config& c) { return c.model == MODEL_SINGLE_SPECIES ? 1 : c.num_species; }

// When set, the HLL part of HLLC-HLL is evaluated only on faces whose sensor
// selects it (the results are unchanged; used by the operation counter).
inline bool g_minimal_hll = false;

// Per-face counters reported back to the caller.
struct Stats {
    long faces;          // midpoint faces reconstructed
    long fallback;       // faces that reverted to first order (bounds check failed)
    long hllc_hll;       // faces where the shock sensor selected HLLC-HLL
};

// ---------------------------------------------------------------------------
// One patch: convective flux (times dt) on all interior faces and the
// advective source (accumulated), i.e. computeConvectiveFluxAndSourceOnPatch,
// WCNS56-HLLC-HLL.cpp:544-1376 (2D) / :1378-2655 (3D).
//   Q      : num_comp(c) arrays over the ghost box (ghost width 4)
//   flux   : dim*neq arrays, axis-major, SAMRAI side layout with 0 ghosts
//   source : neq arrays over the interior (accumulated, +=)
// ---------------------------------------------------------------------------
template <class T>
void conv_flux_source(const Config& c, const int* n, const double* dx, double dt,
                      const T* const* Q, T* const* flux, T* const* source, Stats* stats) {
    const int dim = c.dim;
    const int neq = num_eqn(c);
    const Box b = make_box(dim, n, c.ghosts);
    const long nc = b.ncell();
    Derived<T> D;
    HMRO_PHASE(HMRO_PH_CELLS);
    compute_derived(c, b, Q, D);
    HMRO_PHASE(HMRO_PH_SENSOR);
    const int iu = vel_index(c);
    const bool five = (c.model == MODEL_FIVE_EQN_ALLAIRE);
    const bool multi = (c.model != MODEL_SINGLE_SPECIES);
    const int N = c.num_species;

    // Velocity derivatives, dilatation and vorticity magnitude on the
    // interior grown by 2 (WCNS56-HLLC-HLL.cpp:638-731, 3D :1440-1660);
    // DerivativeFirstOrder.cpp:229 (2nd order: (1/2*(u_R - u_L))/dx).
    std::vector<T> theta(nc, T(0.0)), Omega(nc, T(0.0));
    {
        const int lo2 = (dim == 3) ? -2 : 0, hi2 = (dim == 3) ? b.n[2] + 2 : 1;
        for (int k = lo2; k < hi2; k++)
        for (int j = -2; j < b.n[1] + 2; j++)
        for (int i = -2; i < b.n[0] + 2; i++) {
            const long x = b.cell(i, j, k);
            T du[3][3];  // du[comp][axis]
            for (int comp = 0; comp < dim; comp++) {
                const T* u = &D.V[(size_t)(iu + comp) * nc];
                du[comp][0] = (double(1)/double(2)*(u[b.cell(i + 1, j, k)] - u[b.cell(i - 1, j, k)]))/dx[0];
                du[comp][1] = (double(1)/double(2)*(u[b.cell(i, j + 1, k)] - u[b.cell(i, j - 1, k)]))/dx[1];
                if (dim == 3)
                    du[comp][2] = (double(1)/double(2)*(u[b.cell(i, j, k + 1)] - u[b.cell(i, j, k - 1)]))/dx[2];
            }
            if (dim == 2) {
                theta[x] = du[0][0] + du[1][1];
                Omega[x] = s_fabs(du[1][0] - du[0][1]);
            } else {
                theta[x] = du[0][0] + du[1][1] + du[2][2];
                const T omega_x = du[2][1] - du[1][2];
                const T omega_y = du[0][2] - du[2][0];
                const T omega_z = du[1][0] - du[0][1];
                Omega[x] = s_sqrt(omega_x*omega_x + omega_y*omega_y + omega_z*omega_z);
            }
        }
    }

    // Midpoint fluxes and (five-eqn) midpoint normal velocity per direction.
    std::vector<std::vector<T>> Fmid(dim), umid(dim);
    std::vector<FaceSet> FS(dim);
    long cnt_faces = 0, cnt_fallback = 0, cnt_hll = 0;
    const int nproj = multi ? N + 2 : 2;

    for (int a = 0; a < dim; a++) {
        const FaceSet fs = make_faces(b, a);
        FS[a] = fs;
        const long nf = fs.count();
        std::vector<T> proj((size_t)nproj * nf);
        std::vector<T> W((size_t)6 * neq * nf);
        std::vector<T> Wm((size_t)neq * nf), Wp((size_t)neq * nf);
        std::vector<T> Vm((size_t)neq * nf), Vp((size_t)neq * nf);
        std::vector<int> flag_m(nf, 1), flag_p(nf, 1);
        std::vector<T> F_hllc((size_t)neq * nf), F_hh((size_t)neq * nf);
        std::vector<T> s_face(nf);
        Fmid[a].assign((size_t)neq * nf, T(0.0));
        umid[a].assign(nf, T(0.0));
        const int off[3] = {a == 0, a == 1, a == 2};

        HMRO_PHASE(HMRO_PH_PROJ);
        // Projection variables (SIMPLE averaging).
        //  single: FlowModelBasicUtilitiesSingleSpecies.cpp:4638-5134
        //  five:   FlowModelBasicUtilitiesFiveEqnAllaire.cpp:7474-8207
        for (int k = fs.lo[2]; k < fs.lo[2] + fs.ext[2]; k++)
        for (int j = fs.lo[1]; j < fs.lo[1] + fs.ext[1]; j++)
        for (int i = fs.lo[0]; i < fs.lo[0] + fs.ext[0]; i++) {
            const long f = fs.idx(i, j, k);
            const long xL = b.cell(i - off[0], j - off[1], k - off[2]);
            const long xR = b.cell(i, j, k);
            if (multi) {
                // five: FlowModelBasicUtilitiesFiveEqnAllaire.cpp:7474; four:
                // FlowModelBasicUtilitiesFourEqnConservative.cpp:4638 (same means)
                for (int si = 0; si < N; si++)
                    proj[(size_t)si * nf + f] = double(1)/double(2)*(Q[si][xL] + Q[si][xR]);
                proj[(size_t)N * nf + f] = double(1)/double(2)*(D.rho[xL] + D.rho[xR]);
                proj[(size_t)(N + 1) * nf + f] = double(1)/double(2)*(D.cs[xL] + D.cs[xR]);
            } else {
                proj[f] = double(1)/double(2)*(D.rho[xL] + D.rho[xR]);
                proj[nf + f] = double(1)/double(2)*(D.cs[xL] + D.cs[xR]);
            }
        }

        HMRO_PHASE(HMRO_PH_CHAR);
        // Characteristic variables for the six offsets m-3, m = 0..5
        // (WCNS56-HLLC-HLL.cpp:886-893).
        for (int m = 0; m < 6; m++)
        for (int k = fs.lo[2]; k < fs.lo[2] + fs.ext[2]; k++)
        for (int j = fs.lo[1]; j < fs.lo[1] + fs.ext[1]; j++)
        for (int i = fs.lo[0]; i < fs.lo[0] + fs.ext[0]; i++) {
            const long f = fs.idx(i, j, k);
            const int o = m - 3;
            const long x = b.cell(i + o * off[0], j + o * off[1], k + o * off[2]);
            T pr[10], Vc[16], Wc[16];
            for (int v = 0; v < nproj; v++) pr[v] = proj[(size_t)v * nf + f];
            for (int e = 0; e < neq; e++) Vc[e] = D.V[(size_t)e * nc + x];
            char_from_prim(c, a, pr, Vc, Wc);
            for (int e = 0; e < neq; e++) W[((size_t)m * neq + e) * nf + f] = Wc[e];
        }

        // WENO interpolation (performWENOInterpolation: JS :235-737, LD :417-955,
        // Z WCNS5-Z-HLLC-HLL.cpp:239-741, CU-M2 WCNS6-CU-M2-HLLC-HLL.cpp:326-891 with the
        // grid geometry's spacing along this axis, :383,541,806).
        for (int e = 0; e < neq; e++)
        for (long f = 0; f < nf; f++) {
            T U[6];
            for (int m = 0; m < 6; m++) U[m] = W[((size_t)m * neq + e) * nf + f];
            if (c.scheme == SCHEME_WCNS5_JS) {
                Wm[(size_t)e * nf + f] = js_minus(U, c.p);
                Wp[(size_t)e * nf + f] = js_plus(U, c.p);
            } else if (c.scheme == SCHEME_WCNS6_LD) {
                Wm[(size_t)e * nf + f] = ld_minus(U, c.p, c.q, c.C, c.alpha_tau);
                Wp[(size_t)e * nf + f] = ld_plus(U, c.p, c.q, c.C, c.alpha_tau);
            } else if (c.scheme == SCHEME_WCNS5_Z) {
                Wm[(size_t)e * nf + f] = z_minus(U, c.p);
                Wp[(size_t)e * nf + f] = z_plus(U, c.p);
            } else {
                Wm[(size_t)e * nf + f] = cu_minus(U, c.q, c.C, c.Chi, c.epsilon, c.grid_dx[a]);
                Wp[(size_t)e * nf + f] = cu_plus(U, c.q, c.C, c.Chi, c.epsilon, c.grid_dx[a]);
            }
        }

        HMRO_PHASE(HMRO_PH_INV);
        // Back to primitive variables, bounds check, first-order fallback
        // (WCNS56-HLLC-HLL.cpp:908-1032).
        for (long f = 0; f < nf; f++) {
            T pr[10], wc[16], vc[16];
            for (int v = 0; v < nproj; v++) pr[v] = proj[(size_t)v * nf + f];
            for (int e = 0; e < neq; e++) wc[e] = Wm[(size_t)e * nf + f];
            prim_from_char(c, a, pr, wc, vc);
            for (int e = 0; e < neq; e++) Vm[(size_t)e * nf + f] = vc[e];
            for (int e = 0; e < neq; e++) wc[e] = Wp[(size_t)e * nf + f];
            prim_from_char(c, a, pr, wc, vc);
            for (int e = 0; e < neq; e++) Vp[(size_t)e * nf + f] = vc[e];
        }
        HMRO_PHASE(HMRO_PH_BOUNDS);
        for (long f = 0; f < nf; f++) {
            T vc[16];
            for (int e = 0; e < neq; e++) vc[e] = Vm[(size_t)e * nf + f];
            flag_m[f] = face_bounded(c, vc);
            for (int e = 0; e < neq; e++) vc[e] = Vp[(size_t)e * nf + f];
            flag_p[f] = face_bounded(c, vc);
        }
        for (int k = fs.lo[2]; k < fs.lo[2] + fs.ext[2]; k++)
        for (int j = fs.lo[1]; j < fs.lo[1] + fs.ext[1]; j++)
        for (int i = fs.lo[0]; i < fs.lo[0] + fs.ext[0]; i++) {
            const long f = fs.idx(i, j, k);
            if (flag_m[f] == 0 || flag_p[f] == 0) {
                const long xL = b.cell(i - off[0], j - off[1], k - off[2]);
                const long xR = b.cell(i, j, k);
                for (int e = 0; e < neq; e++) {
                    Vm[(size_t)e * nf + f] = D.V[(size_t)e * nc + xL];
                    Vp[(size_t)e * nf + f] = D.V[(size_t)e * nc + xR];
                }
                cnt_fallback++;
            }
        }

        HMRO_PHASE(HMRO_PH_RIEMANN);
        // Riemann fluxes, Ducros-like sensor and selection (:1038-1194).
        for (int k = fs.lo[2]; k < fs.lo[2] + fs.ext[2]; k++)
        for (int j = fs.lo[1]; j < fs.lo[1] + fs.ext[1]; j++)
        for (int i = fs.lo[0]; i < fs.lo[0] + fs.ext[0]; i++) {
            const long f = fs.idx(i, j, k);
            T VL[16], VR[16], Fc[16], Fh[16], um;
            for (int e = 0; e < neq; e++) { VL[e] = Vm[(size_t)e * nf + f]; VR[e] = Vp[(size_t)e * nf + f]; }
            const long xL = b.cell(i - off[0], j - off[1], k - off[2]);
            const long xR = b.cell(i, j, k);
            const T theta_avg = 0.5*(theta[xL] + theta[xR]);
            const T Omega_avg = 0.5*(Omega[xL] + Omega[xR]);
            const T s = -theta_avg/(s_fabs(theta_avg) + Omega_avg + EPS);
            const bool use_hll = s_val(s) > 0.65;
            // The reference evaluates both midpoint fluxes on every face
            // (WCNS56-HLLC-HLL.cpp:1038-1064); the HLL part only matters where
            // the sensor selects it, which is all the op counter charges.
            riemann_face(c, a, VL, VR, Fc, Fh, um, !g_minimal_hll || use_hll);
            if (use_hll) cnt_hll++;
            for (int e = 0; e < neq; e++) Fmid[a][(size_t)e * nf + f] = use_hll ? Fh[e] : Fc[e];
            umid[a][f] = um;
            cnt_faces++;
        }

        HMRO_PHASE(HMRO_PH_FLUX);
        // Flux reconstruction, :1200-1282 (3D :2370-2480).
        for (int e = 0; e < neq; e++) {
            T* Fout = flux[a * neq + e];
            const T* Fm = &Fmid[a][(size_t)e * nf];
            const T* Fn = &D.Fn[((size_t)a * neq + e) * nc];
            for (int k = 0; k < b.n[2] + off[2]; k++)
            for (int j = 0; j < b.n[1] + off[1]; j++)
            for (int i = 0; i < b.n[0] + off[0]; i++) {
                const long f = fs.idx(i, j, k);
                const long fL = fs.idx(i - off[0], j - off[1], k - off[2]);
                const long fR = fs.idx(i + off[0], j + off[1], k + off[2]);
                const long xL = b.cell(i - off[0], j - off[1], k - off[2]);
                const long xR = b.cell(i, j, k);
                Fout[side_index(b, a, i, j, k)] = dt*(
                    double(1)/double(30)*(Fm[fR] + Fm[fL]) -
                    double(3)/double(10)*(Fn[xR] + Fn[xL]) +
                    double(23)/double(15)*Fm[f]);
            }
        }
    }

    HMRO_PHASE(HMRO_PH_SOURCE);
    // Advective source (five-eqn volume fractions), :1288-1369 (3D :2623).
    if (five) {
        for (int si = 0; si < N - 1; si++) {
            const int ei = N + dim + 1 + si;
            T* S = source[ei];
            for (int k = 0; k < b.n[2]; k++)
            for (int j = 0; j < b.n[1]; j++)
            for (int i = 0; i < b.n[0]; i++) {
                const int ii[3] = {i, j, k};
                T sum = T(0.0);
                for (int a = 0; a < dim; a++) {
                    const int o[3] = {a == 0, a == 1, a == 2};
                    const FaceSet& fs = FS[a];
                    const T* um = umid[a].data();
                    const T* u = &D.V[(size_t)(iu + a) * nc];
                    const long fL = fs.idx(ii[0], ii[1], ii[2]);
                    const long fR = fs.idx(ii[0] + o[0], ii[1] + o[1], ii[2] + o[2]);
                    const long fLL = fs.idx(ii[0] - o[0], ii[1] - o[1], ii[2] - o[2]);
                    const long fRR = fs.idx(ii[0] + 2 * o[0], ii[1] + 2 * o[1], ii[2] + 2 * o[2]);
                    const long xL = b.cell(ii[0] - o[0], ii[1] - o[1], ii[2] - o[2]);
                    const long xR = b.cell(ii[0] + o[0], ii[1] + o[1], ii[2] + o[2]);
                    const T term = (double(3)/double(2)*(um[fR] - um[fL]) -
                         double(3)/double(10)*(u[xR] - u[xL]) +
                         double(1)/double(30)*(um[fRR] - um[fLL]))/dx[a];
                    if (a == 0) sum = term; else sum = sum + term;
                }
                S[interior_index(b, i, j, k)] += dt*Q[ei][b.cell(i, j, k)]*(sum);
            }
        }
    }

    if (stats) {
        stats->faces = cnt_faces;
        stats->fallback = cnt_fallback;
        stats->hllc_hll = cnt_hll;
    }
}

// ---------------------------------------------------------------------------
// Runge-Kutta stage update, Euler::advanceSingleStepOnPatch (Euler.cpp:1003-1680):
//   Q = 0; for n <= stage: Q += alpha_n Q_int[n];
//   Q += beta_n * (-(F_R - F_L)/dx - ... + S_n);  F += gamma_n F_n;  S += gamma_n S_n
// followed by FlowModel*::updateCellDataOfConservativeVariables (five-eqn:
// last volume fraction = 1 - sum of the others, FlowModelFiveEqnAllaire.cpp:1739-1890).
// Q_out covers the ghost box; only the interior is written (ghosts are zeroed,
// as fillCellDataOfConservativeVariablesWithZero does).
// ---------------------------------------------------------------------------
template <class T>
void rk_stage(const Config& c, const int* n, const double* dx, int nstages,
              const double* alpha, const double* beta, const double* gamma,
              const T* const* const* Q_int, const T* const* const* F_int, const T* const* const* S_int,
              T* const* Q_out, T* const* F_acc, T* const* S_acc,
              const T* const* const* Fd_int = nullptr) {
    const int dim = c.dim;
    const int neq = num_eqn(c);
    const int ncomp = num_comp(c);
    const Box b = make_box(dim, n, c.ghosts);
    for (int e = 0; e < ncomp; e++)
        for (long x = 0; x < b.ncell(); x++) Q_out[e][x] = T(0.0);
    for (int s = 0; s < nstages; s++) {
        if (alpha[s] != 0.0) {
            for (int e = 0; e < neq; e++)
            for (int k = 0; k < b.n[2]; k++)
            for (int j = 0; j < b.n[1]; j++)
            for (int i = 0; i < b.n[0]; i++) {
                const long x = b.cell(i, j, k);
                Q_out[e][x] += alpha[s]*Q_int[s][e][x];
            }
        }
        if (beta[s] != 0.0) {
            for (int e = 0; e < neq; e++) {
                const T* Fx = F_int[s][0 * neq + e];
                const T* Fy = F_int[s][1 * neq + e];
                const T* Fz = (dim == 3) ? F_int[s][2 * neq + e] : nullptr;
                const T* S = S_int[s][e];
                const T* Dx = Fd_int ? Fd_int[s][0 * neq + e] : nullptr;
                const T* Dy = Fd_int ? Fd_int[s][1 * neq + e] : nullptr;
                const T* Dz = (Fd_int && dim == 3) ? Fd_int[s][2 * neq + e] : nullptr;
                for (int k = 0; k < b.n[2]; k++)
                for (int j = 0; j < b.n[1]; j++)
                for (int i = 0; i < b.n[0]; i++) {
                    const long x = b.cell(i, j, k);
                    const long is = interior_index(b, i, j, k);
                    const long xl = side_index(b, 0, i, j, k), xr = side_index(b, 0, i + 1, j, k);
                    const long yl = side_index(b, 1, i, j, k), yr = side_index(b, 1, i, j + 1, k);
                    if (Fd_int && dim == 2) {
                        // NavierStokes::advanceSingleStepOnPatch (NavierStokes.cpp:1743-1749, 2D)
                        Q_out[e][x] += beta[s]*
                            (-(Fx[xr] - Fx[xl] + Dx[xr] - Dx[xl])/dx[0] -
                              (Fy[yr] - Fy[yl] + Dy[yr] - Dy[yl])/dx[1] +
                              S[is]);
                    } else if (Fd_int) {
                        // NavierStokes.cpp:2085-2092 (3D)
                        const long zl = side_index(b, 2, i, j, k), zr = side_index(b, 2, i, j, k + 1);
                        Q_out[e][x] += beta[s]*
                            (-(Fx[xr] - Fx[xl] + Dx[xr] - Dx[xl])/dx[0] -
                              (Fy[yr] - Fy[yl] + Dy[yr] - Dy[yl])/dx[1] -
                              (Fz[zr] - Fz[zl] + Dz[zr] - Dz[zl])/dx[2] +
                              S[is]);
                    } else if (dim == 2) {
                        Q_out[e][x] += beta[s]*
                            (-(Fx[side_index(b, 0, i + 1, j, k)] - Fx[side_index(b, 0, i, j, k)])/dx[0] -
                              (Fy[side_index(b, 1, i, j + 1, k)] - Fy[side_index(b, 1, i, j, k)])/dx[1] +
                              S[is]);
                    } else {
                        Q_out[e][x] += beta[s]*
                            (-(Fx[side_index(b, 0, i + 1, j, k)] - Fx[side_index(b, 0, i, j, k)])/dx[0] -
                              (Fy[side_index(b, 1, i, j + 1, k)] - Fy[side_index(b, 1, i, j, k)])/dx[1] -
                              (Fz[side_index(b, 2, i, j, k + 1)] - Fz[side_index(b, 2, i, j, k)])/dx[2] +
                              S[is]);
                    }
                }
            }
        }
        if (gamma[s] != 0.0 && F_acc && S_acc) {
            for (int a = 0; a < dim; a++)
            for (int e = 0; e < neq; e++) {
                const long nfa = (long)(b.n[0] + (a == 0)) * (b.n[1] + (a == 1)) * (b.n[2] + (a == 2));
                for (long f = 0; f < nfa; f++) F_acc[a * neq + e][f] += gamma[s]*F_int[s][a * neq + e][f];
            }
            for (int e = 0; e < neq; e++)
                for (long x = 0; x < (long)b.n[0] * b.n[1] * b.n[2]; x++) S_acc[e][x] += gamma[s]*S_int[s][e][x];
        }
        if (beta[s] != 0.0 && c.model == MODEL_FIVE_EQN_ALLAIRE) {
            const int N = c.num_species;
            T* ZN = Q_out[neq];
            for (int k = 0; k < b.n[2]; k++)
            for (int j = 0; j < b.n[1]; j++)
            for (int i = 0; i < b.n[0]; i++) ZN[b.cell(i, j, k)] = T(1.0);
            for (int si = 0; si < N - 1; si++)
                for (int k = 0; k < b.n[2]; k++)
                for (int j = 0; j < b.n[1]; j++)
                for (int i = 0; i < b.n[0]; i++) {
                    const long x = b.cell(i, j, k);
                    ZN[x] -= Q_out[N + dim + 1 + si][x];
                }
        }
    }
}

// ---------------------------------------------------------------------------
// Navier-Stokes diffusive flux of a single-species patch,
// DiffusiveFluxReconstructorMidpoint::computeDiffusiveFluxOnPatch
//   src/flow/diffusive_flux_reconstructors/midpoint/DiffusiveFluxReconstructorMidpoint.cpp:38-2312
// with the second-order (…MidpointSecondOrder.cpp) and fourth-order
// (…MidpointFourthOrder.cpp) stencils, the single-species coefficient tables of
//   src/flow/flow_models/single-species/FlowModelDiffusiveFluxUtilitiesSingleSpecies.cpp
//   (derivative variables :654-1505, diffusivities at sides :2471-2799, their use :2800-3700),
// constant shear and bulk viscosity and the Prandtl thermal conductivity
// kappa = c_p mu/Pr (EquationOfThermalConductivityPrandtl.cpp:29-63), and the
// temperature T = p/((gamma - 1) c_v rho) (EquationOfStateIdealGas.cpp:2157-2173).
// ---------------------------------------------------------------------------
struct Transport {
    int order;          // 2, 4 or 6: MIDPOINT_SECOND_ORDER / _FOURTH_ORDER / _SIXTH_ORDER (5 ghosts)
    double mu;          // Equation_of_shear_viscosity_mixing_rules.species_mu (CONSTANT)
    double mu_v;        // Equation_of_bulk_viscosity_mixing_rules.species_mu_v (CONSTANT)
    double c_p, Pr;     // Equation_of_thermal_conductivity_mixing_rules.species_c_p, species_Pr (PRANDTL)
    double mu_kappa;    // ... and that model's own (constant) shear viscosity species_mu
};

// One term of a midpoint flux: equation e += D[k] * (derivative of variable v).
// v: 0..dim-1 velocity components, 3 temperature.  Rows follow the reference's
// per-equation order (first the derivatives along x, then y, then z).
struct DiffTerm { int e, v, k; };

// Terms of the flux normal to axis a differentiated along axis d.  The
// reference's D_k at a side normal to a (computeSideDataOfDiffusiveFluxDiffusivities):
//   D0 = -(4/3 mu + mu_v), D1 = 2/3 mu - mu_v, D2 = -mu,
//   D3 = -u_a (4/3 mu + mu_v), D4 = u_a (2/3 mu - mu_v),
//   D5, D6 = -u_t mu for the transverse velocities t in increasing axis order (3D),
//   last = -kappa (D7 in 3D; D6 in 2D, where D5 = -u_t mu).
inline int diff_terms(int dim, int a, int d, DiffTerm* out) {
    static const DiffTerm T3[3][3][7] = {
        {{{1, 0, 0}, {2, 1, 2}, {3, 2, 2}, {4, 0, 3}, {4, 1, 5}, {4, 2, 6}, {4, 3, 7}},
         {{1, 1, 1}, {2, 0, 2}, {4, 0, 5}, {4, 1, 4}},
         {{1, 2, 1}, {3, 0, 2}, {4, 0, 6}, {4, 2, 4}}},
        {{{1, 1, 2}, {2, 0, 1}, {4, 0, 4}, {4, 1, 5}},
         {{1, 0, 2}, {2, 1, 0}, {3, 2, 2}, {4, 0, 5}, {4, 1, 3}, {4, 2, 6}, {4, 3, 7}},
         {{2, 2, 1}, {3, 1, 2}, {4, 1, 6}, {4, 2, 4}}},
        {{{1, 2, 2}, {3, 0, 1}, {4, 0, 4}, {4, 2, 5}},
         {{2, 2, 2}, {3, 1, 1}, {4, 1, 4}, {4, 2, 6}},
         {{1, 0, 2}, {2, 1, 2}, {3, 2, 0}, {4, 0, 5}, {4, 1, 6}, {4, 2, 3}, {4, 3, 7}}}};
    static const int N3[3][3] = {{7, 4, 4}, {4, 7, 4}, {4, 4, 7}};
    static const DiffTerm T2[2][2][5] = {
        {{{1, 0, 0}, {2, 1, 2}, {3, 0, 3}, {3, 1, 5}, {3, 3, 6}},
         {{1, 1, 1}, {2, 0, 2}, {3, 0, 5}, {3, 1, 4}}},
        {{{1, 1, 2}, {2, 0, 1}, {3, 0, 4}, {3, 1, 5}},
         {{1, 0, 2}, {2, 1, 0}, {3, 0, 5}, {3, 1, 3}, {3, 3, 6}}}};
    static const int N2[2][2] = {{5, 4}, {4, 5}};
    const int nt = dim == 3 ? N3[a][d] : N2[a][d];
    for (int t = 0; t < nt; t++) out[t] = dim == 3 ? T3[a][d][t] : T2[a][d][t];
    return nt;
}

// Diffusivities D_k at one side normal to axis a from the side values of mu,
// mu_v, kappa and the velocity (FlowModelDiffusiveFluxUtilitiesSingleSpecies.cpp:2471-2799).
template <class T>
inline void side_diffusivities(int dim, int a, const T& mu, const T& mu_v, const T& kappa, const T* u, T* D) {
    D[0] = -(double(4)/double(3)*mu + mu_v);
    D[1] = double(2)/double(3)*mu - mu_v;
    D[2] = -mu;
    D[3] = -u[a]*(double(4)/double(3)*mu + mu_v);
    D[4] = u[a]*(double(2)/double(3)*mu - mu_v);
    if (dim == 2) {
        D[5] = -u[1 - a]*mu;
        D[6] = -kappa;
    } else {
        const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
        D[5] = -u[t1]*mu;
        D[6] = -u[t2]*mu;
        D[7] = -kappa;
    }
}

// Midpoint stencils (…MidpointSecondOrder.cpp / …MidpointFourthOrder.cpp):
//   derivative at a midpoint   2nd: 1*(u_R - u_L)/dx             4th: (9/8 (u_R - u_L) - 1/24 (u_RR - u_LL))/dx
//   derivative at a node       2nd: 1/2*(u_+1 - u_-1)/dx         4th: (2/3 (u_+1 - u_-1) - 1/12 (u_+2 - u_-2))/dx
//   node -> midpoint value     2nd: 1/2*(u_R + u_L)              4th: 9/16 (u_R + u_L) - 1/16 (u_RR + u_LL)
//   midpoint -> face flux      2nd: dt*1*F                        4th: dt*(13/12 F - 1/24 (F_-1 + F_+1))
// each evaluated in the reference's operation order; dx_inv = 1/dx.
template <class T>
inline T mid_derivative(int order, const T& LL, const T& L, const T& R, const T& RR, double dx_inv) {
    if (order == 2) return double(1)*(R - L)*dx_inv;
    return (double(9)/double(8)*(R - L) + -double(1)/double(24)*(RR - LL))*dx_inv;
}
template <class T>
inline T node_derivative(int order, const T& mm, const T& m, const T& p, const T& pp, double dx_inv) {
    if (order == 2) return double(1)/double(2)*(p - m)*dx_inv;
    return (double(2)/double(3)*(p - m) + -double(1)/double(12)*(pp - mm))*dx_inv;
}
template <class T>
inline T mid_value(int order, const T& LL, const T& L, const T& R, const T& RR) {
    if (order == 2) return double(1)/double(2)*(R + L);
    return double(9)/double(16)*(R + L) + -double(1)/double(16)*(RR + LL);
}
// Sixth order (…MidpointSixthOrder.cpp): midpoint derivative :80-117 (75/64, -25/384, 3/640),
// node derivative :521-558 (3/4, -3/20, 1/60), node -> midpoint value :962-1000
// (75/128, -25/256, 3/256); v[0..5] are the cells at offsets -3..2 (midpoint stencils) or
// -3, -2, -1, 1, 2, 3 (node stencil).
template <class T>
inline T mid_derivative6(const T* v, double dx_inv) {
    const double a = double(75)/double(64), b = -double(25)/double(384), c = double(3)/double(640);
    return (a*(v[3] - v[2]) + b*(v[4] - v[1]) + c*(v[5] - v[0]))*dx_inv;
}
template <class T>
inline T node_derivative6(const T* v, double dx_inv) {
    const double a = double(3)/double(4), b = -double(3)/double(20), c = double(1)/double(60);
    return (a*(v[3] - v[2]) + b*(v[4] - v[1]) + c*(v[5] - v[0]))*dx_inv;
}
template <class T>
inline T mid_value6(const T* v) {
    const double a = double(75)/double(128), b = -double(25)/double(256), c = double(3)/double(256);
    return (a*(v[3] + v[2]) + b*(v[4] + v[1]) + c*(v[5] + v[0]));
}

// Cell fields the diffusive flux reads: velocity and temperature.
template <class T>
void diff_cell_fields(const Config& c, const Box& b, const Derived<T>& D, std::vector<T>& W) {
    const int dim = c.dim;
    const long nc = b.ncell();
    W.assign((size_t)4 * nc, T(0.0));
    const double cv = species_cv(c, 0);
    for (long x = 0; x < nc; x++) {
        for (int d = 0; d < dim; d++) W[(size_t)d * nc + x] = D.V[(size_t)(1 + d) * nc + x];
        const T& rho = D.V[x];
        const T& p = D.V[(size_t)(dim + 1) * nc + x];
        W[(size_t)3 * nc + x] = p/((c.gamma[0] - double(1))*cv*rho);
    }
}

// Midpoint flux (all equations) of the side normal to a between cells xL = x - e_a and x
// (f = index along a of cell x): F_mid of …Midpoint.cpp:1420-1620 (x), analogues for y, z.
template <class T>
void diff_midpoint(const Config& c, const Transport& tr, const Box& b, const std::vector<T>& W, int a,
                   int i, int j, int k, const double* dx, T* F) {
    const int dim = c.dim, neq = num_eqn(c);
    const long nc = b.ncell();
    const int order = tr.order;
    auto at = [&](int v, int ii, int jj, int kk) -> const T& { return W[(size_t)v * nc + b.cell(ii, jj, kk)]; };
    auto sh = [&](int ax, int m, int& ii, int& jj, int& kk) {
        ii = i; jj = j; kk = k;
        if (ax == 0) ii += m; else if (ax == 1) jj += m; else kk += m;
    };
    // value of field v at the midpoint (cells f-2, f-1, f, f+1 along a; f-3 .. f+2 at sixth order)
    auto mid = [&](auto&& cellval) {
        if (order == 6) {
            T v6[6];
            for (int m = -3; m <= 2; m++) {
                int ii, jj, kk;
                sh(a, m, ii, jj, kk);
                v6[m + 3] = cellval(ii, jj, kk);
            }
            return mid_value6(v6);
        }
        int i0, j0, k0, i1, j1, k1, i2, j2, k2, i3, j3, k3;
        sh(a, -2, i0, j0, k0); sh(a, -1, i1, j1, k1); sh(a, 0, i2, j2, k2); sh(a, 1, i3, j3, k3);
        return mid_value(order, cellval(i0, j0, k0), cellval(i1, j1, k1), cellval(i2, j2, k2), cellval(i3, j3, k3));
    };
    // constant transport properties at cells, interpolated like every other side variable
    const double kappa_c = tr.c_p*tr.mu_kappa/tr.Pr;
    const T mu = mid([&](int, int, int) { return T(tr.mu); });
    const T mu_v = mid([&](int, int, int) { return T(tr.mu_v); });
    const T kappa = mid([&](int, int, int) { return T(kappa_c); });
    T u[3] = {T(0.0), T(0.0), T(0.0)};
    for (int d = 0; d < dim; d++) u[d] = mid([&](int ii, int jj, int kk) { return at(d, ii, jj, kk); });
    T D[8];
    side_diffusivities(dim, a, mu, mu_v, kappa, u, D);
    for (int e = 0; e < neq; e++) F[e] = T(0.0);
    for (int d = 0; d < dim; d++) {
        DiffTerm terms[7];
        const int nt = diff_terms(dim, a, d, terms);
        const double dx_inv = double(1)/dx[d];
        for (int t = 0; t < nt; t++) {
            const int v = terms[t].v;
            T g;
            if (d == a && order == 6) {
                T v6[6];
                for (int m = -3; m <= 2; m++) {
                    int ii, jj, kk;
                    sh(a, m, ii, jj, kk);
                    v6[m + 3] = at(v, ii, jj, kk);
                }
                g = mid_derivative6(v6, dx_inv);
            } else if (d == a) {
                int i0, j0, k0, i1, j1, k1, i2, j2, k2, i3, j3, k3;
                sh(a, -2, i0, j0, k0); sh(a, -1, i1, j1, k1); sh(a, 0, i2, j2, k2); sh(a, 1, i3, j3, k3);
                g = mid_derivative(order, at(v, i0, j0, k0), at(v, i1, j1, k1), at(v, i2, j2, k2), at(v, i3, j3, k3),
                                   dx_inv);
            } else {
                // derivative along d at the four cells, then to the midpoint along a
                g = mid([&](int ii, int jj, int kk) {
                    auto node = [&](int m) {
                        int i4 = ii, j4 = jj, k4 = kk;
                        if (d == 0) i4 += m; else if (d == 1) j4 += m; else k4 += m;
                        return at(v, i4, j4, k4);
                    };
                    if (order == 6) {
                        const T v6[6] = {node(-3), node(-2), node(-1), node(1), node(2), node(3)};
                        return node_derivative6(v6, dx_inv);
                    }
                    return node_derivative(order, node(-2), node(-1), node(1), node(2), dx_inv);
                });
            }
            F[terms[t].e] += D[terms[t].k]*g;
        }
    }
}

// Diffusive flux of a patch: dim*neq side arrays (0 ghosts), overwritten.
template <class T>
void diff_flux(const Config& c, const Transport& tr, const int* n, const double* dx, double dt,
               const T* const* Q, T* const* flux) {
    const int dim = c.dim, neq = num_eqn(c);
    const Box b = make_box(dim, n, c.ghosts);
    Derived<T> D;
    compute_derived(c, b, Q, D);
    std::vector<T> W;
    diff_cell_fields(c, b, D, W);
    const double a_r = double(9)/double(8) + -double(1)/double(24), b_r = -double(1)/double(24);
    // sixth order (…MidpointSixthOrder.cpp:1400-1440): a_m + b_m + c_m, b_m + c_m, c_m
    const double a6 = double(75)/double(64), b6 = -double(25)/double(384), c6 = double(3)/double(640);
    const double a_r6 = a6 + b6 + c6, b_r6 = b6 + c6, c_r6 = c6;
    T Fm[5][8], Fo[8];
    for (int a = 0; a < dim; a++) {
        const int e0 = b.n[0] + (a == 0), e1 = b.n[1] + (a == 1), e2 = b.n[2] + (a == 2);
        for (int k = 0; k < e2; k++)
        for (int j = 0; j < e1; j++)
        for (int i = 0; i < e0; i++) {
            const long f = side_index(b, a, i, j, k);
            if (tr.order == 2) {
                diff_midpoint(c, tr, b, W, a, i, j, k, dx, Fo);
                for (int e = 0; e < neq; e++) flux[a * neq + e][f] = T(0.0) + dt*double(1)*Fo[e];
            } else if (tr.order == 6) {
                for (int m = -2; m <= 2; m++)
                    diff_midpoint(c, tr, b, W, a, i + (a == 0 ? m : 0), j + (a == 1 ? m : 0), k + (a == 2 ? m : 0),
                                  dx, Fm[m + 2]);
                for (int e = 0; e < neq; e++)
                    flux[a * neq + e][f] = T(0.0) + dt*(a_r6*(Fm[2][e]) + b_r6*(Fm[1][e] + Fm[3][e]) +
                                                        c_r6*(Fm[0][e] + Fm[4][e]));
            } else {
                for (int m = -1; m <= 1; m++)
                    diff_midpoint(c, tr, b, W, a, i + (a == 0 ? m : 0), j + (a == 1 ? m : 0), k + (a == 2 ? m : 0),
                                  dx, Fm[m + 1]);
                for (int e = 0; e < neq; e++)
                    flux[a * neq + e][f] = T(0.0) + dt*(a_r*(Fm[1][e]) + b_r*(Fm[0][e] + Fm[2][e]));
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Refluxing (synchronisation of a coarse level with the finer one).
//   sync_fluxes      Euler::synchronizeFluxes (src/apps/Euler/Euler.cpp:1682-1943) and
//                    NavierStokes::synchronizeFluxes (NavierStokes.cpp:2425-2700): the coarse
//                    step redone from its old state with the time-integrated fluxes,
//                    Q += -div (F [+ Fd]) + S, then updateCellDataOfConservativeVariables.
//   coarsen_fluxsum  the flux-sum coarsening of RungeKuttaLevelIntegrator.cpp:2140-2160: on the
//                    outer sides of a fine patch each coarse face takes the mean of the r^(d-1)
//                    fine faces it covers.
//   coarsen_cells    the coarsening of fine interiors (RungeKuttaLevelIntegrator.cpp:2190-2230):
//                    each covered coarse cell takes the mean of its r^d fine cells.
// The two coarsening operators are SAMRAI's (CONSERVATIVE_COARSEN: area / volume weighted
// averages), which is not in the reference's tree; the order of their sums here (fine index
// order, then one multiplication by 1/r^k) is this restatement's own.
// ---------------------------------------------------------------------------
template <class T>
void sync_fluxes(const Config& c, const int* n, const double* dx, const T* const* F, const T* const* Fd,
                 const T* const* S, T* const* Q) {
    const int dim = c.dim, neq = num_eqn(c);
    const Box b = make_box(dim, n, c.ghosts);
    for (int e = 0; e < neq; e++) {
        for (int k = 0; k < b.n[2]; k++)
        for (int j = 0; j < b.n[1]; j++)
        for (int i = 0; i < b.n[0]; i++) {
            const long x = b.cell(i, j, k);
            const long is = interior_index(b, i, j, k);
            const long xl = side_index(b, 0, i, j, k), xr = side_index(b, 0, i + 1, j, k);
            const long yl = side_index(b, 1, i, j, k), yr = side_index(b, 1, i, j + 1, k);
            const T* Fx = F[e];
            const T* Fy = F[neq + e];
            if (Fd) {
                const T* Dx = Fd[e];
                const T* Dy = Fd[neq + e];
                if (dim == 2) {
                    Q[e][x] += (-(Fx[xr] - Fx[xl] + Dx[xr] - Dx[xl])/dx[0] -
                                 (Fy[yr] - Fy[yl] + Dy[yr] - Dy[yl])/dx[1] +
                                 S[e][is]);
                } else {
                    const long zl = side_index(b, 2, i, j, k), zr = side_index(b, 2, i, j, k + 1);
                    const T* Fz = F[2 * neq + e];
                    const T* Dz = Fd[2 * neq + e];
                    Q[e][x] += (-(Fx[xr] - Fx[xl] + Dx[xr] - Dx[xl])/dx[0] -
                                 (Fy[yr] - Fy[yl] + Dy[yr] - Dy[yl])/dx[1] -
                                 (Fz[zr] - Fz[zl] + Dz[zr] - Dz[zl])/dx[2] +
                                 S[e][is]);
                }
            } else if (dim == 2) {
                Q[e][x] += (-(Fx[xr] - Fx[xl])/dx[0] -
                             (Fy[yr] - Fy[yl])/dx[1] +
                             S[e][is]);
            } else {
                const long zl = side_index(b, 2, i, j, k), zr = side_index(b, 2, i, j, k + 1);
                const T* Fz = F[2 * neq + e];
                Q[e][x] += (-(Fx[xr] - Fx[xl])/dx[0] -
                             (Fy[yr] - Fy[yl])/dx[1] -
                             (Fz[zr] - Fz[zl])/dx[2] +
                             S[e][is]);
            }
        }
    }
    if (c.model == MODEL_FIVE_EQN_ALLAIRE) {
        // FlowModelFiveEqnAllaire::updateCellDataOfConservativeVariables
        const int N = c.num_species;
        for (int k = 0; k < b.n[2]; k++)
        for (int j = 0; j < b.n[1]; j++)
        for (int i = 0; i < b.n[0]; i++) {
            const long x = b.cell(i, j, k);
            Q[neq][x] = T(1.0);
            for (int si = 0; si < N - 1; si++) Q[neq][x] -= Q[N + dim + 1 + si][x];
        }
    }
}

// Patch placement in a level's index space: first interior cell lo[3], interior size n[3].
// The fine patch's box coarsened by ratio[3] must be aligned (lo and lo + n multiples of r).
inline void coarsen_fluxsum(const Config& c, const int* ratio, const int* cn, const int* clo,
                            const int* fn, const int* flo, const double* const* Ff, double* const* Fc) {
    const int dim = c.dim, neq = num_eqn(c);
    const Box cb = make_box(dim, cn, c.ghosts), fb = make_box(dim, fn, c.ghosts);
    for (int a = 0; a < dim; a++) {
        int area = 1;
        for (int d = 0; d < dim; d++) if (d != a) area *= ratio[d];
        const double w = double(1)/double(area);
        for (int side = 0; side < 2; side++) {
            const int ff = side == 0 ? 0 : fn[a];            // fine face index along a (local)
            const int cf = (flo[a] + ff)/ratio[a] - clo[a];  // coarse face index along a (local)
            if (cf < 0 || cf > cn[a]) continue;
            int lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
            for (int d = 0; d < dim; d++) {
                if (d == a) continue;
                lo[d] = std::max(flo[d]/ratio[d], clo[d]) - clo[d];
                hi[d] = std::min((flo[d] + fn[d])/ratio[d], clo[d] + cn[d]) - clo[d];
            }
            for (int e = 0; e < neq; e++)
            for (int k = lo[2]; k < hi[2]; k++)
            for (int j = lo[1]; j < hi[1]; j++)
            for (int i = lo[0]; i < hi[0]; i++) {
                const int cc[3] = {i, j, k};
                int fi0[3];
                for (int d = 0; d < 3; d++) fi0[d] = d < dim ? (cc[d] + clo[d])*ratio[d] - flo[d] : 0;
                double sum = 0.0;
                const int r1 = a == 1 ? 1 : (dim > 1 ? ratio[1] : 1);
                const int r2 = (dim == 3 && a != 2) ? ratio[2] : 1;
                const int r0 = a == 0 ? 1 : ratio[0];
                for (int q2 = 0; q2 < r2; q2++)
                for (int q1 = 0; q1 < r1; q1++)
                for (int q0 = 0; q0 < r0; q0++) {
                    int f[3] = {fi0[0] + q0, fi0[1] + q1, fi0[2] + q2};
                    f[a] = ff;
                    sum += Ff[a * neq + e][side_index(fb, a, f[0], f[1], f[2])];
                }
                int g[3] = {i, j, k};
                g[a] = cf;
                Fc[a * neq + e][side_index(cb, a, g[0], g[1], g[2])] = sum*w;
            }
        }
    }
}

inline void coarsen_cells(const Config& c, const int* ratio, const int* cn, const int* clo,
                          const int* fn, const int* flo, const double* const* Qf, double* const* Qc) {
    const int dim = c.dim, ncomp = num_comp(c);
    const Box cb = make_box(dim, cn, c.ghosts), fb = make_box(dim, fn, c.ghosts);
    int vol = 1;
    for (int d = 0; d < dim; d++) vol *= ratio[d];
    const double w = double(1)/double(vol);
    int lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
    for (int d = 0; d < dim; d++) {
        lo[d] = std::max(flo[d]/ratio[d], clo[d]) - clo[d];
        hi[d] = std::min((flo[d] + fn[d])/ratio[d], clo[d] + cn[d]) - clo[d];
    }
    const int r0 = ratio[0], r1 = dim > 1 ? ratio[1] : 1, r2 = dim > 2 ? ratio[2] : 1;
    for (int e = 0; e < ncomp; e++)
    for (int k = lo[2]; k < hi[2]; k++)
    for (int j = lo[1]; j < hi[1]; j++)
    for (int i = lo[0]; i < hi[0]; i++) {
        const int fi = (i + clo[0])*r0 - flo[0];
        const int fj = dim > 1 ? (j + clo[1])*r1 - flo[1] : 0;
        const int fk = dim > 2 ? (k + clo[2])*r2 - flo[2] : 0;
        double sum = 0.0;
        for (int q2 = 0; q2 < r2; q2++)
        for (int q1 = 0; q1 < r1; q1++)
        for (int q0 = 0; q0 < r0; q0++) sum += Qf[e][fb.cell(fi + q0, fj + q1, fk + q2)];
        Qc[e][cb.cell(i, j, k)] = sum*w;
    }
}

// ---------------------------------------------------------------------------
// Coarse-fine ghost cells of a fine patch (the fill schedule's interpolation from the next
// coarser level, RungeKuttaLevelIntegrator.cpp:1568,1701 with the operators registered at
// FlowModelSingleSpecies.cpp:578-597): the coarse state at the fine time,
//   Q_c = (1 - theta) Q_c,old + theta Q_c,new
// (linear time interpolation), then conservative linear refinement: in a coarse cell C,
//   q_f = Q_c(C) + sum_d s_d(C) ((f_d + 1/2)/r_d - (C_d + 1/2)),
// with the monotonised-central slope per coarse cell width
//   s_d = sign(D) min(|D|, 2 min(|D-|, |D+|)) if D- D+ > 0 else 0,  D = (D- + D+)/2,
//   D- = Q_c(C) - Q_c(C - e_d),  D+ = Q_c(C + e_d) - Q_c(C).
// The mean of the fine values over a coarse cell is the coarse value.  Both operators are
// SAMRAI's (LINEAR_TIME_INTERPOLATE, CONSERVATIVE_LINEAR_REFINE), outside the reference's
// tree; this is a restatement of the published method, not a copy.  Every fine ghost cell
// whose coarse cell lies inside the coarse patch's interior is written (the coarse patch's
// ghost cells must be filled: the slopes read one coarse cell beyond).
// ---------------------------------------------------------------------------
inline double mc_slope(double dm, double dp) {
    if (!(dm*dp > 0.0)) return 0.0;
    const double d = double(1)/double(2)*(dm + dp);
    const double b = double(2)*std::min(std::fabs(dm), std::fabs(dp));
    return std::fabs(d) < b ? d : (d > 0.0 ? b : -b);
}

inline void refine_ghosts(const Config& c, const int* ratio, const int* fn, const int* flo, const int* cn,
                          const int* clo, const double* const* Qc_old, const double* const* Qc_new, double theta,
                          double* const* Qf) {
    const int dim = c.dim, ncomp = num_comp(c);
    const Box fb = make_box(dim, fn, c.ghosts), cb = make_box(dim, cn, c.ghosts);
    for (int k = -fb.g[2]; k < fb.n[2] + fb.g[2]; k++)
    for (int j = -fb.g[1]; j < fb.n[1] + fb.g[1]; j++)
    for (int i = -fb.g[0]; i < fb.n[0] + fb.g[0]; i++) {
        const int f[3] = {i, j, k};
        bool inside = true, covered = true;
        int C[3] = {0, 0, 0};
        for (int d = 0; d < dim; d++) {
            if (f[d] < 0 || f[d] >= fn[d]) inside = false;
            const int lev = flo[d] + f[d];
            const int cl = (lev >= 0 ? lev/ratio[d] : -((-lev + ratio[d] - 1)/ratio[d]));
            C[d] = cl - clo[d];
            if (C[d] < 0 || C[d] >= cn[d]) covered = false;
        }
        if (inside || !covered) continue;
        for (int e = 0; e < ncomp; e++) {
            auto q = [&](int di, int dj, int dk) {
                const long x = cb.cell(C[0] + di, C[1] + dj, C[2] + dk);
                return (double(1) - theta)*Qc_old[e][x] + theta*Qc_new[e][x];
            };
            const double q0 = q(0, 0, 0);
            double v = q0;
            for (int d = 0; d < dim; d++) {
                const int o[3] = {d == 0, d == 1, d == 2};
                const double s = mc_slope(q0 - q(-o[0], -o[1], -o[2]), q(o[0], o[1], o[2]) - q0);
                const int lev = flo[d] + f[d];
                const double off = (double(lev) + 0.5)/double(ratio[d]) - (double(C[d] + clo[d]) + 0.5);
                v += s*off;
            }
            Qf[e][fb.cell(i, j, k)] = v;
        }
    }
}

// Ghost fill of one patch.  On one level with one patch this is what SAMRAI's periodic shift
// and the reference's boundary conditions produce.  Per axis: mode 0 zero-gradient (nearest
// interior cell, the extrapolation condition), 1 periodic,
// 3 reflecting wall -- the mirror image across the boundary face, the momentum component normal
// to it negated (BasicCartesianBoundaryUtilities2.cpp:349-395 REFLECT for the momentum vector,
// :397-440 SYMMETRY for the scalars, as EulerBoundaryConditions.cpp:205-297 assigns them).
template <class T>
void fill_ghosts(const Config& c, const int* n, const int* periodic, T* const* Q, const double* bvals = nullptr) {
    // Mode per axis: 0 FLOW (copy of the nearest interior cell), 1 periodic, 3 REFLECT (mirror
    // image, normal momentum negated), 5 SYMMETRY (mirror image of every variable as it is,
    // BasicCartesianBoundaryUtilities2.cpp:397-440), 4 DIRICHLET: the side's values bvals[(2 axis + high) ncomp
    // + e] (BasicCartesianBoundaryUtilities2.cpp:150-165); a cell beyond two Dirichlet sides takes
    // the lower axis's values (the corner condition XDIRICHLET, :679-710), one beyond a Dirichlet
    // side and another condition the Dirichlet values.
    const Box b = make_box(c.dim, n, c.ghosts);
    const int ncomp = num_comp(c);
    const int mom0 = vel_index(c);
    auto src = [&](int v, int a) {
        if (v >= 0 && v < b.n[a]) return v;
        if (periodic[a] == 1) return ((v % b.n[a]) + b.n[a]) % b.n[a];
        if (periodic[a] == 3 || periodic[a] == 5) return v < 0 ? -v - 1 : 2 * b.n[a] - 1 - v;
        return v < 0 ? 0 : b.n[a] - 1;
    };
    for (int e = 0; e < ncomp; e++)
        for (int k = -b.g[2]; k < b.n[2] + b.g[2]; k++)
        for (int j = -b.g[1]; j < b.n[1] + b.g[1]; j++)
        for (int i = -b.g[0]; i < b.n[0] + b.g[0]; i++) {
            if (i >= 0 && i < b.n[0] && j >= 0 && j < b.n[1] && k >= 0 && k < b.n[2]) continue;
            const int ijk[3] = {i, j, k};
            int dside = -1;
            for (int a = 0; a < c.dim && dside < 0; a++)
                if (periodic[a] == 4 && (ijk[a] < 0 || ijk[a] >= b.n[a])) dside = 2 * a + (ijk[a] >= 0);
            if (dside >= 0) {
                Q[e][b.cell(i, j, k)] = T(bvals ? bvals[dside * ncomp + e] : 0.0);
                continue;
            }
            bool flip = false;
            for (int a = 0; a < c.dim; a++)
                if (periodic[a] == 3 && (ijk[a] < 0 || ijk[a] >= b.n[a]) && e == mom0 + a) flip = !flip;
            const T v = Q[e][b.cell(src(i, 0), src(j, 1), c.dim == 3 ? src(k, 2) : 0)];
            Q[e][b.cell(i, j, k)] = flip ? -v : v;
        }
}

}  // namespace hmro

// C view of Config taken by the entry points of the oracle libraries
// (hmr_oracle.cpp, hmr_tangent.cpp); oracle.py's _Cfg mirrors it field by field.
extern "C" {
struct hmro_config {
    int model;
    int dim;
    int num_species;
    int scheme;
    double gamma[8];
    double R[8];
    int p;
    int q;
    double C;
    double alpha_tau;
    double Chi;
    double epsilon;
    double grid_dx[3];
    int ghosts;          // 0 means 4
};
}

// C view of Transport (oracle.py's _Transport mirrors it).
extern "C" {
struct hmro_transport {
    int order;
    double mu, mu_v, c_p, Pr, mu_kappa;
};
}

inline hmro::Transport hmro_to_transport(const hmro_transport* t) {
    hmro::Transport r;
    r.order = t->order;
    r.mu = t->mu;
    r.mu_v = t->mu_v;
    r.c_p = t->c_p;
    r.Pr = t->Pr;
    r.mu_kappa = t->mu_kappa;
    return r;
}

inline hmro::Config hmro_to_config(const hmro_config* c) {
    hmro::Config k;
    k.model = c->model;
    k.dim = c->dim;
    k.num_species = c->num_species;
    k.scheme = c->scheme;
    for (int i = 0; i < 8; i++) k.gamma[i] = c->gamma[i];
    for (int i = 0; i < 8; i++) k.R[i] = c->R[i];
    k.p = c->p;
    k.q = c->q;
    k.C = c->C;
    k.alpha_tau = c->alpha_tau;
    k.Chi = c->Chi;
    k.epsilon = c->epsilon;
    for (int i = 0; i < 3; i++) k.grid_dx[i] = c->grid_dx[i];
    k.ghosts = c->ghosts > 0 ? c->ghosts : 4;
    return k;
}
