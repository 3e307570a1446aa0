// Work items of one RK substep on one patch, written as device functions so
// that the per-patch kernels (one launch per phase) and the persistent
// batched kernel (one launch per substep over a worklist) run the same code.
//
// Phases of a substep on a patch with interior n and ghost width 4:
//   1. cells  : primitive variables, density, sound speed on the ghost box
//   2. sensor : dilatation and vorticity magnitude on the interior grown by 2
//   3. faces  : per axis a, every midpoint face f in [-1, n_a+1] x interior:
//               characteristic projection -> WCNS interpolation -> inverse
//               projection -> bounds check / first-order fallback ->
//               HLLC or HLLC-HLL (Ducros-like sensor) -> midpoint flux
//   4. update : per interior cell: 6th-order midpoint-node flux formula,
//               flux divergence, advective source, RK stage combination
// Each face is computed exactly once: FP64 throughput is the scarce
// resource on GB300, so recomputing halo faces inside tiles costs more than
// streaming the midpoint fluxes through L2/HBM.
#pragma once

#include "hmr_physics.cuh"

namespace hmr {

// Ghost width of the WCNS56 stencils (ConvectiveFluxReconstructorWCNS56-HLLC-HLL.cpp:22); a patch's
// arrays carry GHOST cells, or 5 with the sixth-order midpoint diffusive flux (Geom::gh).
constexpr int GHOST = 4;
constexpr int GHOST_MAX = 5;

struct Geom {
    int n[3];       // interior cells (1 on unused axes)
    int G[3];       // ghost-box extents, n + 2 gh
    double dx[3];
    int gh = GHOST; // ghost cells per side
};

struct Comp {
    double* p[MAX_COMP];
};

// Face-flux arrays of a patch: dim x NEQ pointers, axis-major.
struct FluxComp {
    double* p[3 * MAX_COMP];
};

// Scratch of one patch (all on the device).
struct Scratch {
    double* V;        // NEQ x ncell
    double* rho;      // ncell
    double* cs;       // ncell
    double* theta;    // ncell
    double* Omega;    // ncell
    double* Fm[3];    // NEQ x nface(a)
    double* um[3];    // nface(a) (five-equation model only)
    double* Td;       // ncell: temperature (Navier-Stokes only)
    double* Gd;       // DIM*DIM x ncell: node velocity gradient d_d u_c (Navier-Stokes only)
    double* Fd[3];    // NEQ x nface(a): diffusive flux at the midpoints (Navier-Stokes only)
};

__host__ __device__ inline long ncell_of(const Geom& g) { return (long)g.G[0] * g.G[1] * g.G[2]; }
__host__ __device__ inline long nface_of(const Geom& g, int a) {
    long r = 1;
    for (int d = 0; d < 3; d++) r *= (d == a) ? (g.n[d] + 3) : g.n[d];
    return r;
}
__host__ __device__ inline long ninterior_of(const Geom& g) { return (long)g.n[0] * g.n[1] * g.n[2]; }
// Midpoint set of the diffusive flux along a: faces -W .. n_a + W (W = 1, or 2 at sixth order).
__host__ __device__ inline long nface_w(const Geom& g, int a, int W) {
    long r = 1;
    for (int d = 0; d < 3; d++) r *= (d == a) ? (g.n[d] + 1 + 2 * W) : g.n[d];
    return r;
}

template <int DIM>
__device__ __forceinline__ long cidx(const Geom& g, int i, int j, int k) {
    const int gz = DIM == 3 ? g.gh : 0;
    return (long)(i + g.gh) + (long)(j + g.gh) * g.G[0] + (long)(k + gz) * g.G[0] * g.G[1];
}

template <int A>
__device__ __forceinline__ long fidx(const Geom& g, int i, int j, int k) {
    const int e0 = g.n[0] + (A == 0 ? 3 : 0);
    const int e1 = g.n[1] + (A == 1 ? 3 : 0);
    return (long)(i + (A == 0)) + (long)(j + (A == 1)) * e0 + (long)(k + (A == 2)) * e0 * e1;
}
// Index in the diffusive midpoint set of half-width W (W = 1 is fidx).
template <int A, int W>
__device__ __forceinline__ long dfidx(const Geom& g, int i, int j, int k) {
    const int e0 = g.n[0] + (A == 0 ? 1 + 2 * W : 0);
    const int e1 = g.n[1] + (A == 1 ? 1 + 2 * W : 0);
    return (long)(i + (A == 0 ? W : 0)) + (long)(j + (A == 1 ? W : 0)) * e0 + (long)(k + (A == 2 ? W : 0)) * e0 * e1;
}

// Counters reported by the face phase.
struct Counters {
    unsigned long long fallback;   // faces reverted to first order
    unsigned long long hllc_hll;   // faces using HLLC-HLL
};

// ---------------------------------------------------------------------------
// Phase 1: cells.  item in [0, ncell).
// ---------------------------------------------------------------------------
template <int DIM, int MODEL, int NSP>
__device__ __forceinline__ void cells_item(const Params& P, const Geom& g, const Comp& Q,
                                           const Scratch& S, long x) {
    using M = Model<DIM, MODEL, NSP>;
    const long nc = ncell_of(g);
    double q[M::NCOMP], V[M::NEQ], rho, cs;
#pragma unroll
    for (int e = 0; e < M::NCOMP; e++) q[e] = Q.p[e][x];
    cell_derived<DIM, MODEL, NSP>(P, q, V, rho, cs);
#pragma unroll
    for (int e = 0; e < M::NEQ; e++) S.V[e * nc + x] = V[e];
    S.rho[x] = rho;
    S.cs[x] = cs;
}

// ---------------------------------------------------------------------------
// Phase 2: sensor.  item over the interior grown by 2 (DerivativeFirstOrder
// 2nd order: (1/2*(u_R - u_L))/dx; WCNS56-HLLC-HLL.cpp:638-731, 3D :1440-1660).
// ---------------------------------------------------------------------------
template <int DIM, int MODEL, int NSP>
__device__ __forceinline__ void sensor_item(const Geom& g, const Scratch& S, long t) {
    using M = Model<DIM, MODEL, NSP>;
    const int e0 = g.n[0] + 4, e1 = g.n[1] + 4;
    const int i = (int)(t % e0) - 2;
    const int j = (int)((t / e0) % e1) - 2;
    const int k = DIM == 3 ? (int)(t / ((long)e0 * e1)) - 2 : 0;
    const long nc = ncell_of(g);
    const long x = cidx<DIM>(g, i, j, k);
    const long sx = 1, sy = g.G[0], sz = (long)g.G[0] * g.G[1];
    double du[3][3];
#pragma unroll
    for (int c = 0; c < DIM; c++) {
        const double* u = S.V + (M::IU + c) * nc;
        du[c][0] = (double(1)/double(2)*(u[x + sx] - u[x - sx]))/g.dx[0];
        du[c][1] = (double(1)/double(2)*(u[x + sy] - u[x - sy]))/g.dx[1];
        if (DIM == 3) du[c][2] = (double(1)/double(2)*(u[x + sz] - u[x - sz]))/g.dx[2];
    }
    if (DIM == 2) {
        S.theta[x] = du[0][0] + du[1][1];
        S.Omega[x] = fabs(du[1][0] - du[0][1]);
    } else {
        S.theta[x] = du[0][0] + du[1][1] + du[2][2];
        const double ox = du[2][1] - du[1][2];
        const double oy = du[0][2] - du[2][0];
        const double oz = du[1][0] - du[0][1];
        S.Omega[x] = sqrt(add_(add_(mul_(ox, ox), mul_(oy, oy)), mul_(oz, oz)));
    }
}

// ---------------------------------------------------------------------------
// Reconstruction + Riemann solve of one face from its characteristic stencil
// W (6 x NEQ): WCNS interpolation, inverse projection, bounds check with
// first-order fallback (WCNS56-HLLC-HLL.cpp:899-1032), HLLC / HLLC-HLL.
// Returns the bounds flag; `margin` is the relative distance to the nearest
// bound of the reconstructed states.
// ---------------------------------------------------------------------------
template <bool X, int DIM, int MODEL, int NSP, int SCHEME, int A>
__device__ __forceinline__ bool face_eval(const Params& P, const FaceProj<DIM, MODEL, NSP>& F,
                                          const double (&W)[6][Model<DIM, MODEL, NSP>::NEQ], const Scratch& S,
                                          long nc, long xL, long xR, bool use_hll, double rref, double pref,
                                          double* Fo, double& umid, double& margin) {
    using M = Model<DIM, MODEL, NSP>;
    constexpr int NEQ = M::NEQ;
    double Wm[NEQ], Wp[NEQ];
#pragma unroll
    for (int e = 0; e < NEQ; e++) {
        double U[6];
#pragma unroll
        for (int m = 0; m < 6; m++) U[m] = W[m][e];
        if constexpr (SCHEME == WCNS5_JS) js_pair<X>(U, P.p, Wm[e], Wp[e]);
        else if constexpr (SCHEME == WCNS6_LD) ld_pair<X>(U, P, Wm[e], Wp[e]);
        else if constexpr (SCHEME == WCNS5_Z) z_pair<X>(U, P.p, Wm[e], Wp[e]);
        else cu_pair<X, A>(U, P, Wm[e], Wp[e]);
    }
    double VL[NEQ], VR[NEQ];
    prim_from_char<X, DIM, MODEL, NSP, A>(F, Wm, VL);
    prim_from_char<X, DIM, MODEL, NSP, A>(F, Wp, VR);
    double mL, mR;
    const bool ok = face_bounded<DIM, MODEL, NSP>(P, VL, mL) & face_bounded<DIM, MODEL, NSP>(P, VR, mR);
    if constexpr (MODEL == SINGLE_SPECIES) {
        // relative margins: density against the projection density, pressure against the cell pressures
        mL = fmin(fabs(VL[0])/rref, fabs(VL[M::IP])/pref);
        mR = fmin(fabs(VR[0])/rref, fabs(VR[M::IP])/pref);
    } else if constexpr (MODEL == FOUR_EQN_CONSERVATIVE) {
        // add density and pressure, relative like the single-species model
        double rL = 0.0, rR = 0.0;
#pragma unroll
        for (int s = 0; s < NSP; s++) { rL += VL[s]; rR += VR[s]; }
        mL = fmin(mL, fmin(fabs(rL)/rref, fabs(VL[M::IP])/pref));
        mR = fmin(mR, fmin(fabs(rR)/rref, fabs(VR[M::IP])/pref));
    }
    margin = fmin(mL, mR);
    if (!ok) {
#pragma unroll
        for (int e = 0; e < NEQ; e++) {
            VL[e] = S.V[e * nc + xL];
            VR[e] = S.V[e * nc + xR];
        }
    }
    riemann<X, DIM, MODEL, NSP, A>(P, VL, VR, use_hll, Fo, umid);
    return ok;
}

// Ducros-like sensor of the face between cells xL and xR (WCNS56-HLLC-HLL.cpp:1066-1088),
// from the exact cell dilatation and vorticity: true where the face takes HLLC-HLL.
__device__ __forceinline__ bool face_uses_hll(const Scratch& S, long xL, long xR) {
    const double theta_avg = 0.5*(S.theta[xL] + S.theta[xR]);
    const double Omega_avg = 0.5*(S.Omega[xL] + S.Omega[xR]);
    const double s = -theta_avg/(fabs(theta_avg) + Omega_avg + HMR_EPS);
    return s > 0.65;
}

// ---------------------------------------------------------------------------
// Phase 3: one midpoint face normal to axis A.  item over faces(A).
//
// The exact form (X = true) is the reference's operation order.  The fast form
// (X = false) hands a face back (returns true) instead of computing it where
// the reference's own result is ill-conditioned, and the caller queues it for
// the exact form: HLLC-HLL faces (the blending weight sqrt(1 - alpha_1^2)
// amplifies rounding when the velocity jump is almost purely normal),
// first-order fallback faces, and faces whose reconstructed states lie within
// 1e-9 (relative) of a bounds threshold.  Every other face of the fast form is
// within rounding of the exact one.
// ---------------------------------------------------------------------------
template <bool X, int DIM, int MODEL, int NSP, int SCHEME, int A>
__device__ __forceinline__ bool face_item(const Params& P, const Geom& g, const Scratch& S, long t,
                                          Counters* cnt) {
    using M = Model<DIM, MODEL, NSP>;
    constexpr int NEQ = M::NEQ;
    const int e0 = g.n[0] + (A == 0 ? 3 : 0);
    const int e1 = g.n[1] + (A == 1 ? 3 : 0);
    const int i = (int)(t % e0) - (A == 0);
    const int j = (int)((t / e0) % e1) - (A == 1);
    const int k = DIM == 3 ? (int)(t / ((long)e0 * e1)) - (A == 2) : 0;
    const long nc = ncell_of(g);
    const long st = (A == 0) ? 1 : (A == 1 ? (long)g.G[0] : (long)g.G[0] * g.G[1]);
    const long xR = cidx<DIM>(g, i, j, k);      // cell on the + side of the face
    const long xL = xR - st;

    const bool use_hll = face_uses_hll(S, xL, xR);
    if (!X && use_hll) return true;

    // Projection means (SIMPLE averaging).
    FaceProj<DIM, MODEL, NSP> F;
    F.rb = double(1)/double(2)*(S.rho[xL] + S.rho[xR]);
    F.cb = double(1)/double(2)*(S.cs[xL] + S.cs[xR]);
    if constexpr (MODEL != SINGLE_SPECIES) {
#pragma unroll
        for (int q = 0; q < NSP; q++) F.zb[q] = double(1)/double(2)*(S.V[q * nc + xL] + S.V[q * nc + xR]);
    }
    face_proj_setup(F);

    // Characteristic variables at cells face-3 .. face+2.
    double W[6][NEQ];
#pragma unroll
    for (int m = 0; m < 6; m++) {
        double Vc[NEQ];
        const long x = xR + (m - 3) * st;
#pragma unroll
        for (int e = 0; e < NEQ; e++) Vc[e] = S.V[e * nc + x];
        char_from_prim<DIM, MODEL, NSP, A>(F, Vc, W[m]);
    }

    double pref = 1.0;
    if constexpr (MODEL != FIVE_EQN_ALLAIRE)
        pref = fmax(fabs(S.V[M::IP * nc + xL]), fabs(S.V[M::IP * nc + xR]));
    double Fo[NEQ], umid, margin;
    const bool ok = face_eval<X, DIM, MODEL, NSP, SCHEME, A>(P, F, W, S, nc, xL, xR, use_hll, F.rb, pref, Fo,
                                                             umid, margin);
    if (!X && (!ok || margin < 1.0e-9)) return true;

    const long nf = nface_of(g, A);
#pragma unroll
    for (int e = 0; e < NEQ; e++) S.Fm[A][e * nf + t] = Fo[e];
    if constexpr (MODEL == FIVE_EQN_ALLAIRE) S.um[A][t] = umid;

    if (cnt != nullptr) {
        const unsigned mask = __activemask();
        const unsigned fb = __ballot_sync(mask, !ok);
        const unsigned hh = __ballot_sync(mask, use_hll);
        const int lane = threadIdx.x & 31;
        if (lane == __ffs(mask) - 1) {
            if (fb) atomicAdd(&cnt->fallback, (unsigned long long)__popc(fb));
            if (hh) atomicAdd(&cnt->hllc_hll, (unsigned long long)__popc(hh));
        }
    }
    return false;
}

// Queue of faces the fast form hands to the exact form: entries are
// (axis << 56) | item, item being the face's index in the face phase.
struct Redo {
    unsigned long long* list;
    unsigned int* count;
    unsigned long long cap;
    // Optional (per-patch fast form): faces sorted before the fast pass -- the HLLC ones into
    // per-axis lists (axis a at fast + fast_off[a], fast_count[a] entries), the HLLC-HLL ones
    // (fast_count[3] of them) to the head of the queue above -- so that the fast pass runs full
    // warps beside the exact pass over the HLLC-HLL faces.
    unsigned long long* fast = nullptr;
    unsigned int* fast_count = nullptr;
    long fast_off[3] = {0, 0, 0};
};

__device__ __forceinline__ void redo_push(const Redo& R, int axis, long item) {
    const unsigned long long idx = atomicAdd(R.count, 1u);
    if (idx < R.cap) R.list[idx] = ((unsigned long long)axis << 56) | (unsigned long long)item;
}

// ---------------------------------------------------------------------------
// Phase 4: update of one interior cell.
// ---------------------------------------------------------------------------
}  // namespace hmr

#include "hmr_diffusive.cuh"

namespace hmr {

struct UpdateArgs {
    Comp Qint[3];        // stage states Q_int[0..nst-1] (ghost box); Qint[nst-1] is the current one
    double alpha[3];
    int nst;
    double beta;         // weight of the current stage's flux divergence + source
    double dt;
    Comp Qout;           // ghost-box arrays; interior written
    FluxComp Fout;       // optional: dt-scaled face fluxes, SAMRAI side layout (dim*NEQ arrays)
    Comp Sout;           // optional: source (interior, NEQ arrays), accumulated
    int dorder;          // 0: Euler; 2, 4 or 6: NavierStokes, the midpoint diffusive fluxes in S.Fd enter
};

// Node (cell-centre) flux of component e in direction A.
template <int DIM, int MODEL, int NSP, int A>
__device__ __forceinline__ double node_flux(const Scratch& S, const Comp& Q, long nc, long x, int e) {
    using M = Model<DIM, MODEL, NSP>;
    const double un = S.V[(M::IU + A) * nc + x];
    if constexpr (MODEL == SINGLE_SPECIES) {
        if (e == 0) return Q.p[1 + A][x];
        if (e <= DIM) {
            if (e - 1 == A) return un*Q.p[e][x] + S.V[M::IP * nc + x];
            return un*Q.p[e][x];
        }
        return un*(Q.p[DIM + 1][x] + S.V[M::IP * nc + x]);
    } else {
        if (e < NSP) return un*Q.p[e][x];
        if (e < NSP + DIM) {
            if (e - NSP == A) return un*Q.p[e][x] + S.V[M::IP * nc + x];
            return un*Q.p[e][x];
        }
        if (e == NSP + DIM) return un*(Q.p[e][x] + S.V[M::IP * nc + x]);
        return un*Q.p[e][x];
    }
}

// dt-scaled face flux of component e at face index fa (along A) of the face
// set, between cells xm (minus side) and xp (plus side).
template <int DIM, int MODEL, int NSP, int A>
__device__ __forceinline__ double face_flux(const Geom& g, const Scratch& S, const Comp& Q, double dt,
                                            long nc, long f, long fst, long xm, long xp, int e) {
    const long nf = nface_of(g, A);
    const double* Fm = S.Fm[A] + e * nf;
    return dt*(double(1)/double(30)*(Fm[f + fst] + Fm[f - fst]) -
               double(3)/double(10)*(node_flux<DIM, MODEL, NSP, A>(S, Q, nc, xp, e) +
                                     node_flux<DIM, MODEL, NSP, A>(S, Q, nc, xm, e)) +
               double(23)/double(15)*Fm[f]);
}

template <int DIM, int A>
__device__ __forceinline__ long side_idx(const Geom& g, int i, int j, int k) {
    const int e0 = g.n[0] + (A == 0);
    const int e1 = g.n[1] + (A == 1);
    return (long)i + (long)j * e0 + (long)k * e0 * e1;
}

template <int DIM, int MODEL, int NSP, int A>
__device__ __forceinline__ void axis_terms(const Geom& g, const Scratch& S, const Comp& Q, const UpdateArgs& U,
                                           int i, int j, int k, long x, long nc,
                                           double (&fl)[Model<DIM, MODEL, NSP>::NEQ],
                                           double (&fr)[Model<DIM, MODEL, NSP>::NEQ],
                                           double& usrc) {
    using M = Model<DIM, MODEL, NSP>;
    const long st = (A == 0) ? 1 : (A == 1 ? (long)g.G[0] : (long)g.G[0] * g.G[1]);
    const long fst = (A == 0) ? 1 : (A == 1 ? (long)g.n[0] : (long)g.n[0] * g.n[1]);
    const long f = fidx<A>(g, i, j, k);
#pragma unroll
    for (int e = 0; e < M::NEQ; e++) {
        fl[e] = face_flux<DIM, MODEL, NSP, A>(g, S, Q, U.dt, nc, f, fst, x - st, x, e);
        fr[e] = face_flux<DIM, MODEL, NSP, A>(g, S, Q, U.dt, nc, f + fst, fst, x, x + st, e);
    }
    if (U.Fout.p[0] != nullptr) {
        const int ii[3] = {i, j, k};
#pragma unroll
        for (int e = 0; e < M::NEQ; e++) {
            U.Fout.p[A * M::NEQ + e][side_idx<DIM, A>(g, i, j, k)] = fl[e];
            if (ii[A] == g.n[A] - 1)
                U.Fout.p[A * M::NEQ + e][side_idx<DIM, A>(g, i + (A == 0), j + (A == 1), k + (A == 2))] = fr[e];
        }
    }
    if constexpr (MODEL == FIVE_EQN_ALLAIRE) {
        // WCNS56-HLLC-HLL.cpp:1288-1369: (3/2 (u~_R - u~_L) - 3/10 (u_{+1} - u_{-1}) + 1/30 (u~_RR - u~_LL))/dx
        const double* um = S.um[A];
        const double* u = S.V + (M::IU + A) * nc;
        usrc = (double(3)/double(2)*(um[f + fst] - um[f]) -
                double(3)/double(10)*(u[x + st] - u[x - st]) +
                double(1)/double(30)*(um[f + 2 * fst] - um[f - fst]))/g.dx[A];
    } else {
        usrc = 0.0;
    }
}

// LOCAL: U is a per-item local copy (batched form); its stage arrays are then selected with
// constant indices only, since a runtime index into it would put it in local memory.  A
// kernel-parameter U (per-patch launches) is indexed directly.
template <int DIM, int MODEL, int NSP, bool LOCAL = false>
__device__ __forceinline__ void update_item(const Geom& g, const Scratch& S, const UpdateArgs& U, long t) {
    using M = Model<DIM, MODEL, NSP>;
    constexpr int NEQ = M::NEQ;
    const int i = (int)(t % g.n[0]);
    const int j = (int)((t / g.n[0]) % g.n[1]);
    const int k = DIM == 3 ? (int)(t / ((long)g.n[0] * g.n[1])) : 0;
    const long nc = ncell_of(g);
    const long x = cidx<DIM>(g, i, j, k);
    Comp Qsel;
    if constexpr (LOCAL) {
#pragma unroll
        for (int e = 0; e < M::NCOMP; e++)
            Qsel.p[e] = U.nst == 1 ? U.Qint[0].p[e] : (U.nst == 2 ? U.Qint[1].p[e] : U.Qint[2].p[e]);
    }
    const Comp& Q = LOCAL ? Qsel : U.Qint[U.nst - 1];

    double fl[3][NEQ], fr[3][NEQ], us[3];
    axis_terms<DIM, MODEL, NSP, 0>(g, S, Q, U, i, j, k, x, nc, fl[0], fr[0], us[0]);
    axis_terms<DIM, MODEL, NSP, 1>(g, S, Q, U, i, j, k, x, nc, fl[1], fr[1], us[1]);
    if constexpr (DIM == 3) axis_terms<DIM, MODEL, NSP, 2>(g, S, Q, U, i, j, k, x, nc, fl[2], fr[2], us[2]);

    double src[NEQ];
#pragma unroll
    for (int e = 0; e < NEQ; e++) src[e] = 0.0;
    if constexpr (MODEL == FIVE_EQN_ALLAIRE) {
        double sum = us[0] + us[1];
        if constexpr (DIM == 3) sum = sum + us[2];
#pragma unroll
        for (int s = 0; s < NSP - 1; s++) {
            const int e = M::IZ + s;
            src[e] = U.dt*Q.p[e][x]*(sum);
        }
    }
    const long is = (long)i + (long)j * g.n[0] + (long)k * g.n[0] * g.n[1];
    if (U.Sout.p[0] != nullptr) {
#pragma unroll
        for (int e = 0; e < NEQ; e++) U.Sout.p[e][is] += src[e];
    }

    if (U.Qout.p[0] == nullptr) return;   // flux/source only (computeConvectiveFluxAndSourceOnPatch)

    // NavierStokes: diffusive face fluxes of the current stage (single species).
    double dl[3][NEQ], dr[3][NEQ];
    bool ns = false;
    if constexpr (MODEL == SINGLE_SPECIES) {
        if (U.beta != 0.0 && U.dorder == 6) { diff_cell_faces<DIM, 6, NEQ>(g, S, U.dt, i, j, k, dl, dr); ns = true; }
        else if (U.beta != 0.0 && U.dorder == 4) { diff_cell_faces<DIM, 4, NEQ>(g, S, U.dt, i, j, k, dl, dr); ns = true; }
        else if (U.beta != 0.0 && U.dorder == 2) { diff_cell_faces<DIM, 2, NEQ>(g, S, U.dt, i, j, k, dl, dr); ns = true; }
    }

    // Euler::advanceSingleStepOnPatch (Euler.cpp:1188-1660): Q = 0, += alpha_n Q_n, += beta (div + S);
    // NavierStokes::advanceSingleStepOnPatch (NavierStokes.cpp:1743-1749, 2085-2092) adds the
    // diffusive fluxes to the divergence.
    // x/dx: the reference's division in the exact form, a product with the reciprocal in the fast one.
    double rdx[3] = {0.0, 0.0, 0.0};
    if constexpr (HMR_FAST != 0) {
#pragma unroll
        for (int a = 0; a < DIM; a++) rdx[a] = double(1)/g.dx[a];
    }
    auto ddx = [&](double v, int a) { return HMR_FAST != 0 ? v*rdx[a] : v/g.dx[a]; };
    double qn[NEQ];
#pragma unroll
    for (int e = 0; e < NEQ; e++) {
        double acc = 0.0;
        if constexpr (LOCAL) {
#pragma unroll
            for (int n = 0; n < 3; n++)
                if (n < U.nst && U.alpha[n] != 0.0) acc += U.alpha[n]*U.Qint[n].p[e][x];
        } else {
            for (int n = 0; n < U.nst; n++)
                if (U.alpha[n] != 0.0) acc += U.alpha[n]*U.Qint[n].p[e][x];
        }
        if (U.beta != 0.0 && ns) {
            if constexpr (DIM == 2) {
                acc += U.beta*(-ddx(fr[0][e] - fl[0][e] + dr[0][e] - dl[0][e], 0) -
                               ddx(fr[1][e] - fl[1][e] + dr[1][e] - dl[1][e], 1) + (0.0 + src[e]));
            } else {
                acc += U.beta*(-ddx(fr[0][e] - fl[0][e] + dr[0][e] - dl[0][e], 0) -
                               ddx(fr[1][e] - fl[1][e] + dr[1][e] - dl[1][e], 1) -
                               ddx(fr[2][e] - fl[2][e] + dr[2][e] - dl[2][e], 2) + (0.0 + src[e]));
            }
        } else if (U.beta != 0.0) {
            if constexpr (DIM == 2) {
                acc += U.beta*(-ddx(fr[0][e] - fl[0][e], 0) - ddx(fr[1][e] - fl[1][e], 1) + (0.0 + src[e]));
            } else {
                acc += U.beta*(-ddx(fr[0][e] - fl[0][e], 0) - ddx(fr[1][e] - fl[1][e], 1) -
                               ddx(fr[2][e] - fl[2][e], 2) + (0.0 + src[e]));
            }
        }
        qn[e] = acc;
        U.Qout.p[e][x] = acc;
    }
    if constexpr (MODEL == FIVE_EQN_ALLAIRE) {
        // FlowModelFiveEqnAllaire::updateCellDataOfConservativeVariables (:1739-1890)
        if (U.beta != 0.0) {
            double zl = 1.0;
#pragma unroll
            for (int s = 0; s < NSP - 1; s++) zl -= qn[M::IZ + s];
            U.Qout.p[M::NCOMP - 1][x] = zl;
        }
    }
}

// ---------------------------------------------------------------------------
// Ghost fill of a single patch, per axis: mode 0 zero-gradient, 1 periodic,
// 2 provided by the caller (left untouched: neighbour copies, coarse-fine
// interpolation or analytic values), 3 reflecting wall, 5 symmetry plane (the
// mirror image without a sign change), 4 Dirichlet (the
// side's constant values bv[(2 axis + side) ncomp + e],
// BasicCartesianBoundaryUtilities2.cpp:150-165).  A ghost cell beyond a
// Dirichlet side takes that side's values -- beyond two Dirichlet sides, those
// of the lower axis (the reference's corner conditions XDIRICHLET / YDIRICHLET
// name the axis whose values a corner takes, :679-710) -- unless it lies beyond
// a provided side.  item over the ghost box (interior items skip).
// ---------------------------------------------------------------------------
template <int DIM>
__device__ __forceinline__ void fill_item(const Geom& g, const Comp& Q, int ncomp, const int* periodic, long x,
                                          int mom0, const double* bv) {
    int c[3];
    c[0] = (int)(x % g.G[0]) - g.gh;
    c[1] = (int)((x / g.G[0]) % g.G[1]) - g.gh;
    c[2] = DIM == 3 ? (int)(x / ((long)g.G[0] * g.G[1])) - g.gh : 0;
    bool inside = true;
    int s[3];
    int flip = -1, flip2 = -1, flip3 = -1;   // momentum components negated by reflecting walls
    int dside = -1;                          // Dirichlet side (2 axis + high) whose values the cell takes
#pragma unroll
    for (int a = 0; a < 3; a++) {
        s[a] = c[a];
        if (a >= DIM) continue;
        if (c[a] < 0 || c[a] >= g.n[a]) {
            if (periodic[a] == 2) return;
            inside = false;
            if (periodic[a] == 4) {
                if (dside < 0) dside = 2 * a + (c[a] >= 0);
            } else if (periodic[a] == 1) {
                s[a] = ((c[a] % g.n[a]) + g.n[a]) % g.n[a];
            } else if (periodic[a] == 3 || periodic[a] == 5) {
                // reflecting wall: mirror image across the boundary face
                // (BasicCartesianBoundaryUtilities2.cpp:349-440), normal momentum negated;
                // symmetry plane (:397-440 for every variable): the mirror image as it is
                s[a] = c[a] < 0 ? -c[a] - 1 : 2 * g.n[a] - 1 - c[a];
                if (periodic[a] == 3) {
                    if (flip < 0) flip = mom0 + a;
                    else if (flip2 < 0) flip2 = mom0 + a;
                    else flip3 = mom0 + a;
                }
            } else {
                s[a] = c[a] < 0 ? 0 : g.n[a] - 1;
            }
        }
    }
    if (inside) return;
    if (dside >= 0) {
        for (int e = 0; e < ncomp; e++) Q.p[e][x] = bv[dside * ncomp + e];
        return;
    }
    const long y = cidx<DIM>(g, s[0], s[1], s[2]);
    for (int e = 0; e < ncomp; e++) {
        const double v = Q.p[e][y];
        Q.p[e][x] = (e == flip || e == flip2 || e == flip3) ? -v : v;
    }
}

// Physical boundaries of the level's domain for a patch with known position: ghost cell c
// (local) of a patch at level index lo, outside the domain along an axis, takes the value of
// the nearest in-domain cell (zero-gradient, dom_periodic 0) or of its mirror image across the
// domain face with the normal momentum negated (reflecting wall, dom_periodic 3) -- the patch's
// own interior or a ghost cell filled from a neighbour before -- or, beyond a Dirichlet face
// (dom_periodic 4), that face's values (the lower axis's beyond two, as fill_item).  Ghost
// cells inside the domain are left alone (neighbour copies or provided values).
template <int DIM>
__device__ __forceinline__ void domain_fill_item(const Geom& g, const Comp& Q, int ncomp, const int* lo,
                                                 const int* dom, const int* dom_periodic, long x, int mom0,
                                                 const double* bv) {
    int c[3], s[3];
    c[0] = (int)(x % g.G[0]) - g.gh;
    c[1] = (int)((x / g.G[0]) % g.G[1]) - g.gh;
    c[2] = DIM == 3 ? (int)(x / ((long)g.G[0] * g.G[1])) - g.gh : 0;
    bool physical = false;
    int flip = -1, flip2 = -1, flip3 = -1;
    int dside = -1;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        s[a] = c[a];
        if (a >= DIM || dom_periodic[a] == 1) continue;
        const int G = lo[a] + c[a];
        if (G >= 0 && G < dom[a]) continue;
        physical = true;
        if (dom_periodic[a] == 4) {
            if (dside < 0) dside = 2 * a + (G >= 0);
        } else if (dom_periodic[a] == 3 || dom_periodic[a] == 5) {
            // reflecting wall or symmetry plane: mirror image across the domain face, in the
            // level's index space (the normal momentum negated at a reflecting wall)
            s[a] = (G < 0 ? -G - 1 : 2 * dom[a] - 1 - G) - lo[a];
            if (dom_periodic[a] == 3) {
                if (flip < 0) flip = mom0 + a;
                else if (flip2 < 0) flip2 = mom0 + a;
                else flip3 = mom0 + a;
            }
        } else {
            s[a] = G < 0 ? -lo[a] : dom[a] - 1 - lo[a];
        }
    }
    if (!physical) return;
    if (dside >= 0) {
        for (int e = 0; e < ncomp; e++) Q.p[e][x] = bv[dside * ncomp + e];
        return;
    }
    const long y = cidx<DIM>(g, s[0], s[1], s[2]);
    for (int e = 0; e < ncomp; e++) {
        const double v = Q.p[e][y];
        Q.p[e][x] = (e == flip || e == flip2 || e == flip3) ? -v : v;
    }
}

}  // namespace hmr
