// C entry points of the CPU oracle (test infrastructure only; see hmr_oracle.hpp).
// All arrays are contiguous FP64 buffers in SAMRAI layout:
//   state  : ncomp x ghost box (ghost width 4, x fastest)
//   flux   : for axis a = 0..dim-1: neq x (n grown by one along a), concatenated
//   source : neq x interior
#include "hmr_oracle.hpp"

#include <thread>
#include <vector>

using namespace hmro;

extern "C" {

static Config to_cfg(const hmro_config* c) { return hmro_to_config(c); }

static long flux_len(const Config& c, const Box& b) {
    const int neq = num_eqn(c);
    long t = 0;
    for (int a = 0; a < c.dim; a++)
        t += (long)neq * (b.n[0] + (a == 0)) * (b.n[1] + (a == 1)) * (b.n[2] + (a == 2));
    return t;
}

static void flux_ptrs(const Config& c, const Box& b, double* flux, std::vector<double*>& out) {
    const int neq = num_eqn(c);
    out.clear();
    double* p = flux;
    for (int a = 0; a < c.dim; a++) {
        const long nfa = (long)(b.n[0] + (a == 0)) * (b.n[1] + (a == 1)) * (b.n[2] + (a == 2));
        for (int e = 0; e < neq; e++) { out.push_back(p); p += nfa; }
    }
}

int hmro_num_eqn(const hmro_config* cfg) { return num_eqn(to_cfg(cfg)); }
int hmro_num_comp(const hmro_config* cfg) { return num_comp(to_cfg(cfg)); }

// computeConvectiveFluxAndSourceOnPatch for one patch.  source is accumulated.
int hmro_conv_flux_source(const hmro_config* cfg, const int* n, const double* dx, double dt,
                          const double* Q, double* flux, double* source, long* stats) {
    const Config c = to_cfg(cfg);
    const Box b = make_box(c.dim, n, c.ghosts);
    const int ncomp = num_comp(c), neq = num_eqn(c);
    std::vector<const double*> q(ncomp);
    for (int e = 0; e < ncomp; e++) q[e] = Q + (size_t)e * b.ncell();
    std::vector<double*> f;
    flux_ptrs(c, b, flux, f);
    const long nint = (long)b.n[0] * b.n[1] * b.n[2];
    std::vector<double*> s(neq);
    for (int e = 0; e < neq; e++) s[e] = source + (size_t)e * nint;
    Stats st{0, 0, 0};
    conv_flux_source<double>(c, n, dx, dt, q.data(), f.data(), s.data(), &st);
    if (stats) { stats[0] = st.faces; stats[1] = st.fallback; stats[2] = st.hllc_hll; }
    return 0;
}

// advanceSingleStepOnPatch for one stage with nstages (alpha, beta, gamma)
// coefficients.  Q_int, F_int, S_int hold nstages consecutive blocks.
int hmro_rk_stage(const hmro_config* cfg, const int* n, const double* dx, int nstages,
                  const double* alpha, const double* beta, const double* gamma,
                  const double* Q_int, const double* F_int, const double* S_int,
                  double* Q_out, double* F_acc, double* S_acc) {
    const Config c = to_cfg(cfg);
    const Box b = make_box(c.dim, n, c.ghosts);
    const int ncomp = num_comp(c), neq = num_eqn(c);
    const long nint = (long)b.n[0] * b.n[1] * b.n[2];
    const long fl = flux_len(c, b);
    std::vector<std::vector<const double*>> qi(nstages), fi(nstages), si(nstages);
    std::vector<const double* const*> qp(nstages), fp(nstages), sp(nstages);
    for (int s = 0; s < nstages; s++) {
        for (int e = 0; e < ncomp; e++) qi[s].push_back(Q_int + (size_t)s * ncomp * b.ncell() + (size_t)e * b.ncell());
        std::vector<double*> f;
        flux_ptrs(c, b, const_cast<double*>(F_int + (size_t)s * fl), f);
        for (double* p : f) fi[s].push_back(p);
        for (int e = 0; e < neq; e++) si[s].push_back(S_int + (size_t)s * neq * nint + (size_t)e * nint);
        qp[s] = qi[s].data(); fp[s] = fi[s].data(); sp[s] = si[s].data();
    }
    std::vector<double*> qo(ncomp);
    for (int e = 0; e < ncomp; e++) qo[e] = Q_out + (size_t)e * b.ncell();
    std::vector<double*> fa, sa;
    if (F_acc) flux_ptrs(c, b, F_acc, fa);
    if (S_acc) for (int e = 0; e < neq; e++) sa.push_back(S_acc + (size_t)e * nint);
    rk_stage<double>(c, n, dx, nstages, alpha, beta, gamma, qp.data(), fp.data(), sp.data(),
                     qo.data(), F_acc ? fa.data() : nullptr, S_acc ? sa.data() : nullptr);
    return 0;
}

// DiffusiveFluxReconstructorMidpoint::computeDiffusiveFluxOnPatch for one
// single-species patch (flux overwritten, dt-scaled, same layout as the convective flux).
int hmro_diff_flux(const hmro_config* cfg, const hmro_transport* tr, const int* n, const double* dx, double dt,
                   const double* Q, double* flux) {
    const Config c = to_cfg(cfg);
    if (c.model != MODEL_SINGLE_SPECIES || (tr->order != 2 && tr->order != 4 && tr->order != 6)) return -1;
    if (tr->order == 6 && c.ghosts < 5) return -1;
    const Box b = make_box(c.dim, n, c.ghosts);
    const int ncomp = num_comp(c);
    std::vector<const double*> q(ncomp);
    for (int e = 0; e < ncomp; e++) q[e] = Q + (size_t)e * b.ncell();
    std::vector<double*> f;
    flux_ptrs(c, b, flux, f);
    diff_flux<double>(c, hmro_to_transport(tr), n, dx, dt, q.data(), f.data());
    return 0;
}

// NavierStokes::advanceSingleStepOnPatch: hmro_rk_stage with the diffusive
// fluxes Fd_int (same blocks as F_int) entering the divergence.
int hmro_rk_stage_ns(const hmro_config* cfg, const int* n, const double* dx, int nstages,
                     const double* alpha, const double* beta, const double* gamma,
                     const double* Q_int, const double* F_int, const double* Fd_int, const double* S_int,
                     double* Q_out) {
    const Config c = to_cfg(cfg);
    const Box b = make_box(c.dim, n, c.ghosts);
    const int ncomp = num_comp(c), neq = num_eqn(c);
    const long nint = (long)b.n[0] * b.n[1] * b.n[2];
    const long fl = flux_len(c, b);
    std::vector<std::vector<const double*>> qi(nstages), fi(nstages), di(nstages), si(nstages);
    std::vector<const double* const*> qp(nstages), fp(nstages), dp(nstages), sp(nstages);
    for (int s = 0; s < nstages; s++) {
        for (int e = 0; e < ncomp; e++) qi[s].push_back(Q_int + (size_t)s * ncomp * b.ncell() + (size_t)e * b.ncell());
        std::vector<double*> f;
        flux_ptrs(c, b, const_cast<double*>(F_int + (size_t)s * fl), f);
        for (double* p : f) fi[s].push_back(p);
        flux_ptrs(c, b, const_cast<double*>(Fd_int + (size_t)s * fl), f);
        for (double* p : f) di[s].push_back(p);
        for (int e = 0; e < neq; e++) si[s].push_back(S_int + (size_t)s * neq * nint + (size_t)e * nint);
        qp[s] = qi[s].data(); fp[s] = fi[s].data(); dp[s] = di[s].data(); sp[s] = si[s].data();
    }
    std::vector<double*> qo(ncomp);
    for (int e = 0; e < ncomp; e++) qo[e] = Q_out + (size_t)e * b.ncell();
    rk_stage<double>(c, n, dx, nstages, alpha, beta, gamma, qp.data(), fp.data(), sp.data(),
                     qo.data(), nullptr, nullptr, dp.data());
    return 0;
}

// Euler / NavierStokes synchronizeFluxes on one coarse patch (Fd null for Euler): Q (ghost
// box, interior updated) += -div (F [+ Fd]) + S with the time-integrated fluxes.
int hmro_sync_fluxes(const hmro_config* cfg, const int* n, const double* dx, const double* F,
                     const double* Fd, const double* S, double* Q) {
    const Config c = to_cfg(cfg);
    const Box b = make_box(c.dim, n, c.ghosts);
    const int ncomp = num_comp(c), neq = num_eqn(c);
    const long nint = (long)b.n[0] * b.n[1] * b.n[2];
    std::vector<double*> f, d, q(ncomp);
    flux_ptrs(c, b, const_cast<double*>(F), f);
    if (Fd) flux_ptrs(c, b, const_cast<double*>(Fd), d);
    std::vector<const double*> fc(f.begin(), f.end()), dc(d.begin(), d.end()), sc(neq);
    for (int e = 0; e < neq; e++) sc[e] = S + (size_t)e * nint;
    for (int e = 0; e < ncomp; e++) q[e] = Q + (size_t)e * b.ncell();
    sync_fluxes<double>(c, n, dx, fc.data(), Fd ? dc.data() : nullptr, sc.data(), q.data());
    return 0;
}

// Flux-sum coarsening of one fine patch onto one coarse patch (flux arrays as hmro_conv_flux_source's).
int hmro_coarsen_fluxsum(const hmro_config* cfg, const int* ratio, const int* cn, const int* clo, const int* fn,
                         const int* flo, const double* Ff, double* Fc) {
    const Config c = to_cfg(cfg);
    std::vector<double*> ff, fc;
    flux_ptrs(c, make_box(c.dim, fn, c.ghosts), const_cast<double*>(Ff), ff);
    flux_ptrs(c, make_box(c.dim, cn, c.ghosts), Fc, fc);
    std::vector<const double*> ffc(ff.begin(), ff.end());
    coarsen_fluxsum(c, ratio, cn, clo, fn, flo, ffc.data(), fc.data());
    return 0;
}

// Coarsening of a fine patch's interior onto the covered cells of a coarse patch (ghost boxes).
int hmro_coarsen_cells(const hmro_config* cfg, const int* ratio, const int* cn, const int* clo, const int* fn,
                       const int* flo, const double* Qf, double* Qc) {
    const Config c = to_cfg(cfg);
    const int ncomp = num_comp(c);
    const Box cb = make_box(c.dim, cn, c.ghosts), fb = make_box(c.dim, fn, c.ghosts);
    std::vector<const double*> qf(ncomp);
    std::vector<double*> qc(ncomp);
    for (int e = 0; e < ncomp; e++) { qf[e] = Qf + (size_t)e * fb.ncell(); qc[e] = Qc + (size_t)e * cb.ncell(); }
    coarsen_cells(c, ratio, cn, clo, fn, flo, qf.data(), qc.data());
    return 0;
}

// Coarse-fine ghost cells of a fine patch from a coarse patch at the time fraction theta.
int hmro_refine_ghosts(const hmro_config* cfg, const int* ratio, const int* fn, const int* flo, const int* cn,
                       const int* clo, const double* Qc_old, const double* Qc_new, double theta, double* Qf) {
    const Config c = to_cfg(cfg);
    const int ncomp = num_comp(c);
    const Box cb = make_box(c.dim, cn, c.ghosts), fb = make_box(c.dim, fn, c.ghosts);
    std::vector<const double*> qo(ncomp), qn(ncomp);
    std::vector<double*> qf(ncomp);
    for (int e = 0; e < ncomp; e++) {
        qo[e] = Qc_old + (size_t)e * cb.ncell();
        qn[e] = Qc_new + (size_t)e * cb.ncell();
        qf[e] = Qf + (size_t)e * fb.ncell();
    }
    refine_ghosts(c, ratio, fn, flo, cn, clo, qo.data(), qn.data(), theta, qf.data());
    return 0;
}

int hmro_fill_ghosts(const hmro_config* cfg, const int* n, const int* periodic, double* Q) {
    const Config c = to_cfg(cfg);
    const Box b = make_box(c.dim, n, c.ghosts);
    std::vector<double*> q(num_comp(c));
    for (int e = 0; e < num_comp(c); e++) q[e] = Q + (size_t)e * b.ncell();
    fill_ghosts<double>(c, n, periodic, q.data());
    return 0;
}

// As hmro_fill_ghosts, with the values of DIRICHLET sides (mode 4): bvals[(2 axis + high) ncomp + e].
int hmro_fill_ghosts_bv(const hmro_config* cfg, const int* n, const int* periodic, const double* bvals, double* Q) {
    const Config c = to_cfg(cfg);
    const Box b = make_box(c.dim, n, c.ghosts);
    std::vector<double*> q(num_comp(c));
    for (int e = 0; e < num_comp(c); e++) q[e] = Q + (size_t)e * b.ncell();
    fill_ghosts<double>(c, n, periodic, q.data(), bvals);
    return 0;
}

// SSPRK(3,3) weights, RungeKuttaLevelIntegrator.cpp:3909-3927.
static const double RK3_ALPHA[3][3] = {{1.0, 0, 0}, {3.0/4.0, 1.0/4.0, 0}, {1.0/3.0, 0.0, 2.0/3.0}};
static const double RK3_BETA[3][3]  = {{1.0, 0, 0}, {0.0, 1.0/4.0, 0}, {0.0, 0.0, 2.0/3.0}};
static const double RK3_GAMMA[3][3] = {{1.0/6.0, 0, 0}, {0.0, 1.0/6.0, 0}, {0.0, 0.0, 2.0/3.0}};

// One patch advanced by nsteps SSPRK3 steps with ghost fill before every
// stage (the stage loop of RungeKuttaLevelIntegrator::advanceLevel,
// RungeKuttaLevelIntegrator.cpp:1672-1748).  Q holds the ghost box and is
// updated in place (interior; ghosts are refilled).
int hmro_rk3_advance_bv(const hmro_config* cfg, const int* n, const double* dx, double dt,
                        const int* periodic, const double* bvals, int nsteps, double* Q, long* stats);

int hmro_rk3_advance(const hmro_config* cfg, const int* n, const double* dx, double dt,
                     const int* periodic, int nsteps, double* Q, long* stats) {
    return hmro_rk3_advance_bv(cfg, n, dx, dt, periodic, nullptr, nsteps, Q, stats);
}

// As hmro_rk3_advance, with the values of DIRICHLET sides (hmro_fill_ghosts_bv).
int hmro_rk3_advance_bv(const hmro_config* cfg, const int* n, const double* dx, double dt,
                        const int* periodic, const double* bvals, int nsteps, double* Q, long* stats) {
    const Config c = to_cfg(cfg);
    const Box b = make_box(c.dim, n, c.ghosts);
    const int ncomp = num_comp(c), neq = num_eqn(c);
    const long nint = (long)b.n[0] * b.n[1] * b.n[2];
    const long fl = flux_len(c, b);
    const size_t qs = (size_t)ncomp * b.ncell();
    std::vector<double> Qint(3 * qs), Fint(3 * fl), Sint(3 * (size_t)neq * nint), Qout(qs);
    long tot[3] = {0, 0, 0};
    for (int step = 0; step < nsteps; step++) {
        for (int sn = 0; sn < 3; sn++) {
            // copyTimeDependentData(scratch -> intermediate[sn]) + ghost fill
            std::copy(Q, Q + qs, Qint.begin() + sn * qs);
            hmro_fill_ghosts_bv(cfg, n, periodic, bvals, Qint.data() + sn * qs);
            std::fill(Sint.begin() + sn * (size_t)neq * nint, Sint.begin() + (sn + 1) * (size_t)neq * nint, 0.0);
            long st[3];
            hmro_conv_flux_source(cfg, n, dx, dt, Qint.data() + sn * qs, Fint.data() + sn * fl,
                                  Sint.data() + sn * (size_t)neq * nint, st);
            for (int i = 0; i < 3; i++) tot[i] += st[i];
            hmro_rk_stage(cfg, n, dx, sn + 1, RK3_ALPHA[sn], RK3_BETA[sn], RK3_GAMMA[sn],
                          Qint.data(), Fint.data(), Sint.data(), Qout.data(), nullptr, nullptr);
            std::copy(Qout.begin(), Qout.end(), Q);
        }
        hmro_fill_ghosts_bv(cfg, n, periodic, bvals, Q);
    }
    if (stats) for (int i = 0; i < 3; i++) stats[i] = tot[i];
    (void)neq;
    return 0;
}

// The same SSPRK3 loop for NavierStokes: convective + diffusive fluxes.
int hmro_ns_rk3_advance(const hmro_config* cfg, const hmro_transport* tr, const int* n, const double* dx,
                        double dt, const int* periodic, int nsteps, double* Q) {
    const Config c = to_cfg(cfg);
    const Box b = make_box(c.dim, n, c.ghosts);
    const int ncomp = num_comp(c), neq = num_eqn(c);
    const long nint = (long)b.n[0] * b.n[1] * b.n[2];
    const long fl = flux_len(c, b);
    const size_t qs = (size_t)ncomp * b.ncell();
    std::vector<double> Qint(3 * qs), Fint(3 * fl), Dint(3 * fl), Sint(3 * (size_t)neq * nint), Qout(qs);
    for (int step = 0; step < nsteps; step++) {
        for (int sn = 0; sn < 3; sn++) {
            std::copy(Q, Q + qs, Qint.begin() + sn * qs);
            hmro_fill_ghosts(cfg, n, periodic, Qint.data() + sn * qs);
            std::fill(Sint.begin() + sn * (size_t)neq * nint, Sint.begin() + (sn + 1) * (size_t)neq * nint, 0.0);
            hmro_conv_flux_source(cfg, n, dx, dt, Qint.data() + sn * qs, Fint.data() + sn * fl,
                                  Sint.data() + sn * (size_t)neq * nint, nullptr);
            const int r = hmro_diff_flux(cfg, tr, n, dx, dt, Qint.data() + sn * qs, Dint.data() + sn * fl);
            if (r) return r;
            hmro_rk_stage_ns(cfg, n, dx, sn + 1, RK3_ALPHA[sn], RK3_BETA[sn], RK3_GAMMA[sn],
                             Qint.data(), Fint.data(), Dint.data(), Sint.data(), Qout.data());
            std::copy(Qout.begin(), Qout.end(), Q);
        }
        hmro_fill_ghosts(cfg, n, periodic, Q);
    }
    return 0;
}

// Euler::computeSpectralRadiusesAndStableDtOnPatch (Euler.cpp:489-900) for one
// patch: max over the cells of the ghost box (the reference's loops run from
// -num_ghosts to n + num_ghosts, Euler.cpp:699-736, 841-880) of sum_d (|u_d| + c)/dx_d (max
// wave speed |u_d| + c, FlowModelSingleSpecies.cpp:3959 and the other models'
// analogues); the stable dt is 1/max.  With tr non-null, NavierStokes's
// (NavierStokes.cpp:595-1100, diffusive radius :884, :1074, dt :893, :1085): the max also
// covers 2 max_d(D/dx_d^2) with D = max(mu/rho, mu_v/rho, kappa/(rho c_p))
// (FlowModelSingleSpecies.cpp:4569-4573), and the stable dt is 1/(max + eps).
double hmro_spectral_radius_ns(const hmro_config* cfg, const hmro_transport* tr, const int* n, const double* dx,
                               const double* Q) {
    const Config c = to_cfg(cfg);
    const Box b = make_box(c.dim, n, c.ghosts);
    const int ncomp = num_comp(c);
    std::vector<const double*> q(ncomp);
    for (int e = 0; e < ncomp; e++) q[e] = Q + (size_t)e * b.ncell();
    Derived<double> D;
    compute_derived(c, b, q.data(), D);
    const int iu = vel_index(c);
    const long nc = b.ncell();
    double m = 0.0, md = 0.0;
    for (long x = 0; x < nc; x++) {
        double s = (std::fabs(D.V[(size_t)iu * nc + x]) + D.cs[x])/dx[0];
        for (int d = 1; d < c.dim; d++) s = s + (std::fabs(D.V[(size_t)(iu + d) * nc + x]) + D.cs[x])/dx[d];
        m = std::fmax(m, s);
        if (tr) {
            const double rho = D.V[x];
            const double c_p = c.gamma[0]/(c.gamma[0] - double(1))*c.R[0];
            const double kappa = tr->c_p*tr->mu_kappa/tr->Pr;
            double Dm = std::fmax(tr->mu/rho, tr->mu_v/rho);
            Dm = std::fmax(Dm, kappa/(rho*c_p));
            double r = Dm/(dx[0]*dx[0]);
            if (c.dim == 2) r = std::fmax(r, Dm/(dx[1]*dx[1]));
            else r = std::fmax(r, std::fmax(Dm/(dx[1]*dx[1]), Dm/(dx[2]*dx[2])));
            md = std::fmax(md, double(2)*r);
        }
    }
    return tr ? std::fmax(md, m) : m;
}

double hmro_spectral_radius(const hmro_config* cfg, const int* n, const double* dx, const double* Q) {
    return hmro_spectral_radius_ns(cfg, nullptr, n, dx, Q);
}

// CPU baseline: the patch is split along its slowest axis into nthreads
// equal sub-patches (as SAMRAI's partitioner would hand one patch to each
// rank); every std::thread advances its own sub-patch through one RK stage
// (flux + stage update) with ghosts taken from the parent patch.  Returns
// the interior cells updated.
long hmro_stage_threads(const hmro_config* cfg, const int* n, const double* dx, double dt,
                        const double* Q, int nthreads) {
    const Config c = to_cfg(cfg);
    const int dim = c.dim;
    const int slow = dim - 1;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > n[slow]) nthreads = n[slow];
    const Box b = make_box(dim, n, c.ghosts);
    const int ncomp = num_comp(c), neq = num_eqn(c);
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; t++) {
        th.emplace_back([&, t]() {
            const int lo = (int)((long)n[slow] * t / nthreads);
            const int hi = (int)((long)n[slow] * (t + 1) / nthreads);
            int sn[3] = {n[0], n[1], dim == 3 ? n[2] : 1};
            sn[slow] = hi - lo;
            const Box sb = make_box(dim, sn, c.ghosts);
            std::vector<double> sq((size_t)ncomp * sb.ncell());
            for (int e = 0; e < ncomp; e++)
                for (int k = -sb.g[2]; k < sb.n[2] + sb.g[2]; k++)
                for (int j = -sb.g[1]; j < sb.n[1] + sb.g[1]; j++)
                for (int i = -sb.g[0]; i < sb.n[0] + sb.g[0]; i++) {
                    int s3[3] = {i, j, k};
                    s3[slow] += lo;
                    sq[(size_t)e * sb.ncell() + sb.cell(i, j, k)] =
                        Q[(size_t)e * b.ncell() + b.cell(s3[0], s3[1], s3[2])];
                }
            const long nint = (long)sb.n[0] * sb.n[1] * sb.n[2];
            std::vector<double> f(flux_len(c, sb)), s((size_t)neq * nint, 0.0), qo(sq.size());
            hmro_conv_flux_source(cfg, sn, dx, dt, sq.data(), f.data(), s.data(), nullptr);
            const double one = 1.0, zero = 0.0;
            hmro_rk_stage(cfg, sn, dx, 1, &one, &one, &zero, sq.data(), f.data(), s.data(),
                          qo.data(), nullptr, nullptr);
        });
    }
    for (auto& x : th) x.join();
    return (long)n[0] * n[1] * (dim == 3 ? n[2] : 1);
}

}  // extern "C"
