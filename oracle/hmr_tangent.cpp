// Tangent of the oracle (test infrastructure only).
//
// Instantiates the oracle on a forward-mode dual number, giving the exact
// directional derivative J v of one RK substep along the branch the substep
// takes at the given state.  The reference has no derivative code, so the
// GPU adjoint is checked against this tangent with the dot-product identity
// <w, J v> = <J^T w, v>, and the tangent itself against central differences
// of the oracle.
//
// Derivative conventions at non-smooth points, shared with the GPU adjoint:
//   |x|         : sign(x), 0 at x = 0
//   fmin(a, b)  : the derivative of a if a < b, else of b
//   fmax(a, b)  : the derivative of a if a > b, else of b
//   sqrt(x)     : 1/(2 sqrt(x)), 0 at x = 0
// Discrete decisions (bounds check and first-order fallback, shock sensor,
// HLLC side, WCNS6-LD tau switch) are taken on the values and carry no
// derivative.
#include <cmath>

namespace hmro_dual {
struct D {
    double v, d;
    D() : v(0.0), d(0.0) {}
    D(double x) : v(x), d(0.0) {}
    D(double x, double y) : v(x), d(y) {}
};
inline D operator+(D a, D b) { return D(a.v + b.v, a.d + b.d); }
inline D operator-(D a, D b) { return D(a.v - b.v, a.d - b.d); }
inline D operator*(D a, D b) { return D(a.v * b.v, a.d * b.v + a.v * b.d); }
inline D operator/(D a, D b) {
    const double q = a.v / b.v;
    return D(q, (a.d - q * b.d) / b.v);
}
inline D operator-(D a) { return D(-a.v, -a.d); }
inline D operator+(D a, double b) { return a + D(b); }
inline D operator-(D a, double b) { return a - D(b); }
inline D operator*(D a, double b) { return a * D(b); }
inline D operator/(D a, double b) { return a / D(b); }
inline D operator+(double a, D b) { return D(a) + b; }
inline D operator-(double a, D b) { return D(a) - b; }
inline D operator*(double a, D b) { return D(a) * b; }
inline D operator/(double a, D b) { return D(a) / b; }
inline D& operator+=(D& a, D b) { a = a + b; return a; }
inline D& operator-=(D& a, D b) { a = a - b; return a; }
inline D& operator*=(D& a, D b) { a = a * b; return a; }
}  // namespace hmro_dual

namespace hmro {
inline hmro_dual::D s_sqrt(hmro_dual::D a) {
    const double r = std::sqrt(a.v);
    return hmro_dual::D(r, r > 0.0 ? a.d / (2.0 * r) : 0.0);
}
inline hmro_dual::D s_fabs(hmro_dual::D a) {
    return hmro_dual::D(std::fabs(a.v), a.v > 0.0 ? a.d : (a.v < 0.0 ? -a.d : 0.0));
}
inline hmro_dual::D s_fmin(hmro_dual::D a, hmro_dual::D b) { return a.v < b.v ? a : b; }
inline hmro_dual::D s_fmax(hmro_dual::D a, hmro_dual::D b) { return a.v > b.v ? a : b; }
inline double s_val(hmro_dual::D a) { return a.v; }
}  // namespace hmro

#include "hmr_oracle.hpp"

#include <vector>

extern "C" {

// Tangent of the fused substep: Q_out = sum_{n<=stage} alpha[n] Q_int[n]
// + beta * (-div F(Q_int[stage]) + S(Q_int[stage])) (the forward of
// hmr_rk_substep_patch).  Q_int / dQ_int hold stage+1 consecutive ghost-box
// states (ncomp components each, ghosts of the last one filled); Q_out and
// dQ_out receive the output state and its derivative along dQ_int (ghost box,
// interior written).
// With tr non-null the substep is NavierStokes's: the diffusive flux of
// Q_int[stage] enters the divergence too.
int hmro_tangent_substep(const hmro_config* cfg, const int* n, const double* dx, double dt, int stage,
                         const double* alpha, double beta, const double* Q_int, const double* dQ_int,
                         double* Q_out, double* dQ_out, const hmro_transport* tr) {
    using hmro_dual::D;
    const hmro::Config c = hmro_to_config(cfg);
    const hmro::Box b = hmro::make_box(c.dim, n, c.ghosts);
    const int ncomp = hmro::num_comp(c), neq = hmro::num_eqn(c);
    const long nc = b.ncell();
    const long nint = (long)b.n[0] * b.n[1] * b.n[2];
    const int nst = stage + 1;

    std::vector<D> q((size_t)nst * ncomp * nc);
    for (size_t i = 0; i < q.size(); i++) q[i] = D(Q_int[i], dQ_int[i]);
    std::vector<std::vector<const D*>> qp(nst, std::vector<const D*>(ncomp));
    for (int s = 0; s < nst; s++)
        for (int e = 0; e < ncomp; e++) qp[s][e] = q.data() + ((size_t)s * ncomp + e) * nc;

    // flux and source of the current stage; zero arrays for the others (beta 0)
    std::vector<std::vector<D>> flux;
    for (int a = 0; a < c.dim; a++)
        for (int e = 0; e < neq; e++)
            flux.emplace_back((size_t)(b.n[0] + (a == 0)) * (b.n[1] + (a == 1)) * (b.n[2] + (a == 2)));
    std::vector<D*> fp;
    for (auto& f : flux) fp.push_back(f.data());
    std::vector<std::vector<D>> src(neq, std::vector<D>(nint));
    std::vector<D*> sp;
    for (auto& s : src) sp.push_back(s.data());
    hmro::conv_flux_source<D>(c, n, dx, dt, qp[stage].data(), fp.data(), sp.data(), nullptr);
    std::vector<std::vector<D>> dflux;
    std::vector<D*> dfp;
    if (tr) {
        for (auto& f : flux) dflux.emplace_back(f.size());
        for (auto& f : dflux) dfp.push_back(f.data());
        hmro::diff_flux<D>(c, hmro_to_transport(tr), n, dx, dt, qp[stage].data(), dfp.data());
    }

    std::vector<const D* const*> qpp(nst), fpp(nst), spp(nst), dpp(nst);
    std::vector<double> betas(nst, 0.0), gammas(nst, 0.0);
    betas[stage] = beta;
    for (int s = 0; s < nst; s++) {
        qpp[s] = qp[s].data();
        fpp[s] = fp.data();
        spp[s] = sp.data();
        dpp[s] = tr ? dfp.data() : nullptr;
    }
    std::vector<D> qo((size_t)ncomp * nc);
    std::vector<D*> qop(ncomp);
    for (int e = 0; e < ncomp; e++) qop[e] = qo.data() + (size_t)e * nc;
    hmro::rk_stage<D>(c, n, dx, nst, alpha, betas.data(), gammas.data(), qpp.data(), fpp.data(), spp.data(),
                      qop.data(), nullptr, nullptr, tr ? dpp.data() : nullptr);
    for (size_t i = 0; i < qo.size(); i++) {
        Q_out[i] = qo[i].v;
        dQ_out[i] = qo[i].d;
    }
    return 0;
}

}  // extern "C"
