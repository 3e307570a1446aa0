// Operation counter for the oracle (test / measurement infrastructure only).
// Instantiates the oracle on a scalar type that counts every FP64 operation
// (add, sub, mul, div, sqrt, fabs, fmin, fmax: 1 each), giving the
// algorithmic FP64 operation count of one RK substep per cell-update.
#include <cmath>

namespace hmro_count {
inline unsigned long long g_ops = 0;
inline int g_phase = 0;
inline unsigned long long g_phase_ops[16] = {};
// every counted operation is also charged to the oracle's current sub-phase (HMRO_PHASE)
inline void tick() { g_ops++; g_phase_ops[g_phase]++; }
struct C {
    double v;
    C() : v(0.0) {}
    C(double x) : v(x) {}
};
inline C operator+(C a, C b) { tick(); return C(a.v + b.v); }
inline C operator-(C a, C b) { tick(); return C(a.v - b.v); }
inline C operator*(C a, C b) { tick(); return C(a.v * b.v); }
inline C operator/(C a, C b) { tick(); return C(a.v / b.v); }
inline C operator-(C a) { return C(-a.v); }
inline C operator+(C a, double b) { return a + C(b); }
inline C operator-(C a, double b) { return a - C(b); }
inline C operator*(C a, double b) { return a * C(b); }
inline C operator/(C a, double b) { return a / C(b); }
inline C operator+(double a, C b) { return C(a) + b; }
inline C operator-(double a, C b) { return C(a) - b; }
inline C operator*(double a, C b) { return C(a) * b; }
inline C operator/(double a, C b) { return C(a) / b; }
inline C& operator+=(C& a, C b) { a = a + b; return a; }
inline C& operator-=(C& a, C b) { a = a - b; return a; }
inline C& operator*=(C& a, C b) { a = a * b; return a; }
}  // namespace hmro_count

namespace hmro {
inline hmro_count::C s_sqrt(hmro_count::C a) { hmro_count::tick(); return hmro_count::C(std::sqrt(a.v)); }
inline hmro_count::C s_fabs(hmro_count::C a) { hmro_count::tick(); return hmro_count::C(std::fabs(a.v)); }
inline hmro_count::C s_fmin(hmro_count::C a, hmro_count::C b) { hmro_count::tick(); return hmro_count::C(std::fmin(a.v, b.v)); }
inline hmro_count::C s_fmax(hmro_count::C a, hmro_count::C b) { hmro_count::tick(); return hmro_count::C(std::fmax(a.v, b.v)); }
inline double s_val(hmro_count::C a) { return a.v; }
}  // namespace hmro

#define HMRO_PHASE(k) (hmro_count::g_phase = (k))
#include "hmr_oracle.hpp"

#include <vector>

extern "C" {

// FP64 operations of one RK stage (flux + source + stage update) of one patch
// per interior cell.  Q: ncomp x ghost box; cfg fields as hmro_config.
double hmro_count_ops(int model, int dim, int nsp, int scheme, const double* gamma, const int* n,
                      const double* dx, const double* Q) {
    using hmro_count::C;
    hmro::Config c;
    c.model = model; c.dim = dim; c.num_species = nsp; c.scheme = scheme;
    for (int i = 0; i < 8; i++) c.gamma[i] = i < nsp ? gamma[i] : 1.4;
    for (int i = 0; i < 8; i++) c.R[i] = 1.0;
    c.p = 2; c.q = 4; c.C = 1.0e9; c.alpha_tau = 35.0; c.Chi = 1.0e8; c.epsilon = 1.0e-8;
    for (int i = 0; i < 3; i++) c.grid_dx[i] = dx[i];
    const hmro::Box b = hmro::make_box(dim, n, 4);
    const int ncomp = hmro::num_comp(c), neq = hmro::num_eqn(c);
    std::vector<C> q((size_t)ncomp * b.ncell());
    for (size_t i = 0; i < q.size(); i++) q[i] = C(Q[i]);
    std::vector<const C*> qp(ncomp);
    for (int e = 0; e < ncomp; e++) qp[e] = q.data() + (size_t)e * b.ncell();
    const long nint = (long)b.n[0] * b.n[1] * b.n[2];
    std::vector<std::vector<C>> flux;
    std::vector<C*> fp;
    for (int a = 0; a < dim; a++)
        for (int e = 0; e < neq; e++) {
            flux.emplace_back((size_t)(b.n[0] + (a == 0)) * (b.n[1] + (a == 1)) * (b.n[2] + (a == 2)));
        }
    for (auto& f : flux) fp.push_back(f.data());
    std::vector<std::vector<C>> src(neq, std::vector<C>(nint));
    std::vector<C*> sp;
    for (auto& s : src) sp.push_back(s.data());
    hmro::g_minimal_hll = true;
    hmro_count::g_ops = 0;
    for (int k = 0; k < 16; k++) hmro_count::g_phase_ops[k] = 0;
    hmro::conv_flux_source<C>(c, n, dx, 1.0e-3, qp.data(), fp.data(), sp.data(), nullptr);
    // stage update: Q = 1*Q + 1*(div + S)
    std::vector<C> qo((size_t)ncomp * b.ncell());
    std::vector<C*> qop(ncomp);
    for (int e = 0; e < ncomp; e++) qop[e] = qo.data() + (size_t)e * b.ncell();
    const C* const* qi[1] = {qp.data()};
    const C* const* fi[1] = {fp.data()};
    const C* const* si[1] = {sp.data()};
    const double one = 1.0, zero = 0.0;
    hmro_count::g_phase = hmro::HMRO_PH_STAGE;
    hmro::rk_stage<C>(c, n, dx, 1, &one, &one, &zero, qi, fi, si, qop.data(), nullptr, nullptr);
    hmro::g_minimal_hll = false;
    return (double)hmro_count::g_ops / (double)nint;
}

// Operations per interior cell of the last hmro_count_ops call, by sub-phase (HMRO_NPH values:
// cell data, sensor, projection factors, characteristic variables, smoothness indicators,
// weights and interpolation, inverse projection, bounds, Riemann, flux formula, source, stage).
void hmro_count_phases(const int* n, int dim, double* out) {
    long nint = 1;
    for (int d = 0; d < dim; d++) nint *= n[d];
    for (int k = 0; k < hmro::HMRO_NPH; k++) out[k] = (double)hmro_count::g_phase_ops[k] / (double)nint;
}

}  // extern "C"
