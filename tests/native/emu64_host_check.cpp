// Host build of hamers_gb300/csrc/hmr_emu64.cuh (test infrastructure): the CUDA intrinsics it
// uses are given their host meaning below, and every emulated multiply, add and subtract is
// compared bit for bit with the host's IEEE-754 double operation (correctly rounded, round to
// nearest even; built with -ffp-contract=off).  Operand families: typical magnitudes, arbitrary
// bit patterns (NaN, infinities, subnormals), exponents at both ends of the range, short
// significands (exact products and rounding ties), near-cancelling pairs, one binade, zeros.
// Usage: emu64_host_check <cases per family>; exit status = number of failing families.
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#define __device__
#define __forceinline__ inline
static inline long long __double_as_longlong(double d) { long long x; std::memcpy(&x, &d, 8); return x; }
static inline double __longlong_as_double(long long x) { double d; std::memcpy(&d, &x, 8); return d; }
static inline int __double2hiint(double d) { return (int)(__double_as_longlong(d) >> 32); }
static inline int __double2loint(double d) { return (int)(unsigned)__double_as_longlong(d); }
static inline double __hiloint2double(int h, int l) {
    return __longlong_as_double((long long)(((unsigned long long)(unsigned)h << 32) | (unsigned)l));
}
static inline unsigned __funnelshift_r(unsigned lo, unsigned hi, unsigned sh) {
    return (unsigned)((((unsigned long long)hi << 32) | lo) >> (sh & 31u));
}
static inline int __clzll(long long x) { return x == 0 ? 64 : __builtin_clzll((unsigned long long)x); }
static inline double __dmul_rn(double a, double b) { volatile double r = a * b; return r; }
static inline double __dadd_rn(double a, double b) { volatile double r = a + b; return r; }
static inline double __dsub_rn(double a, double b) { volatile double r = a - b; return r; }
#include "../../hamers_gb300/csrc/hmr_emu64.cuh"

using hmr::emu_dadd;
using hmr::emu_dmul;
using hmr::emu_dsub;

static inline uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static double operand(uint64_t& s, int family, double other) {
    const uint64_t r = splitmix(s), r2 = splitmix(s);
    const uint64_t sign = r & 0x8000000000000000ull;
    uint64_t frac = r & 0x000FFFFFFFFFFFFFull;
    unsigned e = 1023;
    switch (family) {
    case 0: e = 1023 - 40 + (unsigned)(r2 % 81); break;
    case 1: return __longlong_as_double((long long)r);
    case 2: e = (r2 & 1) ? (unsigned)(r2 >> 1) % 40 : 2046 - (unsigned)(r2 >> 1) % 40;
            if ((r2 >> 20) % 7 == 0) e = 0;
            break;
    case 3: { const int k = 1 + (int)(r2 % 30);
              frac &= ~((1ull << (52 - k)) - 1ull) & 0x000FFFFFFFFFFFFFull;
              e = 1023 - 20 + (unsigned)((r2 >> 8) % 41);
              break; }
    case 4: { const uint64_t uo = (uint64_t)__double_as_longlong(other);
              const uint64_t flip = splitmix(s) & ((1ull << ((r2 % 53) + 1)) - 1ull);
              uint64_t v = (uo ^ 0x8000000000000000ull) ^ flip;
              if ((r2 >> 40) & 1)
                  v = (v & ~0x7FF0000000000000ull) | ((((v >> 52) & 0x7FF) + ((r2 >> 41) & 3) - 1) & 0x7FF) << 52;
              return __longlong_as_double((long long)v); }
    case 5: e = 1023 + (unsigned)(r2 % 3) - 1; frac &= ~0xFFFull; break;
    case 6: if (r2 & 1) return __longlong_as_double((long long)sign);
            e = 1023 - 10 + (unsigned)((r2 >> 1) % 21);
            break;
    }
    return __longlong_as_double((long long)(sign | ((uint64_t)e << 52) | frac));
}

static bool same(double x, double y) {
    return __double_as_longlong(x) == __double_as_longlong(y) || (x != x && y != y);
}

int main(int argc, char** argv) {
    const long long n = argc > 1 ? atoll(argv[1]) : 1000000;
    const char* names[3] = {"mul", "add", "sub"};
    int failing = 0;
    for (int op = 0; op < 3; op++)
        for (int family = 0; family < 7; family++) {
            if (op == 0 && family == 4) continue;   // cancellation matters for additions only
            std::atomic<long long> bad(0);
            std::vector<std::thread> pool;
            const int nt = 4;
            for (int t = 0; t < nt; t++)
                pool.emplace_back([&, t]() {
                    uint64_t s = 0xC0FFEEull + 131ull * op + 17ull * family + 1000003ull * t;
                    for (long long i = 0; i < n / nt; i++) {
                        const double a = operand(s, family == 4 ? 0 : family, 0.0), b = operand(s, family, a);
                        double want, got;
                        if (op == 0) { want = __dmul_rn(a, b); got = emu_dmul(a, b); }
                        else if (op == 1) { want = __dadd_rn(a, b); got = emu_dadd(a, b); }
                        else { want = __dsub_rn(a, b); got = emu_dsub(a, b); }
                        if (!same(want, got) && bad.fetch_add(1) < 3)
                            std::printf("  %s(%a, %a): native %a, emulated %a\n", names[op], a, b, want, got);
                    }
                });
            for (auto& t : pool) t.join();
            std::printf("%s family %d: %lld mismatches in %lld\n", names[op], family, bad.load(), n);
            failing += bad.load() != 0;
        }
    return failing;
}
