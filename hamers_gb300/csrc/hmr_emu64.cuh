// IEEE-754 binary64 multiply, add and subtract, round to nearest even, computed on the integer
// pipes.  Results are bit for bit those of __dmul_rn / __dadd_rn / __dsub_rn for every input:
// normal and zero operands with a normal (or overflowing) result take the integer path; every
// other case (subnormal operands or results, infinities, NaN) takes the native instruction.
//
// Why: GB300's FP64 pipe executes 2 thread operations per clock per SM, so a warp-wide FP64
// instruction holds it for about 64 cycles, while the integer ALU and IMAD pipes of an
// FP64-bound kernel sit idle.  An operation emulated there runs beside the native ones and
// raises the kernel's FP64 operation rate without changing a single result bit.
//
// Method (standard software floating point), on 32-bit words so that every shift has a
// known word and range: the 53-bit significands are multiplied exactly into 106 bits with four
// 32x32->64 multiply-adds; or aligned, with the shifted-out bits jammed into a sticky bit, and
// added in 64 bits, then normalised with a count of leading zeros; the result is rounded to
// nearest even from the bits below the significand.
#ifndef HMR_EMU64_CUH
#define HMR_EMU64_CUH

namespace hmr {

namespace emu64_detail {

__device__ __forceinline__ unsigned hi32(double x) { return (unsigned)__double2hiint(x); }
__device__ __forceinline__ unsigned lo32(double x) { return (unsigned)__double2loint(x); }
__device__ __forceinline__ double from32(unsigned hi, unsigned lo) { return __hiloint2double((int)hi, (int)lo); }

// Round the significand (mh:ml, hidden bit at bit 20 of mh) up when the bits below it -- the
// top-aligned word `x` and the sticky flag `st` (any nonzero bit below x) -- exceed half an
// ulp, or equal it with ml odd; pack with the biased exponent e in [1, 2046] (a carry out of the
// rounding moves the exponent up, to infinity past 2046) and the sign word.
__device__ __forceinline__ double pack_rne(unsigned mh, unsigned ml, unsigned x, bool st, int e,
                                           unsigned sign) {
    const bool up = (x > 0x80000000u) | ((x == 0x80000000u) & (st | (ml & 1u)));
    const unsigned long long m = (((unsigned long long)mh << 32) | ml) + (unsigned long long)up;
    const unsigned hi = (unsigned)(m >> 32) + ((unsigned)(e - 1) << 20);
    return from32(hi | sign, (unsigned)m);
}

}  // namespace emu64_detail

__device__ __forceinline__ double emu_dmul(double a, double b) {
    using namespace emu64_detail;
    const unsigned ah = hi32(a), al = lo32(a), bh = hi32(b), bl = lo32(b);
    const unsigned ea = (ah >> 20) & 0x7FFu, eb = (bh >> 20) & 0x7FFu;
    const unsigned sign = (ah ^ bh) & 0x80000000u;
    const int e0 = (int)(ea + eb) - 1023;   // biased exponent of the product for a significand in [1, 2)
    if ((ea - 1u < 2046u) & (eb - 1u < 2046u) & ((unsigned)(e0 - 1) < 2045u)) {
        const unsigned mah = (ah & 0x000FFFFFu) | 0x00100000u, mbh = (bh & 0x000FFFFFu) | 0x00100000u;
        // 106-bit product w3:w2:w1:w0 of (mah:al) and (mbh:bl)
        const unsigned long long t0 = (unsigned long long)al * bl;
        const unsigned long long t1 = (unsigned long long)mah * bl + (t0 >> 32);
        const unsigned long long t2 = (unsigned long long)al * mbh + (unsigned)t1;
        const unsigned long long t3 = (unsigned long long)mah * mbh + (t1 >> 32) + (t2 >> 32);
        const unsigned w0 = (unsigned)t0, w1 = (unsigned)t2, w2 = (unsigned)t3, w3 = (unsigned)(t3 >> 32);
        const unsigned s = w3 >> 9;                       // 1 if the product is >= 2^105
        const unsigned sh = 20u + s;                      // significand = product >> (52 + s)
        const unsigned ml = __funnelshift_r(w1, w2, sh), mh = __funnelshift_r(w2, w3, sh);
        const unsigned x = w1 << (12u - s);               // bits of w1 below the significand, top-aligned
        return pack_rne(mh, ml, x, w0 != 0u, e0 + (int)s, sign);
    }
    const bool za = ((ah << 1) | al) == 0u, zb = ((bh << 1) | bl) == 0u;
    if ((za & (eb < 2047u)) | (zb & (ea < 2047u))) return from32(sign, 0u);   // 0 * finite
    return __dmul_rn(a, b);
}

__device__ __forceinline__ double emu_dadd(double a, double b) {
    using namespace emu64_detail;
    unsigned ah = hi32(a), al = lo32(a), bh = hi32(b), bl = lo32(b);
    // order by magnitude: |a| >= |b|
    const unsigned long long ma_ = ((unsigned long long)(ah & 0x7FFFFFFFu) << 32) | al;
    const unsigned long long mb_ = ((unsigned long long)(bh & 0x7FFFFFFFu) << 32) | bl;
    if (mb_ > ma_) {
        unsigned t = ah; ah = bh; bh = t;
        t = al; al = bl; bl = t;
    }
    const unsigned ea = (ah >> 20) & 0x7FFu, eb = (bh >> 20) & 0x7FFu;
    const unsigned sign = ah & 0x80000000u;
    if ((ea - 1u < 2046u) & (eb - 1u < 2046u)) {
        // significands with the hidden bit at 62 (10 rounding bits below)
        const unsigned long long ma = (((unsigned long long)((ah & 0x000FFFFFu) | 0x00100000u) << 32) | al) << 10;
        const unsigned long long mb0 = (((unsigned long long)((bh & 0x000FFFFFu) | 0x00100000u) << 32) | bl) << 10;
        const unsigned d = ea - eb;
        unsigned long long mb;
        if (d == 0u) mb = mb0;
        else if (d < 64u) mb = (mb0 >> d) | (unsigned long long)((mb0 << (64u - d)) != 0ull);
        else mb = 1ull;                                   // sticky only
        int e = (int)ea;
        unsigned long long sum;
        if (((ah ^ bh) & 0x80000000u) == 0u) {
            sum = ma + mb;                                // < 2^64
            const unsigned c = (unsigned)(sum >> 63);
            sum = (sum >> c) | (sum & (unsigned long long)c);
            e += (int)c;
        } else {
            sum = ma - mb;
            if (sum == 0ull) return 0.0;                  // x - x = +0
            const int lz = __clzll((long long)sum) - 1;   // hidden bit back to 62
            sum <<= lz;
            e -= lz;
        }
        if ((unsigned)(e - 1) < 2046u) {
            const unsigned sh = (unsigned)(sum >> 32), sl = (unsigned)sum;
            return pack_rne(sh >> 10, __funnelshift_r(sl, sh, 10), sl << 22, false, e, sign);
        }
    } else if ((((bh << 1) | bl) == 0u) & (ea < 2047u)) {   // b = +-0, a finite
        if (((ah << 1) | al) != 0u) return from32(ah, al);
        return from32(ah & bh, 0u);                         // +-0 + +-0
    }
    return __dadd_rn(a, b);
}

__device__ __forceinline__ double emu_dsub(double a, double b) {
    return emu_dadd(a, __longlong_as_double(__double_as_longlong(b) ^ (long long)0x8000000000000000ull));
}

}  // namespace hmr

#endif  // HMR_EMU64_CUH
