// Device self-check of the integer-pipe binary64 arithmetic (hmr_emu64.cuh): emulated
// multiply, add and subtract against __dmul_rn / __dadd_rn / __dsub_rn on seeded operand
// families (typical and extreme exponents, arbitrary bit patterns, exact products and rounding
// ties, cancellation, one binade, zeros).  Verification utility, not part of the hot path.
#include <cuda_runtime.h>

#include "hmr_emu64.cuh"

namespace {

__device__ __forceinline__ unsigned long long splitmix(unsigned long long& s) {
    unsigned long long z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ double operand(unsigned long long& s, int family, double other) {
    const unsigned long long r = splitmix(s), r2 = splitmix(s);
    const unsigned long long sign = r & 0x8000000000000000ull;
    unsigned long long frac = r & 0x000FFFFFFFFFFFFFull;
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
    case 4: { const unsigned long long uo = (unsigned long long)__double_as_longlong(other);
              const unsigned long long flip = splitmix(s) & ((1ull << ((r2 % 53) + 1)) - 1ull);
              unsigned long long v = (uo ^ 0x8000000000000000ull) ^ flip;
              if ((r2 >> 40) & 1)
                  v = (v & ~0x7FF0000000000000ull) | ((((v >> 52) & 0x7FF) + ((r2 >> 41) & 3) - 1) & 0x7FF) << 52;
              return __longlong_as_double((long long)v); }
    case 5: e = 1023 + (unsigned)(r2 % 3) - 1; frac &= ~0xFFFull; break;
    case 6: if (r2 & 1) return __longlong_as_double((long long)sign);
            e = 1023 - 10 + (unsigned)((r2 >> 1) % 21);
            break;
    }
    return __longlong_as_double((long long)(sign | ((unsigned long long)e << 52) | frac));
}

__global__ void emu_check_kernel(int iters, unsigned long long* bad) {
    const int op = blockIdx.y / 7, family = blockIdx.y % 7;
    unsigned long long s = 0xC0FFEEull + 131ull * op + 17ull * family +
                           0x1234567ull * (blockIdx.x * blockDim.x + threadIdx.x + 1);
    unsigned long long mine = 0;
    for (int i = 0; i < iters; i++) {
        const double a = operand(s, family == 4 ? 0 : family, 0.0), b = operand(s, family, a);
        double want, got;
        if (op == 0) { want = __dmul_rn(a, b); got = hmr::emu_dmul(a, b); }
        else if (op == 1) { want = __dadd_rn(a, b); got = hmr::emu_dadd(a, b); }
        else { want = __dsub_rn(a, b); got = hmr::emu_dsub(a, b); }
        const bool same = __double_as_longlong(want) == __double_as_longlong(got) || (want != want && got != got);
        mine += same ? 0ull : 1ull;
    }
    if (mine) atomicAdd(&bad[blockIdx.y], mine);
}

}  // namespace

// Runs `iters` operand pairs per thread for each operation (multiply, add, subtract) and operand
// family (7 each; multiply skips the cancellation family), on 4 blocks of 256 threads per SM;
// writes the 21 mismatch counts (index op * 7 + family) to bad_out.  Returns a CUDA status.
extern "C" int hmr_emu64_check(int iters, unsigned long long* bad_out) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -3;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    unsigned long long* bad = nullptr;
    if (cudaMalloc(&bad, 21 * sizeof(unsigned long long)) != cudaSuccess) return -4;
    cudaMemset(bad, 0, 21 * sizeof(unsigned long long));
    emu_check_kernel<<<dim3(sms * 4, 21), 256>>>(iters, bad);
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(bad_out, bad, 21 * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
    cudaFree(bad);
    return (int)e;
}
