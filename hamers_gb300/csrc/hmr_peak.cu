// FP64 fused-multiply-add throughput of the device: the denominator of the
// FP64-pipe roofline fraction (this GPU's published peak is not measured by
// the copy/GEMM peaks).  Eight independent FMA chains per thread, every SM
// filled; flops = 2 x FMAs.  Measurement utility, not part of the hot path.
#include <cuda_runtime.h>

namespace {

__global__ void dfma_chains(double* out, double a, double b, int iters) {
    double x0 = 1e-9 * threadIdx.x, x1 = x0 + 1e-3, x2 = x0 + 2e-3, x3 = x0 + 3e-3;
    double x4 = x0 + 4e-3, x5 = x0 + 5e-3, x6 = x0 + 6e-3, x7 = x0 + 7e-3;
    for (int i = 0; i < iters; i++) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
}

}  // namespace

extern "C" int hmr_measure_fp64_fma(double* tflops_out, double* ms_out) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -3;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int threads = 256, blocks = sms * 8, iters = 1 << 15;
    double* out = nullptr;
    if (cudaMalloc(&out, sizeof(double) * threads * blocks) != cudaSuccess) return -4;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    dfma_chains<<<blocks, threads>>>(out, 0.9999999, 1e-7, iters);   // warm-up
    float best = 1e30f;
    for (int r = 0; r < 5; r++) {
        cudaEventRecord(e0);
        dfma_chains<<<blocks, threads>>>(out, 0.9999999, 1e-7, iters);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) best = ms;
    }
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess) return (int)err;
    const double flops = 2.0 * 8.0 * (double)iters * threads * blocks;
    *tflops_out = flops / (best * 1e-3) / 1e12;
    *ms_out = best;
    return 0;
}
