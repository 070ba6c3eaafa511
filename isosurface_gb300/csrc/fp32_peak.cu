// FP32 issue-rate probe for the sampler's roofline: the measured rate of
// dependent-chain FMAs (2 flops each) on every SM, timed with CUDA events.
// Built into its own small library (libiso_fp32_peak.so) that only the
// benchmark loads; it is not part of the extraction library's C ABI.
#include <cuda_runtime.h>

namespace {

constexpr int CHAINS = 8;       // independent accumulators per thread
constexpr int ITERS = 4096;     // FMAs per chain
constexpr int THREADS = 256;
constexpr int BLOCKS_PER_SM = 8;

__global__ void __launch_bounds__(THREADS) fma_chains(float* out, float b, float c) {
    float a[CHAINS];
#pragma unroll
    for (int k = 0; k < CHAINS; ++k) a[k] = (float)(threadIdx.x + k);
#pragma unroll 16
    for (int i = 0; i < ITERS; ++i) {
#pragma unroll
        for (int k = 0; k < CHAINS; ++k) a[k] = __fmaf_rn(a[k], b, c);
    }
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < CHAINS; ++k) s += a[k];
    // b and c keep the values bounded; the store is never taken for them
    if (s == 123.456f) out[blockIdx.x * THREADS + threadIdx.x] = s;
}

}  // namespace

// Best of `reps` launches: FP32 TFLOP/s (2 flops per FMA) and that launch's
// milliseconds.  Returns 0 on success, the CUDA error code otherwise.
extern "C" __attribute__((visibility("default"))) int iso_fp32_fma_peak(int device, int reps, double* tflops,
                                                                       double* ms) {
    cudaError_t e = cudaSetDevice(device);
    int sms = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) return (int)e;
    const int blocks = sms * BLOCKS_PER_SM;
    float* out = nullptr;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    e = cudaMalloc(&out, sizeof(float) * blocks * THREADS);
    if (e == cudaSuccess) e = cudaEventCreate(&t0);
    if (e == cudaSuccess) e = cudaEventCreate(&t1);
    float best = 1e30f;
    for (int r = 0; e == cudaSuccess && r < reps + 1; ++r) {
        cudaEventRecord(t0);
        fma_chains<<<blocks, THREADS>>>(out, 0.999999f, 1e-7f);
        cudaEventRecord(t1);
        e = cudaEventSynchronize(t1);
        float m = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&m, t0, t1);
        if (r > 0 && m < best) best = m;  // the first launch warms up
    }
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
    if (out) cudaFree(out);
    if (e != cudaSuccess) return (int)e;
    const double flops = 2.0 * CHAINS * ITERS * (double)blocks * THREADS;
    *ms = best;
    *tflops = flops / (best * 1e-3) / 1e12;
    return 0;
}
