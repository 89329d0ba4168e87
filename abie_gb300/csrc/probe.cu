// Throughput probes for the roofline denominators: FP64 and FP32 FMA rates
// measured on this device with CUDA events (the denominators for the
// compute-bound force kernels, which no vendor table states for sm_103).
#include "abi_state.cuh"

namespace abie {

// Lanes >= active of each warp skip the chains (active = 32: all lanes).
template <typename T>
__global__ void __launch_bounds__(256) fma_probe_kernel(T *out, int iters, T b, T c, int active)
{
    T a0 = threadIdx.x * (T)1e-3, a1 = a0 + (T)1, a2 = a0 + (T)2, a3 = a0 + (T)3;
    T a4 = a0 + (T)4, a5 = a0 + (T)5, a6 = a0 + (T)6, a7 = a0 + (T)7;
    if ((int)(threadIdx.x & 31) < active) {
        for (int i = 0; i < iters; i++) {
            a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
            a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
        }
    }
    T s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == (T)-12345.0) out[0] = s;  // keeps the chains alive
}

// tflops: FMA rate counting every lane of every warp (2 flop per FMA), so
// with fewer active lanes it reads as the rate the warps were charged for.
template <typename T>
static int run_probe(int iters, int active, double *tflops)
{
    int rc = ensure_device(-1);
    if (rc) return rc;
    Sim &s = g_sim;
    T *out = nullptr;
    ABIE_CUDA(cudaMalloc(&out, sizeof(T)));
    int blocks = s.num_sms * 8;
    cudaEvent_t e0, e1;
    ABIE_CUDA(cudaEventCreate(&e0));
    ABIE_CUDA(cudaEventCreate(&e1));
    fma_probe_kernel<T><<<blocks, 256, 0, s.st>>>(out, iters / 8 + 1, (T)0.999999, (T)1e-7, active);
    ABIE_CUDA(cudaEventRecord(e0, s.st));
    fma_probe_kernel<T><<<blocks, 256, 0, s.st>>>(out, iters, (T)0.999999, (T)1e-7, active);
    ABIE_CUDA(cudaEventRecord(e1, s.st));
    ABIE_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    ABIE_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    double flops = 2.0 * 8.0 * (double)iters * (double)blocks * 256.0;
    *tflops = flops / (ms * 1e-3) / 1e12;
    return 0;
}

}  // namespace abie

extern "C" {
// Measured FMA throughput of this device, in TFLOP/s (an FMA counts 2).
int abie_measure_fp64_peak(int iters, double *tflops)
{
    return abie::run_probe<double>(iters > 0 ? iters : 4096, 32, tflops);
}
int abie_measure_fp32_peak(int iters, double *tflops)
{
    return abie::run_probe<float>(iters > 0 ? iters : 65536, 32, tflops);
}
// The FP64 probe with only the first active_lanes lanes of each warp working,
// reported as if every lane had: equal to the full-warp figure when the
// FP64 pipe charges a warp instruction the same whatever its active lanes.
int abie_measure_fp64_issue(int active_lanes, double *tflops)
{
    if (active_lanes < 1 || active_lanes > 32) return ABIE_ERR_ARGUMENT;
    return abie::run_probe<double>(4096, active_lanes, tflops);
}
}
