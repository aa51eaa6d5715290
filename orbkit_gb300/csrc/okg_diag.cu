// Diagnostics: measured FP64 FMA issue rate of the device (the roofline
// denominator of the FP64 kernels; not part of the grid path).
#include "okg_internal.cuh"

namespace okg {
__global__ void __launch_bounds__(256) dfma_rate_kernel(long long iters, double seed, double* sink)
{
    double a0 = seed + threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6,
           a7 = a0 + 7;
    const double m = 0.999999, c = 1e-7;
    for (long long i = 0; i < iters; ++i) {
        a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
        a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
    }
    const double s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == 12345.678) sink[blockIdx.x] = s;  // keeps the chains live
}
}  // namespace okg

using namespace okg;

extern "C" int okg_diag_fp64_fma_rate(long long iters, double* fma_per_s)
{
    if (!fma_per_s || iters <= 0) return set_error(OKG_ERR_ARG, "okg_diag_fp64_fma_rate: bad argument");
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    double* sink = nullptr;
    cudaError_t e = cudaMalloc(&sink, sizeof(double) * sms * 4);
    if (e != cudaSuccess) return cuda_status(e, "okg_diag_fp64_fma_rate: cudaMalloc");
    cudaEvent_t t0, t1;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    // full-length warm-up (the clocks ramp up), then the fastest of three timed runs
    dfma_rate_kernel<<<sms * 4, 256>>>(iters, 1.0, sink);
    float ms = 0.f;
    for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) {
        cudaEventRecord(t0);
        dfma_rate_kernel<<<sms * 4, 256>>>(iters, 1.0, sink);
        cudaEventRecord(t1);
        e = cudaEventSynchronize(t1);
        float m = 0.f;
        cudaEventElapsedTime(&m, t0, t1);
        ms = (rep == 0 || m < ms) ? m : ms;
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    cudaFree(sink);
    if (e != cudaSuccess) return cuda_status(e, "okg_diag_fp64_fma_rate");
    *fma_per_s = (double)sms * 4 * 256 * 8 * (double)iters / (ms * 1e-3);
    return OKG_OK;
}
