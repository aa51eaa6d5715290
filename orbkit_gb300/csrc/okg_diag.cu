// Diagnostics: measured FP64 FMA issue rate of the device (the roofline
// denominator of the FP64 kernels; not part of the grid path).
#include "okg_internal.cuh"

namespace okg {
// DIAG_CHAINS independent FMA chains per thread, DIAG_UNROLL FMAs per chain per loop
// trip, so loop overhead is a small fraction of the issued instructions.
#define DIAG_CHAINS 8
#define DIAG_UNROLL 8
__global__ void __launch_bounds__(256) dfma_rate_kernel(long long iters, double seed, double* sink)
{
    double a[DIAG_CHAINS];
#pragma unroll
    for (int k = 0; k < DIAG_CHAINS; ++k) a[k] = seed + threadIdx.x + k;
    const double m = 0.999999, c = 1e-7;
    for (long long i = 0; i < iters; i += DIAG_UNROLL) {
#pragma unroll
        for (int u = 0; u < DIAG_UNROLL; ++u)
#pragma unroll
            for (int k = 0; k < DIAG_CHAINS; ++k) a[k] = fma(a[k], m, c);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < DIAG_CHAINS; ++k) s += a[k];
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
    const long long trips = (iters + DIAG_UNROLL - 1) / DIAG_UNROLL;
    *fma_per_s = (double)sms * 4 * 256 * DIAG_CHAINS * (double)(trips * DIAG_UNROLL) / (ms * 1e-3);
    return OKG_OK;
}
