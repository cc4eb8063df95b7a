// ppf_peak.cu -- ppf_measure_fp64_peak: the FP64 FMA rate of the current
// device, the denominator of the FP64 step's roofline (the FP64 step is
// bound by the FP64 pipe, not by HBM, on this GPU).
//
// Every thread runs eight independent FMA chains (enough to cover the FMA
// latency), a persistent-sized grid covers every SM, and the launches are
// timed with CUDA events after one warm-up launch.  FLOPs = 2 per FMA.
#include <cuda_runtime.h>

#include <cstdio>

#include "ppf.h"
#include "ppf_internal.h"

namespace {

__global__ void __launch_bounds__(256) dfma_chains(double *sink, int iters, double a, double b) {
    double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
    double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
        x0 = fma(x0, a, b);
        x1 = fma(x1, a, b);
        x2 = fma(x2, a, b);
        x3 = fma(x3, a, b);
        x4 = fma(x4, a, b);
        x5 = fma(x5, a, b);
        x6 = fma(x6, a, b);
        x7 = fma(x7, a, b);
    }
    const double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == 1.25e300) sink[blockIdx.x] = s;   // keeps the chains live; never true for these inputs
}

}  // namespace

extern "C" int ppf_measure_fp64_peak(double *tflops) {
    if (!tflops) return ppf::set_last_error(PPF_EINVAL, "null argument");
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess)
        return ppf::set_last_error(PPF_ECUDA, "no CUDA device");
    const int grid = sms * 8, iters = 16384, reps = 4;
    double *sink = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaStream_t s = nullptr;
    int rc = PPF_OK;
    float ms = 0.0f;
    if (cudaMalloc(&sink, (size_t)grid * sizeof(double)) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess) {
        rc = ppf::set_last_error(PPF_ECUDA, "FP64 peak: setup failed");
    } else {
        dfma_chains<<<grid, 256, 0, s>>>(sink, iters, 0.9999999, 1e-7);   // warm-up
        cudaEventRecord(e0, s);
        for (int r = 0; r < reps; ++r) dfma_chains<<<grid, 256, 0, s>>>(sink, iters, 0.9999999, 1e-7);
        cudaEventRecord(e1, s);
        if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess || ms <= 0)
            rc = ppf::set_last_error(PPF_ECUDA, "FP64 peak: timing failed");
    }
    if (rc == PPF_OK) *tflops = 2.0 * 8.0 * iters * 256.0 * grid * reps / (ms * 1e-3) / 1e12;
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
    if (sink) cudaFree(sink);
    return rc;
}
