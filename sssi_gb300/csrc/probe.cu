// Measurement helper: the FP64 fused-multiply-add rate of the current GPU,
// the denominator of the FP64 drop-in's roofline (the FP64 stencil is bound by
// the FP64 pipe, not by HBM, on GB300).  Each thread advances eight independent
// FMA chains, so the pipe, not the dependency latency, sets the rate.
#include "sssi_internal.h"

namespace sssi {
namespace {

constexpr int kChains = 8;

__global__ void fp64_fma_rate_kernel(int iters, double b, double c, double* out) {
    double a[kChains];
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = threadIdx.x * 1e-3 + k;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int r = 0; r < 16; ++r)
#pragma unroll
            for (int k = 0; k < kChains; ++k) a[k] = fma(a[k], b, c);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < kChains; ++k) s += a[k];
    if (s == 12345.678) out[0] = s;  // keeps the chains alive; never true for these operands
}

}  // namespace
}  // namespace sssi

extern "C" int sssi_measure_fp64_rate(double* fma_per_s) {
    using namespace sssi;
    return guarded([&] {
        SSSI_REQUIRE(fma_per_s != nullptr, SSSI_ERR_ARG, "fma_per_s is NULL");
        ensure_device();
        int dev = 0, sms = 0;
        SSSI_CHECK_CUDA(cudaGetDevice(&dev));
        SSSI_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        DeviceBuffer sink(sizeof(double));
        cudaStream_t s = current_stream();
        const int blocks = sms * 8, threads = 256, iters = 2048;
        cudaEvent_t e0, e1;
        SSSI_CHECK_CUDA(cudaEventCreate(&e0));
        SSSI_CHECK_CUDA(cudaEventCreate(&e1));
        float best = 1e30f;
        for (int rep = 0; rep < 4; ++rep) {  // the first launch warms up; the fastest counts
            SSSI_CHECK_CUDA(cudaEventRecord(e0, s));
            fp64_fma_rate_kernel<<<blocks, threads, 0, s>>>(iters, 0.9999999, 1e-7, sink.as<double>());
            count_launch();
            SSSI_CHECK_CUDA(cudaEventRecord(e1, s));
            SSSI_CHECK_CUDA(cudaEventSynchronize(e1));
            float ms = 0.0f;
            SSSI_CHECK_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            if (rep > 0 && ms < best) best = ms;
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        SSSI_CHECK_CUDA(cudaGetLastError());
        const double fmas = (double)blocks * threads * iters * 16.0 * kChains;
        *fma_per_s = fmas / (best * 1e-3);
    });
}
