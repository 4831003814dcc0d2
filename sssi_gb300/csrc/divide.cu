// Test entry of the constant-divisor division (divide.cuh): the strict FP64
// forms rely on div_rn(a, d) being the IEEE quotient bit for bit, and
// sssi_debug_divide lets a test compare the two over chosen dividends.
#include <algorithm>
#include <cmath>

#include "api_util.cuh"
#include "divide.cuh"

namespace sssi {
namespace {

__global__ void divide_kernel(const double* __restrict__ a, int64_t n, const Divisor<double> v, double* fast,
                              double* ieee) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        fast[i] = div_rn(a[i], v);
        ieee[i] = __ddiv_rn(a[i], v.d);
    }
}

}  // namespace
}  // namespace sssi

using namespace sssi;

extern "C" int sssi_debug_divide(const double* a, int64_t n, double d, double* fast, double* ieee) {
    return guarded([&] {
        SSSI_REQUIRE(n >= 0 && n < (int64_t(1) << 32), SSSI_ERR_ARG, "sssi_debug_divide: bad count %lld",
                     (long long)n);
        SSSI_REQUIRE(n == 0 || (a && fast && ieee), SSSI_ERR_ARG, "sssi_debug_divide: NULL buffer");
        if (n == 0) return;
        ensure_device();
        cudaStream_t s = current_stream();
        api::DeviceView da(a, (size_t)n, true, s);
        api::DeviceView df(fast, (size_t)n, false, s);
        api::DeviceView di(ieee, (size_t)n, false, s);
        const int grid = (int)std::min<int64_t>((n + 255) / 256, 4096);
        divide_kernel<<<grid, 256, 0, s>>>(da.ptr, n, make_divisor<double>(d), df.ptr, di.ptr);
        count_launch();
        SSSI_CHECK_CUDA(cudaGetLastError());
        df.download(fast, (size_t)n, s);
        di.download(ieee, (size_t)n, s);
        SSSI_CHECK_CUDA(cudaStreamSynchronize(s));
    });
}
