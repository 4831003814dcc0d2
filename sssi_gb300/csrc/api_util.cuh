// Staging of the API's double arrays (host or device memory) into device
// arrays of a propagator's element type, shared by the 2D and 3D entry points.
#pragma once

#include <algorithm>
#include <cstring>
#include <type_traits>
#include <vector>

#include "sssi_internal.h"

namespace sssi {
namespace api {

constexpr size_t kChunkBytes = size_t(256) << 20;  // host<->device streaming granularity

inline std::vector<double> host_copy(const double* p, size_t n, cudaStream_t s) {
    std::vector<double> h(n);
    if (n == 0) return h;
    if (is_device_pointer(p)) {
        SSSI_CHECK_CUDA(cudaMemcpyAsync(h.data(), p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
        SSSI_CHECK_CUDA(cudaStreamSynchronize(s));
    } else {
        std::memcpy(h.data(), p, n * sizeof(double));
    }
    return h;
}

// A device view of a caller array: the caller's pointer if it is device memory,
// otherwise a cached device buffer (filled from the host when `upload`).
struct DeviceView {
    double* ptr = nullptr;
    bool caller_device = false;
    DeviceBuffer buf;
    DeviceView(const double* p, size_t n, bool upload, cudaStream_t s) {
        if (!p) return;
        if (is_device_pointer(p)) {
            ptr = const_cast<double*>(p);
            caller_device = true;
            return;
        }
        buf.allocate(std::max<size_t>(n, 1) * sizeof(double));
        ptr = buf.as<double>();
        if (upload && n)
            SSSI_CHECK_CUDA(cudaMemcpyAsync(ptr, p, n * sizeof(double), cudaMemcpyHostToDevice, s));
    }
    void download(double* host, size_t n, cudaStream_t s) const {
        if (!host || caller_device || n == 0) return;
        SSSI_CHECK_CUDA(cudaMemcpyAsync(host, ptr, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    }
};

static __global__ void fill_kernel(double* p, int64_t n, double v) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        p[q] = v;
}

inline void fill(double* p, int64_t n, double v, cudaStream_t s) {
    fill_kernel<<<152 * 4, 256, 0, s>>>(p, n, v);
    count_launch();
    SSSI_CHECK_CUDA(cudaGetLastError());
}

// Elementwise conversion between the API's double arrays and a propagator's
// element type (a no-op copy is never launched: callers skip T == double).
template <typename From, typename To>
__global__ void convert_kernel(const From* in, To* out, int64_t n) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        out[q] = static_cast<To>(in[q]);
}

template <typename From, typename To>
void convert(const From* in, To* out, int64_t n, cudaStream_t s) {
    if (n <= 0) return;
    convert_kernel<From, To><<<152 * 4, 256, 0, s>>>(in, out, n);
    count_launch();
    SSSI_CHECK_CUDA(cudaGetLastError());
}

// A device array of T holding (or receiving) a caller array of doubles.
// When T is double and the caller's memory is on the device, it is used in
// place; otherwise a cached device buffer stages it (and converts).
template <typename T>
struct Staged {
    T* ptr = nullptr;
    const double* caller = nullptr;
    bool in_place = false;
    size_t n = 0;
    DeviceBuffer buf, tmp;

    Staged(const double* p, size_t count, bool upload, cudaStream_t s) : caller(p), n(count) {
        if (!p) return;
        const bool dev = is_device_pointer(p);
        if (std::is_same<T, double>::value && dev) {
            ptr = reinterpret_cast<T*>(const_cast<double*>(p));
            in_place = true;
            return;
        }
        buf.allocate(std::max<size_t>(n, 1) * sizeof(T));
        ptr = buf.as<T>();
        if (!upload || n == 0) return;
        if (std::is_same<T, double>::value) {
            SSSI_CHECK_CUDA(cudaMemcpyAsync(ptr, p, n * sizeof(double), cudaMemcpyHostToDevice, s));
        } else {
            const double* src = p;
            if (!dev) {
                tmp.allocate(n * sizeof(double));
                SSSI_CHECK_CUDA(cudaMemcpyAsync(tmp.get(), p, n * sizeof(double), cudaMemcpyHostToDevice, s));
                src = tmp.as<double>();
            }
            convert(src, ptr, (int64_t)n, s);
        }
    }
    // Copies the device contents back into the caller's array (host or device).
    void download(double* out, cudaStream_t s) {
        if (!out || in_place || n == 0) return;
        const bool dev = is_device_pointer(out);
        if (std::is_same<T, double>::value) {
            SSSI_CHECK_CUDA(cudaMemcpyAsync(out, ptr, n * sizeof(double), dev ? cudaMemcpyDeviceToDevice
                                                                               : cudaMemcpyDeviceToHost, s));
            return;
        }
        if (dev) {
            convert(ptr, out, (int64_t)n, s);
            return;
        }
        tmp.allocate(n * sizeof(double));
        convert(ptr, tmp.as<double>(), (int64_t)n, s);
        SSSI_CHECK_CUDA(cudaMemcpyAsync(out, tmp.get(), n * sizeof(double), cudaMemcpyDeviceToHost, s));
    }
};

// A chunk of K time slices of nz x nx streamed between the caller's array
// (host or device, double) and a device array of T.
template <typename T>
struct SliceStream {
    double* caller;
    bool caller_dev = false;
    int64_t n, K;
    DeviceBuffer tbuf, dbuf;
    T* base = nullptr;  // device slices of the current chunk (or the caller's when usable in place)

    SliceStream(double* p, int64_t cells, int64_t k) : caller(p), n(cells), K(k) {
        if (!p) return;
        caller_dev = is_device_pointer(p);
        if (!(std::is_same<T, double>::value && caller_dev)) tbuf.allocate(sizeof(T) * n * K);
        if (!std::is_same<T, double>::value && !caller_dev) dbuf.allocate(sizeof(double) * n * K);
    }
    bool in_place() const { return std::is_same<T, double>::value && caller_dev; }
    // device pointer of slice t (chunk starting at t0)
    T* slice(int64_t t, int64_t t0) {
        if (in_place()) return reinterpret_cast<T*>(caller) + t * n;
        return tbuf.as<T>() + (t - t0) * n;
    }
    // input: bring slices [t0, t0+kk) to the device
    void load(int64_t t0, int64_t kk, cudaStream_t s) {
        if (!caller || in_place()) return;
        const size_t bytes = sizeof(double) * n * kk;
        if (std::is_same<T, double>::value) {
            SSSI_CHECK_CUDA(cudaMemcpyAsync(tbuf.get(), caller + t0 * n, bytes, cudaMemcpyHostToDevice, s));
        } else if (caller_dev) {
            convert(caller + t0 * n, tbuf.as<T>(), n * kk, s);
        } else {
            SSSI_CHECK_CUDA(cudaMemcpyAsync(dbuf.get(), caller + t0 * n, bytes, cudaMemcpyHostToDevice, s));
            convert(dbuf.as<double>(), tbuf.as<T>(), n * kk, s);
        }
    }
    // output: send slices [t0, t0+kk) to the caller
    void store(int64_t t0, int64_t kk, cudaStream_t s) {
        if (!caller || in_place()) return;
        const size_t bytes = sizeof(double) * n * kk;
        if (std::is_same<T, double>::value) {
            SSSI_CHECK_CUDA(cudaMemcpyAsync(caller + t0 * n, tbuf.get(), bytes, cudaMemcpyDeviceToHost, s));
        } else if (caller_dev) {
            convert(tbuf.as<T>(), caller + t0 * n, n * kk, s);
        } else {
            convert(tbuf.as<T>(), dbuf.as<double>(), n * kk, s);
            SSSI_CHECK_CUDA(cudaMemcpyAsync(caller + t0 * n, dbuf.get(), bytes, cudaMemcpyDeviceToHost, s));
        }
        SSSI_CHECK_CUDA(cudaStreamSynchronize(s));
    }
};

inline int64_t chunk_steps(int64_t nt, int64_t cells) {
    return std::max<int64_t>(1, std::min<int64_t>(nt, (int64_t)(kChunkBytes / (sizeof(double) * cells))));
}


// Exact-order imaging: M = f_t*r_t + M, s2 = f_t^2 + s2 for t = 0..nt-1
// (mainRtmTimeCpmlFor2dAw.m:268-275,
// mainRtmTimeSpongeFor2dAw.m:263-268), then image = M ./ s2.
static __global__ void image_ascending_kernel(const double* f, const double* r, int64_t n, int64_t nt, double eps,
                                       double* image) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        double m = 0.0, s2 = eps;
        for (int64_t t = 0; t < nt; ++t) {
            const double ft = f[q + t * n], rt = r[q + t * n];
            m = __dadd_rn(__dmul_rn(ft, rt), m);
            s2 = __dadd_rn(__dmul_rn(ft, ft), s2);
        }
        image[q] = __ddiv_rn(m, s2);
    }
}

// image = (scale*M) / (eps + scale*S2)
static __global__ void image_finish_kernel(const double* m, const double* s2, int64_t n, double scale, double eps,
                                    double* image) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        image[q] = (scale * m[q]) / (eps + scale * s2[q]);
}

// Same from compensated FP32 sums (hi + lo).
static __global__ void image_finish_comp_kernel(const float2* m, const float2* s2, int64_t n, double scale, double eps,
                                         double* image) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const double mm = (double)m[q].x + (double)m[q].y, ss = (double)s2[q].x + (double)s2[q].y;
        image[q] = (scale * mm) / (eps + scale * ss);
    }
}

// out = a - b in T
template <typename T>
__global__ void diff_kernel(const T* a, const T* b, T* out, int64_t n) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        out[q] = a[q] - b[q];
}

// out = a + b in T
template <typename T>
__global__ void sum_kernel(const T* a, const T* b, T* out, int64_t n) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        out[q] = a[q] + b[q];
}

}  // namespace api
}  // namespace sssi
