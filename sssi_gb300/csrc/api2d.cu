// C-ABI entry points of the 2D propagators and the RTM shot.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "cpml2d.cuh"

namespace sssi {

namespace {

constexpr size_t kChunkBytes = size_t(256) << 20;  // host<->device streaming granularity

std::vector<double> host_copy(const double* p, size_t n, cudaStream_t s) {
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

// Launch shape for a grid: rows per block (a power of two <= 256) and the
// number of columns each block marches over.
void pick_launch(int64_t nz, int64_t nx, int& bz, int& w) {
    bz = nz >= 512 ? 128 : (nz >= 96 ? 64 : 32);
    const int64_t target_warps = 152 * 8;
    const int64_t zblocks = (nz + bz - 1) / bz;
    w = 16;
    for (int cand : {256, 128, 64, 32}) {
        const int64_t blocks = zblocks * ((nx + cand - 1) / cand);
        if (blocks * (bz / 32) >= target_warps) {
            w = cand;
            break;
        }
    }
}

void check_common(int64_t nz, int64_t nx, int64_t nt, int N, int nB, double dz, double dx, double dt, int mode) {
    SSSI_REQUIRE(nz > 0 && nx > 0 && nt >= 0, SSSI_ERR_ARG, "bad sizes nz=%lld nx=%lld nt=%lld", (long long)nz,
                 (long long)nx, (long long)nt);
    SSSI_REQUIRE(N >= 1 && N <= kMaxOrder, SSSI_ERR_ARG, "nDiffOrder must be in 1..%d (got %d)", kMaxOrder, N);
    SSSI_REQUIRE(nB >= 0, SSSI_ERR_ARG, "nBoundary must be >= 0 (got %d)", nB);
    SSSI_REQUIRE(dz > 0 && dx > 0 && dt > 0, SSSI_ERR_ARG, "dz, dx, dt must be positive");
    SSSI_REQUIRE(mode == SSSI_MODE_FP64_STRICT || mode == SSSI_MODE_FP64 || mode == SSSI_MODE_FP32, SSSI_ERR_ARG,
                 "unknown mode %d", mode);
}

// Copies the padded field (ldp rows per column, interior origin) to a dense
// (nz+2l) x (nx+2l) double array (device).
template <typename T>
__global__ void padded_to_dense_kernel(const T* base, int64_t ldp, int64_t row0, int64_t rows, int64_t cols,
                                       double* out) {
    const int64_t n = rows * cols;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = q % rows, c = q / rows;
        out[q] = static_cast<double>(base[row0 + r + c * ldp]);
    }
}

// Exact-order imaging: M = f_t*r_t + M, s2 = f_t^2 + s2 for t = 0..nt-1
// (mainRtmTimeCpmlFor2dAw.m:268-275), then image = M ./ s2.
__global__ void image_ascending_kernel(const double* f, const double* r, int64_t n, int64_t nt, double eps,
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
__global__ void image_finish_kernel(const double* m, const double* s2, int64_t n, double scale, double eps,
                                    double* image) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        image[q] = (scale * m[q]) / (eps + scale * s2[q]);
}

__global__ void fill_kernel(double* p, int64_t n, double v) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        p[q] = v;
}

void fill(double* p, int64_t n, double v, cudaStream_t s) {
    fill_kernel<<<152 * 4, 256, 0, s>>>(p, n, v);
    count_launch();
    SSSI_CHECK_CUDA(cudaGetLastError());
}

template <typename T>
void download_padded(const Cpml2d<T, double>& st, bool previous, double* model, cudaStream_t s) {
    const int L = st.L();
    const int64_t rows = st.nz() + 2 * L, cols = st.padded_cols();
    DeviceView out(model, (size_t)(rows * cols), false, s);
    const int k = previous ? 1 : 0;
    // field(k) is relative to the current index; base() indexes the raw buffers
    const T* f = previous ? st.previous() : st.current();
    const T* base = f - st.origin();
    const int64_t row0 = (st.origin() % st.ldp()) - L;
    (void)k;
    padded_to_dense_kernel<T><<<152 * 4, 256, 0, s>>>(base, st.ldp(), row0, rows, cols, out.ptr);
    count_launch();
    SSSI_CHECK_CUDA(cudaGetLastError());
    out.download(model, (size_t)(rows * cols), s);
}

// ---------------------------------------------------------------- forward
template <typename T>
void fwd2d_dense(const double* v, const double* source, int64_t nz, int64_t nx, int64_t nt, int N, int nB, double dz,
                 double dx, double dt, double* data, double* snapshot, bool strict) {
    cudaStream_t s = current_stream();
    const int64_t n = nz * nx;
    std::vector<double> vh = host_copy(v, (size_t)n, s);
    Cpml2d<T, double> st(vh.data(), nz, nx, N, nB, dz, dx, dt, strict, s);
    int bz, w;
    pick_launch(nz, nx, bz, w);
    st.set_launch(bz, w);

    DeviceView ddata(data, (size_t)(nx * nt), false, s);
    const bool src_dev = source && is_device_pointer(source);
    const bool snap_dev = snapshot && is_device_pointer(snapshot);
    const int64_t K = std::max<int64_t>(1, std::min<int64_t>(nt, (int64_t)(kChunkBytes / (sizeof(double) * n))));
    DeviceBuffer srcbuf, snapbuf;
    if (source && !src_dev) srcbuf.allocate(sizeof(double) * n * K);
    if (snapshot && !snap_dev) snapbuf.allocate(sizeof(double) * n * K);

    for (int64_t t0 = 0; t0 < nt; t0 += K) {
        const int64_t kk = std::min(K, nt - t0);
        if (source && !src_dev)
            SSSI_CHECK_CUDA(cudaMemcpyAsync(srcbuf.get(), source + t0 * n, sizeof(double) * n * kk,
                                            cudaMemcpyHostToDevice, s));
        for (int64_t t = t0; t < t0 + kk; ++t) {
            StepIO io;
            io.t = (int)t;
            if (source) io.src_dense = src_dev ? source + t * n : srcbuf.as<double>() + (t - t0) * n;
            if (data) io.rec = ddata.ptr + t * nx;
            if (snapshot) io.snap = snap_dev ? snapshot + t * n : snapbuf.as<double>() + (t - t0) * n;
            st.step(io);
        }
        if (snapshot && !snap_dev) {
            SSSI_CHECK_CUDA(cudaMemcpyAsync(snapshot + t0 * n, snapbuf.get(), sizeof(double) * n * kk,
                                            cudaMemcpyDeviceToHost, s));
            SSSI_CHECK_CUDA(cudaStreamSynchronize(s));
        }
    }
    ddata.download(data, (size_t)(nx * nt), s);
    SSSI_CHECK_CUDA(cudaStreamSynchronize(s));
}

template <typename T>
void fwd2d_point(const double* v, int64_t nz, int64_t nx, int64_t nt, int N, int nB, double dz, double dx, double dt,
                 int nsrc, const int64_t* iz, const int64_t* ix, const double* wavelets, double* data,
                 double* snapshot, bool strict) {
    cudaStream_t s = current_stream();
    const int64_t n = nz * nx;
    std::vector<double> vh = host_copy(v, (size_t)n, s);
    Cpml2d<T, double> st(vh.data(), nz, nx, N, nB, dz, dx, dt, strict, s);
    int bz, w;
    pick_launch(nz, nx, bz, w);
    st.set_launch(bz, w);
    DeviceView dwav(wavelets, (size_t)(nsrc * nt), true, s);
    st.set_point_sources(nsrc, iz, ix, dwav.ptr, (int)nt);
    DeviceView ddata(data, (size_t)(nx * nt), false, s);
    const bool snap_dev = snapshot && is_device_pointer(snapshot);
    const int64_t K = std::max<int64_t>(1, std::min<int64_t>(nt, (int64_t)(kChunkBytes / (sizeof(double) * n))));
    DeviceBuffer snapbuf;
    if (snapshot && !snap_dev) snapbuf.allocate(sizeof(double) * n * K);
    timing_begin(s);
    for (int64_t t0 = 0; t0 < nt; t0 += K) {
        const int64_t kk = std::min(K, nt - t0);
        for (int64_t t = t0; t < t0 + kk; ++t) {
            StepIO io;
            io.t = (int)t;
            if (data) io.rec = ddata.ptr + t * nx;
            if (snapshot) io.snap = snap_dev ? snapshot + t * n : snapbuf.as<double>() + (t - t0) * n;
            st.step(io);
        }
        if (snapshot && !snap_dev) {
            SSSI_CHECK_CUDA(cudaMemcpyAsync(snapshot + t0 * n, snapbuf.get(), sizeof(double) * n * kk,
                                            cudaMemcpyDeviceToHost, s));
            SSSI_CHECK_CUDA(cudaStreamSynchronize(s));
        }
    }
    timing_end(s);
    ddata.download(data, (size_t)(nx * nt), s);
    SSSI_CHECK_CUDA(cudaStreamSynchronize(s));
}

// ---------------------------------------------------------------- reverse
template <typename T>
void rvs2d_dense(const double* v, const double* data, int64_t nz, int64_t nx, int64_t nt, int N, int nB, double dz,
                 double dx, double dt, double* model, double* snapshot, bool strict) {
    cudaStream_t s = current_stream();
    const int64_t n = nz * nx;
    std::vector<double> vh = host_copy(v, (size_t)n, s);
    Cpml2d<T, double> st(vh.data(), nz, nx, N, nB, dz, dx, dt, strict, s);
    int bz, w;
    pick_launch(nz, nx, bz, w);
    st.set_launch(bz, w);
    DeviceView ddata(data, (size_t)(nx * nt), true, s);
    const bool snap_dev = snapshot && is_device_pointer(snapshot);
    const int64_t K = std::max<int64_t>(1, std::min<int64_t>(nt, (int64_t)(kChunkBytes / (sizeof(double) * n))));
    DeviceBuffer snapbuf;
    if (snapshot && !snap_dev) snapbuf.allocate(sizeof(double) * n * K);
    // chunks [t0, t0+kk) visited from the end of time to the start
    for (int64_t t_hi = nt; t_hi > 0; t_hi -= K) {
        const int64_t t0 = std::max<int64_t>(0, t_hi - K);
        for (int64_t t = t_hi - 1; t >= t0; --t) {
            StepIO io;
            io.t = (int)t;
            if (data) io.src_row = ddata.ptr + t * nx;
            if (snapshot) io.snap = snap_dev ? snapshot + t * n : snapbuf.as<double>() + (t - t0) * n;
            st.step(io);
        }
        if (snapshot && !snap_dev) {
            SSSI_CHECK_CUDA(cudaMemcpyAsync(snapshot + t0 * n, snapbuf.get(), sizeof(double) * n * (t_hi - t0),
                                            cudaMemcpyDeviceToHost, s));
            SSSI_CHECK_CUDA(cudaStreamSynchronize(s));
        }
    }
    // the reference returns the field held as "old" after its final rotation
    if (model) download_padded<T>(st, nt > 0, model, s);
    SSSI_CHECK_CUDA(cudaStreamSynchronize(s));
}

// ---------------------------------------------------------------- RTM shot
template <typename T>
void rtm2d(const double* v, const double* vs, int64_t nz, int64_t nx, int64_t nt, int N, int nB, double dz, double dx,
           double dt, const double* wavelet, int64_t src_iz, int64_t src_ix, double eps, int mode, int stride,
           double* image, double* data_true, double* data_smooth) {
    cudaStream_t s = current_stream();
    const int64_t n = nz * nx;
    const bool strict = mode == SSSI_MODE_FP64_STRICT;
    const bool f16 = mode == SSSI_MODE_FP32;
    if (!f16) stride = 1;
    SSSI_REQUIRE(stride >= 1, SSSI_ERR_ARG, "snap_stride must be >= 1");
    std::vector<double> vh = host_copy(v, (size_t)n, s);
    std::vector<double> vsh = host_copy(vs, (size_t)n, s);
    Cpml2d<T, double> A(vh.data(), nz, nx, N, nB, dz, dx, dt, strict, s);
    Cpml2d<T, double> B(vsh.data(), nz, nx, N, nB, dz, dx, dt, strict, s);
    int bz, w;
    pick_launch(nz, nx, bz, w);
    A.set_launch(bz, w);
    B.set_launch(bz, w);
    DeviceView dwav(wavelet, (size_t)nt, true, s);
    A.set_point_sources(1, &src_iz, &src_ix, dwav.ptr, (int)nt);
    B.set_point_sources(1, &src_iz, &src_ix, dwav.ptr, (int)nt);
    DeviceView dtrue(data_true, (size_t)(nx * nt), false, s);
    DeviceView dsmooth(data_smooth, (size_t)(nx * nt), false, s);
    DeviceBuffer dtrue_own, dsmooth_own;
    double* d_true = dtrue.ptr;
    double* d_smooth = dsmooth.ptr;
    if (!d_true) {
        dtrue_own.allocate(sizeof(double) * nx * std::max<int64_t>(nt, 1));
        d_true = dtrue_own.as<double>();
    }
    if (!d_smooth) {
        dsmooth_own.allocate(sizeof(double) * nx * std::max<int64_t>(nt, 1));
        d_smooth = dsmooth_own.as<double>();
    }

    const int64_t nsnap = f16 ? (nt + stride - 1) / stride : nt;
    DeviceBuffer fsnap, rsnap, amax, inv, M, S2;
    if (f16) {
        fsnap.allocate(sizeof(__half) * n * std::max<int64_t>(nsnap, 1));
        amax.allocate(sizeof(unsigned) * std::max<int64_t>(nsnap, 1));
        amax.zero(s);
        inv.allocate(sizeof(float) * std::max<int64_t>(nsnap, 1));
    } else {
        fsnap.allocate(sizeof(double) * n * std::max<int64_t>(nt, 1));
        if (strict) rsnap.allocate(sizeof(double) * n * std::max<int64_t>(nt, 1));
    }
    if (!strict) {
        M.allocate(sizeof(double) * n);
        S2.allocate(sizeof(double) * n);
        M.zero(s);
        if (f16)
            S2.zero(s);
        else
            fill(S2.as<double>(), n, eps, s);
    }

    // forward modelling in the true and the migration model
    timing_begin(s);
    for (int64_t t = 0; t < nt; ++t) {
        StepIO io;
        io.t = (int)t;
        io.rec = d_true + t * nx;
        A.step(io);
        StepIO jo;
        jo.t = (int)t;
        jo.rec = d_smooth + t * nx;
        if (!f16) {
            jo.snap = fsnap.as<double>() + t * n;
        } else {
            if (t % stride == 0) jo.amax = amax.as<unsigned>() + t / stride;
            if (t >= 1 && (t - 1) % stride == 0) {
                const int64_t k = (t - 1) / stride;
                jo.pack = fsnap.as<__half>() + k * n;
                jo.pack_amax = amax.as<unsigned>() + k;
                jo.pack_inv_scale_out = inv.as<float>() + k;
            }
        }
        B.step(jo);
    }
    if (f16 && nt >= 1 && (nt - 1) % stride == 0) {
        const int64_t k = (nt - 1) / stride;
        launch_pack_f16(reinterpret_cast<const float*>(B.current()), B.ldp(), (int)nz, (int)nx,
                        amax.as<unsigned>() + k, fsnap.as<__half>() + k * n, inv.as<float>() + k, s);
    }

    timing_mark(s);
    // reverse propagation of dataTrue - dataSmooth in the true model, imaging
    A.reset();
    A.set_point_sources(0, nullptr, nullptr, nullptr, (int)nt);
    for (int64_t t = nt - 1; t >= 0; --t) {
        StepIO io;
        io.t = (int)t;
        io.src_row = d_true + t * nx;
        io.src_row_sub = d_smooth + t * nx;
        if (strict) {
            io.snap = rsnap.as<double>() + t * n;
        } else if (!f16) {
            io.img_f64 = fsnap.as<double>() + t * n;
            io.img_m = M.as<double>();
            io.img_s2 = S2.as<double>();
        } else if (t % stride == 0) {
            io.img_f16 = fsnap.as<__half>() + (t / stride) * n;
            io.img_inv_scale = inv.as<float>() + t / stride;
            io.img_m = M.as<double>();
            io.img_s2 = S2.as<double>();
        }
        A.step(io);
    }
    timing_mark(s);

    DeviceView dimg(image, (size_t)n, false, s);
    if (strict) {
        image_ascending_kernel<<<152 * 4, 256, 0, s>>>(fsnap.as<double>(), rsnap.as<double>(), n, nt, eps, dimg.ptr);
    } else {
        image_finish_kernel<<<152 * 4, 256, 0, s>>>(M.as<double>(), S2.as<double>(), n, f16 ? (double)stride : 1.0,
                                                     f16 ? eps : 0.0, dimg.ptr);
    }
    count_launch();
    SSSI_CHECK_CUDA(cudaGetLastError());
    timing_end(s);
    dimg.download(image, (size_t)n, s);
    dtrue.download(data_true, (size_t)(nx * nt), s);
    dsmooth.download(data_smooth, (size_t)(nx * nt), s);
    SSSI_CHECK_CUDA(cudaStreamSynchronize(s));
}

}  // namespace
}  // namespace sssi

using namespace sssi;

extern "C" int sssi_fwdTimeCpmlFor2dAw(const double* v, const double* source, int64_t nz, int64_t nx, int64_t nt,
                                       int nDiffOrder, int nBoundary, double dz, double dx, double dt, double* data,
                                       double* snapshot, int mode) {
    return guarded([&] {
        check_common(nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, mode);
        SSSI_REQUIRE(v != nullptr, SSSI_ERR_ARG, "v is NULL");
        ensure_device();
        if (mode == SSSI_MODE_FP32)
            fwd2d_dense<float>(v, source, nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, data, snapshot, false);
        else
            fwd2d_dense<double>(v, source, nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, data, snapshot,
                                mode == SSSI_MODE_FP64_STRICT);
    });
}

extern "C" int sssi_fwdTimeCpmlFor2dAwPoint(const double* v, int64_t nz, int64_t nx, int64_t nt, int nDiffOrder,
                                            int nBoundary, double dz, double dx, double dt, int nsrc,
                                            const int64_t* src_iz, const int64_t* src_ix, const double* wavelets,
                                            double* data, double* snapshot, int mode) {
    return guarded([&] {
        check_common(nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, mode);
        SSSI_REQUIRE(v != nullptr, SSSI_ERR_ARG, "v is NULL");
        SSSI_REQUIRE(nsrc >= 0 && nsrc <= kMaxPointSources, SSSI_ERR_ARG, "nsrc must be in 0..%d", kMaxPointSources);
        SSSI_REQUIRE(nsrc == 0 || (src_iz && src_ix && wavelets), SSSI_ERR_ARG, "point-source arrays are NULL");
        ensure_device();
        if (mode == SSSI_MODE_FP32)
            fwd2d_point<float>(v, nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, nsrc, src_iz, src_ix, wavelets, data,
                               snapshot, false);
        else
            fwd2d_point<double>(v, nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, nsrc, src_iz, src_ix, wavelets,
                                data, snapshot, mode == SSSI_MODE_FP64_STRICT);
    });
}

extern "C" int sssi_rvsTimeCpmlFor2dAw(const double* v, const double* data, int64_t nz, int64_t nx, int64_t nt,
                                       int nDiffOrder, int nBoundary, double dz, double dx, double dt, double* model,
                                       double* snapshot, int mode) {
    return guarded([&] {
        check_common(nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, mode);
        SSSI_REQUIRE(v != nullptr, SSSI_ERR_ARG, "v is NULL");
        ensure_device();
        if (mode == SSSI_MODE_FP32)
            rvs2d_dense<float>(v, data, nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, model, snapshot, false);
        else
            rvs2d_dense<double>(v, data, nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, model, snapshot,
                                mode == SSSI_MODE_FP64_STRICT);
    });
}

extern "C" int sssi_rtmTimeCpmlFor2dAw(const double* v, const double* vs, int64_t nz, int64_t nx, int64_t nt,
                                       int nDiffOrder, int nBoundary, double dz, double dx, double dt,
                                       const double* wavelet, int64_t src_iz, int64_t src_ix, double epsilon,
                                       int mode, int snap_stride, double* image, double* data_true,
                                       double* data_smooth) {
    return guarded([&] {
        check_common(nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, mode);
        SSSI_REQUIRE(v && vs && wavelet && image, SSSI_ERR_ARG, "v, vs, wavelet and image are required");
        SSSI_REQUIRE(src_iz >= 0 && src_iz < nz && src_ix >= 0 && src_ix < nx, SSSI_ERR_ARG,
                     "source (%lld, %lld) outside the model", (long long)src_iz, (long long)src_ix);
        SSSI_REQUIRE(epsilon >= 0, SSSI_ERR_ARG, "epsilon must be >= 0");
        ensure_device();
        if (mode == SSSI_MODE_FP32)
            rtm2d<float>(v, vs, nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, wavelet, src_iz, src_ix, epsilon, mode,
                         snap_stride, image, data_true, data_smooth);
        else
            rtm2d<double>(v, vs, nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, wavelet, src_iz, src_ix, epsilon,
                          mode, snap_stride, image, data_true, data_smooth);
    });
}
