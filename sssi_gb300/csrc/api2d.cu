// C-ABI entry points of the 2D propagators and the RTM shot.
#include <algorithm>
#include <initializer_list>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "api_util.cuh"
#include "batch2d.cuh"
#include "cpml2d.cuh"

namespace sssi {

namespace {

using namespace api;

// Launch shape for a grid: rows per block (a power of two <= 256) and the
// number of columns each block marches over.
void pick_launch(int64_t nz, int64_t nx, int& bz, int& w) {
    // widest march (least halo recomputation: 2N-1 extra columns per block) that
    // still gives about eight warps per SM; small grids, which reach that with no
    // shape, take the most warps (32-row blocks, 4-column marches)
    const int64_t target_warps = 152 * 8;
    for (int cbz : {128, 64, 32}) {
        if ((cbz == 128 && nz < 512) || (cbz == 64 && nz < 96)) continue;
        const int64_t zblocks = (nz + cbz - 1) / cbz;
        for (int cand : {256, 128, 64, 32, 16, 8}) {
            const int64_t blocks = zblocks * ((nx + cand - 1) / cand);
            if (blocks * (cbz / 32) >= target_warps) {
                bz = cbz;
                w = cand;
                return;
            }
        }
    }
    bz = 32;
    w = 4;
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

template <class Prop>
void download_padded(const Prop& st, bool previous, double* model, cudaStream_t s) {
    using T = typename Prop::value_type;
    const int L = st.L();
    const int64_t rows = st.nz() + 2 * L, cols = st.padded_cols();
    DeviceView out(model, (size_t)(rows * cols), false, s);
    const T* f = previous ? st.previous() : st.current();
    const T* base = f - st.origin();
    const int64_t row0 = (st.origin() % st.ldp()) - L;
    padded_to_dense_kernel<T><<<152 * 4, 256, 0, s>>>(base, st.ldp(), row0, rows, cols, out.ptr);
    count_launch();
    SSSI_CHECK_CUDA(cudaGetLastError());
    out.download(model, (size_t)(rows * cols), s);
}

// ---------------------------------------------------------------- forward
template <class Prop>
void fwd2d_dense(const double* v, const double* source, int64_t nz, int64_t nx, int64_t nt, int N, int nB, double dz,
                 double dx, double dt, double* data, double* snapshot, bool strict) {
    using T = typename Prop::value_type;
    cudaStream_t s = current_stream();
    const int64_t n = nz * nx;
    std::vector<double> vh = host_copy(v, (size_t)n, s);
    Prop st(vh.data(), nz, nx, N, nB, dz, dx, dt, strict, s);
    int bz, w;
    pick_launch(nz, nx, bz, w);
    st.set_launch(bz, w);
    Staged<T> rec(data, (size_t)(nx * nt), false, s);
    const int64_t K = chunk_steps(nt, n);
    SliceStream<T> src(const_cast<double*>(source), n, K), snap(snapshot, n, K);
    timing_begin(s);
    for (int64_t t0 = 0; t0 < nt; t0 += K) {
        const int64_t kk = std::min(K, nt - t0);
        src.load(t0, kk, s);
        for (int64_t t = t0; t < t0 + kk; ++t) {
            StepIO<T> io;
            io.t = (int)t;
            if (source) io.src_dense = src.slice(t, t0);
            if (data) io.rec = rec.ptr + t * nx;
            if (snapshot) io.snap = snap.slice(t, t0);
            st.step(io);
        }
        snap.store(t0, kk, s);
    }
    timing_end(s);
    st.check_errors();
    rec.download(data, s);
    SSSI_CHECK_CUDA(cudaStreamSynchronize(s));
}

template <class Prop>
void fwd2d_point(const double* v, int64_t nz, int64_t nx, int64_t nt, int N, int nB, double dz, double dx, double dt,
                 int nsrc, const int64_t* iz, const int64_t* ix, const double* wavelets, double* data,
                 double* snapshot, bool strict) {
    using T = typename Prop::value_type;
    cudaStream_t s = current_stream();
    const int64_t n = nz * nx;
    std::vector<double> vh = host_copy(v, (size_t)n, s);
    Prop st(vh.data(), nz, nx, N, nB, dz, dx, dt, strict, s);
    int bz, w;
    pick_launch(nz, nx, bz, w);
    st.set_launch(bz, w);
    Staged<T> wav(wavelets, (size_t)(nsrc * nt), true, s);
    st.set_point_sources(nsrc, iz, ix, wav.ptr, (int)nt);
    Staged<T> rec(data, (size_t)(nx * nt), false, s);
    const int64_t K = chunk_steps(nt, n);
    SliceStream<T> snap(snapshot, n, K);
    timing_begin(s);
    for (int64_t t0 = 0; t0 < nt; t0 += K) {
        const int64_t kk = std::min(K, nt - t0);
        for (int64_t t = t0; t < t0 + kk; ++t) {
            StepIO<T> io;
            io.t = (int)t;
            if (data) io.rec = rec.ptr + t * nx;
            if (snapshot) io.snap = snap.slice(t, t0);
            st.step(io);
        }
        snap.store(t0, kk, s);
    }
    timing_end(s);
    st.check_errors();
    rec.download(data, s);
    SSSI_CHECK_CUDA(cudaStreamSynchronize(s));
}

// ---------------------------------------------------------------- reverse
template <class Prop>
void rvs2d_dense(const double* v, const double* data, int64_t nz, int64_t nx, int64_t nt, int N, int nB, double dz,
                 double dx, double dt, double* model, double* snapshot, bool strict) {
    using T = typename Prop::value_type;
    cudaStream_t s = current_stream();
    const int64_t n = nz * nx;
    std::vector<double> vh = host_copy(v, (size_t)n, s);
    Prop st(vh.data(), nz, nx, N, nB, dz, dx, dt, strict, s);
    int bz, w;
    pick_launch(nz, nx, bz, w);
    st.set_launch(bz, w);
    Staged<T> rows(data, (size_t)(nx * nt), true, s);
    const int64_t K = chunk_steps(nt, n);
    SliceStream<T> snap(snapshot, n, K);
    timing_begin(s);
    // chunks [t0, t_hi) visited from the end of time to the start
    for (int64_t t_hi = nt; t_hi > 0; t_hi -= K) {
        const int64_t t0 = std::max<int64_t>(0, t_hi - K);
        for (int64_t t = t_hi - 1; t >= t0; --t) {
            StepIO<T> io;
            io.t = (int)t;
            if (data) io.src_row = rows.ptr + t * nx;
            if (snapshot) io.snap = snap.slice(t, t0);
            st.step(io);
        }
        snap.store(t0, t_hi - t0, s);
    }
    timing_end(s);
    st.check_errors();
    // the reference returns the field held as "old" after its final rotation
    if (model) download_padded(st, nt > 0, model, s);
    SSSI_CHECK_CUDA(cudaStreamSynchronize(s));
}

// ---------------------------------------------------------------- RTM shot, strict FP64
// The reference's operation order throughout: the row-marching kernel for the
// three propagations, every reverse snapshot kept, and the imaging sums taken
// in ascending time (mainRtmTimeCpmlFor2dAw.m:268-275), so the image is
// bit-identical to the reference's.
void rtm2d_strict(const double* v, const double* vs, int64_t nz, int64_t nx, int64_t nt, int N, int nB, double dz,
                  double dx, double dt, const double* wavelet, int64_t src_iz, int64_t src_ix, double eps,
                  double* image, double* data_true, double* data_smooth) {
    using Prop = Cpml2d<double, double>;
    cudaStream_t s = current_stream();
    const int64_t n = nz * nx;
    std::vector<double> vh = host_copy(v, (size_t)n, s);
    std::vector<double> vsh = host_copy(vs, (size_t)n, s);
    Prop A(vh.data(), nz, nx, N, nB, dz, dx, dt, true, s);
    Prop B(vsh.data(), nz, nx, N, nB, dz, dx, dt, true, s);
    int bz, w;
    pick_launch(nz, nx, bz, w);
    A.set_launch(bz, w);
    B.set_launch(bz, w);
    Staged<double> wav(wavelet, (size_t)nt, true, s);
    A.set_point_sources(1, &src_iz, &src_ix, wav.ptr, (int)nt);
    B.set_point_sources(1, &src_iz, &src_ix, wav.ptr, (int)nt);
    const size_t ndata = (size_t)(nx * std::max<int64_t>(nt, 1));
    Staged<double> dtrue(data_true, ndata, false, s), dsmooth(data_smooth, ndata, false, s);
    DeviceBuffer dtrue_own, dsmooth_own, delta;
    double* d_true = dtrue.ptr;
    double* d_smooth = dsmooth.ptr;
    if (!d_true) {
        dtrue_own.allocate(sizeof(double) * ndata);
        d_true = dtrue_own.as<double>();
    }
    if (!d_smooth) {
        dsmooth_own.allocate(sizeof(double) * ndata);
        d_smooth = dsmooth_own.as<double>();
    }
    delta.allocate(sizeof(double) * ndata);
    DeviceBuffer fsnap, rsnap;
    fsnap.allocate(sizeof(double) * n * std::max<int64_t>(nt, 1));
    rsnap.allocate(sizeof(double) * n * std::max<int64_t>(nt, 1));

    // forward modelling in the true and the migration model
    timing_begin(s);
    for (int64_t t = 0; t < nt; ++t) {
        StepIO<double> io;
        io.t = (int)t;
        io.rec = d_true + t * nx;
        A.step(io);
        StepIO<double> jo;
        jo.t = (int)t;
        jo.rec = d_smooth + t * nx;
        jo.snap = fsnap.as<double>() + t * n;
        B.step(jo);
    }
    // dataTrue - dataSmooth (mainRtmTimeCpmlFor2dAw.m:252), injected in reverse time
    diff_kernel<double><<<152 * 4, 256, 0, s>>>(d_true, d_smooth, delta.as<double>(), nx * nt);
    count_launch();
    SSSI_CHECK_CUDA(cudaGetLastError());
    timing_mark(s);

    // reverse propagation in the true model, every snapshot kept
    A.reset();
    A.set_point_sources(0, nullptr, nullptr, nullptr, (int)nt);
    for (int64_t t = nt - 1; t >= 0; --t) {
        StepIO<double> io;
        io.t = (int)t;
        io.src_row = delta.as<double>() + t * nx;
        io.snap = rsnap.as<double>() + t * n;
        A.step(io);
    }
    timing_mark(s);

    DeviceView dimg(image, (size_t)n, false, s);
    image_ascending_kernel<<<152 * 4, 256, 0, s>>>(fsnap.as<double>(), rsnap.as<double>(), n, nt, eps, dimg.ptr);
    count_launch();
    SSSI_CHECK_CUDA(cudaGetLastError());
    timing_end(s);
    A.check_errors();
    B.check_errors();
    dimg.download(image, (size_t)n, s);
    if (dtrue.ptr) dtrue.download(data_true, s);
    if (dsmooth.ptr) dsmooth.download(data_smooth, s);
    SSSI_CHECK_CUDA(cudaStreamSynchronize(s));
}

// ================================================================ batched engine
// Fails the call with SSSI_ERR_UNSTABLE when a step found a non-finite value on
// the receiver row of one of the shots ks.
template <typename T>
void require_stable(Batch2d<T>& B, std::initializer_list<int> ks) {
    const std::vector<int> st = B.statuses();
    for (int k : ks)
        SSSI_REQUIRE(k < 0 || k >= (int)st.size() || st[k] != SSSI_ERR_UNSTABLE, SSSI_ERR_UNSTABLE,
                     "the wavefield became non-finite (is dt beyond the stability limit of the grid and the "
                     "velocities?)");
}

// Dense copy of a padded field (device) for the reverse pass's model output.
template <typename T>
void download_field(const T* field, int64_t ldp, int L, int64_t nz, int64_t nx, double* model, cudaStream_t s) {
    const int64_t rows = nz + 2 * L, cols = nx + 2 * L;
    DeviceView out(model, (size_t)(rows * cols), false, s);
    // field points at interior (0,0); padded (0,0) is L rows up and L columns left
    const T* base = field - L - (int64_t)L * ldp;
    padded_to_dense_kernel<T><<<152 * 4, 256, 0, s>>>(base, ldp, 0, rows, cols, out.ptr);
    count_launch();
    SSSI_CHECK_CUDA(cudaGetLastError());
    out.download(model, (size_t)(rows * cols), s);
}

template <typename T>
void bfwd2d(const double* v, const double* source, int64_t nz, int64_t nx, int64_t nt, int N, int nB, double dz,
            double dx, double dt, int nsrc, const int64_t* iz, const int64_t* ix, const double* wavelets, double* data,
            double* snapshot) {
    cudaStream_t s = current_stream();
    const int64_t n = nz * nx;
    Batch2d<T> B(N, dz, dx, s);
    const int k = B.add_shot(v, nz, nx, nB, dt, (int)nt, 0, false);
    Staged<T> wav(wavelets, (size_t)(nsrc * nt), true, s);
    if (nsrc) B.set_point_sources(k, nsrc, iz, ix, wav.ptr);
    Staged<T> rec(data, (size_t)(nx * nt), false, s);
    B.shot(k).rec = rec.ptr;
    // dense sources and snapshots stream through the device in chunks of steps
    const int64_t K = (source || snapshot) ? chunk_steps(nt, n) : std::max<int64_t>(nt, 1);
    SliceStream<T> src(const_cast<double*>(source), n, K), snap(snapshot, n, K);
    B.finalize();
    B.set_step(0);
    timing_begin(s);
    for (int64_t t0 = 0; t0 < nt; t0 += K) {
        const int64_t kk = std::min(K, nt - t0);
        src.load(t0, kk, s);
        ShotTail<T>& d = B.shot(k);
        d.src_dense = source ? src.slice(t0, t0) : nullptr;
        d.dense_t0 = (int)t0;
        d.snap = snapshot ? snap.slice(t0, t0) : nullptr;
        d.snap_t0 = (int)t0;
        B.sync_desc(k);
        B.run((int)kk);
        snap.store(t0, kk, s);
    }
    timing_end(s);
    B.check_errors();
    require_stable(B, {k});
    rec.download(data, s);
    SSSI_CHECK_CUDA(cudaStreamSynchronize(s));
}

template <typename T>
void brvs2d(const double* v, const double* data, int64_t nz, int64_t nx, int64_t nt, int N, int nB, double dz,
            double dx, double dt, double* model, double* snapshot) {
    cudaStream_t s = current_stream();
    const int64_t n = nz * nx;
    Batch2d<T> B(N, dz, dx, s);
    const int k = B.add_shot(v, nz, nx, nB, dt, (int)nt, 0, true);
    Staged<T> rows(data, (size_t)(nx * nt), true, s);
    B.shot(k).src_row = data ? rows.ptr : nullptr;
    const int64_t K = snapshot ? chunk_steps(nt, n) : std::max<int64_t>(nt, 1);
    SliceStream<T> snap(snapshot, n, K);
    B.finalize();
    B.set_step(0);
    timing_begin(s);
    // chunks [t0, t_hi) visited from the end of time to the start
    for (int64_t t_hi = nt; t_hi > 0; t_hi -= K) {
        const int64_t t0 = std::max<int64_t>(0, t_hi - K);
        ShotTail<T>& d = B.shot(k);
        d.snap = snapshot ? snap.slice(t0, t0) : nullptr;
        d.snap_t0 = (int)t0;
        B.sync_desc(k);
        B.run((int)(t_hi - t0));
        snap.store(t0, t_hi - t0, s);
    }
    timing_end(s);
    B.check_errors();
    require_stable(B, {k});
    // the reference returns the field held as "old" after its final rotation:
    // the result of the step before the last one
    if (model) {
        const ShotTail<T>& d = B.shot(k);
        const T* prev = d.field[(nt + 1) & 1];
        download_field(prev, d.ldp, B.L(), nz, nx, model, s);
    }
    SSSI_CHECK_CUDA(cudaStreamSynchronize(s));
}

template <typename T>
void brtm2d(const double* v, const double* vs, int64_t nz, int64_t nx, int64_t nt, int N, int nB, double dz,
            double dx, double dt, const double* wavelet, int64_t src_iz, int64_t src_ix, double eps, int stride,
            double* image, double* data_true, double* data_smooth) {
    constexpr bool kF16 = std::is_same<T, float>::value;
    cudaStream_t s = current_stream();
    const int64_t n = nz * nx;
    if (!kF16) stride = 1;
    SSSI_REQUIRE(stride >= 1, SSSI_ERR_ARG, "snap_stride must be >= 1");
    Batch2d<T> B(N, dz, dx, s);
    // Forward over batch steps [0, nt), reverse in v over [nt, 2nt).  FP32: the
    // field in vs and the residual D = (field in v) - (field in vs) advance as
    // one residual pair, so dataTrue - dataSmooth (D's row 0) keeps FP32
    // accuracy relative to itself even where the two fields nearly cancel.
    // FP64: the two forward shots and their difference, as the reference.
    int kA = -1, kB = -1, kR = -1;
    if (kF16) {
        kB = B.add_pair_shot(vs, v, nz, nx, nB, dt, (int)nt, 0);
        kR = B.add_shot(v, nz, nx, nB, dt, (int)nt, (int)nt, true);
    } else {
        kA = B.add_shot(v, nz, nx, nB, dt, (int)nt, 0, false);
        kB = B.add_shot(vs, nz, nx, nB, dt, (int)nt, 0, false);
        kR = B.add_shot_like(kA, (int)nt, (int)nt, true);
    }
    Staged<T> wav(wavelet, (size_t)nt, true, s);
    if (kA >= 0) B.set_point_sources(kA, 1, &src_iz, &src_ix, wav.ptr);
    B.set_point_sources(kB, 1, &src_iz, &src_ix, wav.ptr);
    const size_t ndata = (size_t)(nx * std::max<int64_t>(nt, 1));
    Staged<T> dtrue(data_true, ndata, false, s), dsmooth(data_smooth, ndata, false, s);
    DeviceBuffer dtrue_own, dsmooth_own, delta;
    T* d_true = dtrue.ptr;
    T* d_smooth = dsmooth.ptr;
    if (!d_true && !kF16) {
        dtrue_own.allocate(sizeof(T) * ndata);
        d_true = dtrue_own.as<T>();
    }
    if (!d_smooth) {
        dsmooth_own.allocate(sizeof(T) * ndata);
        d_smooth = dsmooth_own.as<T>();
    }
    delta.allocate(sizeof(T) * ndata);
    const int64_t nsnap = (nt + stride - 1) / stride;
    const int64_t nblk = ((nz + 31) / 32) * ((nx + 31) / 32);  // FP16 scale blocks of 32 x 32 cells
    DeviceBuffer fsnap, amax, perr, M, S2;
    if (kF16) {
        fsnap.allocate(sizeof(__half) * n * std::max<int64_t>(nsnap, 1));
        amax.allocate(sizeof(unsigned) * nblk * std::max<int64_t>(nsnap, 1));
        amax.zero(s);
        perr.allocate(sizeof(float) * n);
        perr.zero(s);
    } else {
        fsnap.allocate(sizeof(double) * n * std::max<int64_t>(nt, 1));
    }
    M.allocate(sizeof(double) * n);  // FP64 sums, or compensated FP32 (hi, lo) pairs of the same size
    S2.allocate(sizeof(double) * n);
    M.zero(s);
    if (kF16)
        S2.zero(s);
    else
        fill(S2.as<double>(), n, eps, s);

    if (kA >= 0) B.shot(kA).rec = d_true;
    ShotTail<T>& b = B.shot(kB);
    b.rec = d_smooth;
    if (kF16) b.rec_d = delta.as<T>();
    if (kF16) {
        b.stride = stride;
        b.amax = amax.as<unsigned>();
        b.pack = fsnap.as<__half>();
        b.s2acc = S2.as<float2>();  // the illumination from the FP32 forward field
        b.perr = perr.as<float>();
    } else {
        b.snap = reinterpret_cast<T*>(fsnap.as<double>());
        b.snap_t0 = 0;
    }
    ShotTail<T>& r = B.shot(kR);
    r.src_row = delta.as<T>();
    if (kF16) {
        r.stride = stride;
        r.img_f16 = fsnap.as<__half>();
        r.img_amax = amax.as<unsigned>();
        r.img_m2 = M.as<float2>();
    } else {
        r.img_f64 = fsnap.as<double>();
        r.img_m = M.as<double>();
        r.img_s2 = S2.as<double>();
    }
    // only the shots active in a phase take part in its schedule
    B.enable(kR, false);
    B.finalize();
    B.set_step(0);

    timing_begin(s);
    B.run((int)nt);
    if (kF16 && nt >= 1 && (nt - 1) % stride == 0) {
        const int64_t k = (nt - 1) / stride;
        launch_pack_f16(reinterpret_cast<const float*>(B.current_field(kB)), B.ldp(kB), (int)nz, (int)nx,
                        amax.as<unsigned>() + k * nblk, fsnap.as<__half>() + k * n, perr.as<float>(), s);
    }
    // dataTrue - dataSmooth (mainRtmTimeCpmlFor2dAw.m:252), injected in reverse
    // time: D's row 0 for the residual pair, else the difference of the two
    if (!kF16) {
        diff_kernel<T><<<152 * 4, 256, 0, s>>>(d_true, d_smooth, delta.as<T>(), nx * nt);
        count_launch();
    } else if (d_true) {
        sum_kernel<T><<<152 * 4, 256, 0, s>>>(d_smooth, delta.as<T>(), d_true, nx * nt);
        count_launch();
    }
    SSSI_CHECK_CUDA(cudaGetLastError());
    timing_mark(s);
    if (kA >= 0) B.enable(kA, false);
    B.enable(kB, false);
    B.enable(kR, true);
    B.finalize();
    B.run((int)nt);
    timing_mark(s);

    DeviceView dimg(image, (size_t)n, false, s);
    if (kF16)
        image_finish_comp_kernel<<<152 * 4, 256, 0, s>>>(M.as<float2>(), S2.as<float2>(), n, (double)stride, eps,
                                                          dimg.ptr);
    else
        image_finish_kernel<<<152 * 4, 256, 0, s>>>(M.as<double>(), S2.as<double>(), n, 1.0, 0.0, dimg.ptr);
    count_launch();
    SSSI_CHECK_CUDA(cudaGetLastError());
    timing_end(s);
    B.check_errors();
    require_stable(B, {kA, kB, kR});
    dimg.download(image, (size_t)n, s);
    if (dtrue.ptr) dtrue.download(data_true, s);
    if (dsmooth.ptr) dsmooth.download(data_smooth, s);
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
        if (mode == SSSI_MODE_FP64_STRICT)
            fwd2d_dense<Cpml2d<double, double>>(v, source, nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, data,
                                                snapshot, mode == SSSI_MODE_FP64_STRICT);
        else if (mode == SSSI_MODE_FP32)
            bfwd2d<float>(v, source, nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, 0, nullptr, nullptr, nullptr, data,
                          snapshot);
        else
            bfwd2d<double>(v, source, nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, 0, nullptr, nullptr, nullptr,
                           data, snapshot);
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
        if (mode == SSSI_MODE_FP64_STRICT)
            fwd2d_point<Cpml2d<double, double>>(v, nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, nsrc, src_iz, src_ix,
                                                wavelets, data, snapshot, mode == SSSI_MODE_FP64_STRICT);
        else if (mode == SSSI_MODE_FP32)
            bfwd2d<float>(v, nullptr, nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, nsrc, src_iz, src_ix, wavelets,
                          data, snapshot);
        else
            bfwd2d<double>(v, nullptr, nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, nsrc, src_iz, src_ix, wavelets,
                           data, snapshot);
    });
}

extern "C" int sssi_rvsTimeCpmlFor2dAw(const double* v, const double* data, int64_t nz, int64_t nx, int64_t nt,
                                       int nDiffOrder, int nBoundary, double dz, double dx, double dt, double* model,
                                       double* snapshot, int mode) {
    return guarded([&] {
        check_common(nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, mode);
        SSSI_REQUIRE(v != nullptr, SSSI_ERR_ARG, "v is NULL");
        ensure_device();
        if (mode == SSSI_MODE_FP64_STRICT)
            rvs2d_dense<Cpml2d<double, double>>(v, data, nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, model, snapshot,
                                                mode == SSSI_MODE_FP64_STRICT);
        else if (mode == SSSI_MODE_FP32)
            brvs2d<float>(v, data, nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, model, snapshot);
        else
            brvs2d<double>(v, data, nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, model, snapshot);
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
            brtm2d<float>(v, vs, nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, wavelet, src_iz, src_ix, epsilon,
                          snap_stride, image, data_true, data_smooth);
        else if (mode == SSSI_MODE_FP64)
            brtm2d<double>(v, vs, nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, wavelet, src_iz, src_ix, epsilon, 1,
                           image, data_true, data_smooth);
        else
            rtm2d_strict(v, vs, nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, wavelet, src_iz, src_ix, epsilon,
                         image, data_true, data_smooth);
    });
}
