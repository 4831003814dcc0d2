// C-ABI entry points of the 3D propagator (fwdTimeCpmlFor3dAw.m).
#include <algorithm>

#include "api_util.cuh"
#include "prop3d.cuh"

namespace sssi {

namespace {

using namespace api;

void check3d(int64_t nz, int64_t nx, int64_t ny, int64_t nt, int N, int nB, double dz, double dx, double dy,
             double dt, int mode) {
    SSSI_REQUIRE(nz > 0 && nx > 0 && ny > 0 && nt >= 0, SSSI_ERR_ARG, "bad sizes nz=%lld nx=%lld ny=%lld nt=%lld",
                 (long long)nz, (long long)nx, (long long)ny, (long long)nt);
    SSSI_REQUIRE(N >= 1 && N <= kMaxOrder, SSSI_ERR_ARG, "nDiffOrder must be in 1..%d (got %d)", kMaxOrder, N);
    SSSI_REQUIRE(nB >= 0, SSSI_ERR_ARG, "nBoundary must be >= 0 (got %d)", nB);
    SSSI_REQUIRE(dz > 0 && dx > 0 && dy > 0 && dt > 0, SSSI_ERR_ARG, "dz, dx, dy, dt must be positive");
    SSSI_REQUIRE(mode == SSSI_MODE_FP64_STRICT || mode == SSSI_MODE_FP64 || mode == SSSI_MODE_FP32, SSSI_ERR_ARG,
                 "unknown mode %d", mode);
}

template <typename T>
void fwd3d(const double* v, const double* source, int64_t nz, int64_t nx, int64_t ny, int64_t nt, int N, int nB,
           double dz, double dx, double dy, double dt, int nsrc, const int64_t* iz, const int64_t* ix,
           const int64_t* iy, const double* wavelets, double* data, double* snapshot) {
    cudaStream_t s = current_stream();
    const int64_t n = nz * nx * ny;
    Prop3d<T> P(v, nz, nx, ny, N, nB, dz, dx, dy, dt, (int)nt, s);
    Staged<T> wav(wavelets, (size_t)(nsrc * nt), true, s);
    if (nsrc) P.set_point_sources(nsrc, iz, ix, iy, wav.ptr);
    Staged<T> rec(data, (size_t)(nx * ny * nt), false, s);
    Desc3<T>& d = P.desc();
    d.rec = rec.ptr;
    // dense sources and snapshots stream through the device in chunks of steps
    const int64_t K = (source || snapshot) ? chunk_steps(nt, n) : std::max<int64_t>(nt, 1);
    SliceStream<T> src(const_cast<double*>(source), n, K), snap(snapshot, n, K);
    timing_begin(s);
    for (int64_t t0 = 0; t0 < nt; t0 += K) {
        const int64_t kk = std::min(K, nt - t0);
        src.load(t0, kk, s);
        d.src_dense = source ? src.slice(t0, t0) : nullptr;
        d.dense_t0 = (int)t0;
        d.snap = snapshot ? snap.slice(t0, t0) : nullptr;
        d.snap_t0 = (int)t0;
        P.sync_desc();
        P.run((int)kk);
        snap.store(t0, kk, s);
    }
    timing_end(s);
    P.check_errors();
    rec.download(data, s);
    SSSI_CHECK_CUDA(cudaStreamSynchronize(s));
}

}  // namespace

}  // namespace sssi

using namespace sssi;

extern "C" int sssi_fwdTimeCpmlFor3dAw(const double* v, const double* source, int64_t nz, int64_t nx, int64_t ny,
                                       int64_t nt, int nDiffOrder, int nBoundary, double dz, double dx, double dy,
                                       double dt, double* data, double* snapshot, int mode) {
    return guarded([&] {
        check3d(nz, nx, ny, nt, nDiffOrder, nBoundary, dz, dx, dy, dt, mode);
        SSSI_REQUIRE(v != nullptr, SSSI_ERR_ARG, "v is NULL");
        ensure_device();
        if (mode == SSSI_MODE_FP32)
            fwd3d<float>(v, source, nz, nx, ny, nt, nDiffOrder, nBoundary, dz, dx, dy, dt, 0, nullptr, nullptr,
                         nullptr, nullptr, data, snapshot);
        else
            fwd3d<double>(v, source, nz, nx, ny, nt, nDiffOrder, nBoundary, dz, dx, dy, dt, 0, nullptr, nullptr,
                          nullptr, nullptr, data, snapshot);
    });
}

extern "C" int sssi_fwdTimeCpmlFor3dAwPoint(const double* v, int64_t nz, int64_t nx, int64_t ny, int64_t nt,
                                            int nDiffOrder, int nBoundary, double dz, double dx, double dy, double dt,
                                            int nsrc, const int64_t* src_iz, const int64_t* src_ix,
                                            const int64_t* src_iy, const double* wavelets, double* data,
                                            double* snapshot, int mode) {
    return guarded([&] {
        check3d(nz, nx, ny, nt, nDiffOrder, nBoundary, dz, dx, dy, dt, mode);
        SSSI_REQUIRE(v != nullptr, SSSI_ERR_ARG, "v is NULL");
        SSSI_REQUIRE(nsrc >= 0 && nsrc <= kMaxPointSources, SSSI_ERR_ARG, "nsrc must be in 0..%d", kMaxPointSources);
        SSSI_REQUIRE(nsrc == 0 || (src_iz && src_ix && src_iy && wavelets), SSSI_ERR_ARG,
                     "point-source arrays are NULL");
        ensure_device();
        if (mode == SSSI_MODE_FP32)
            fwd3d<float>(v, nullptr, nz, nx, ny, nt, nDiffOrder, nBoundary, dz, dx, dy, dt, nsrc, src_iz, src_ix,
                         src_iy, wavelets, data, snapshot);
        else
            fwd3d<double>(v, nullptr, nz, nx, ny, nt, nDiffOrder, nBoundary, dz, dx, dy, dt, nsrc, src_iz, src_ix,
                          src_iy, wavelets, data, snapshot);
    });
}
