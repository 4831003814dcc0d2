// Host side of the tiled 2D CPML step: device state, tensor maps, launches.
#include <cmath>
#include <cudaTypedefs.h>

#include <mutex>

#include "tile2d.cuh"

namespace sssi {

bool encode_tensor_map_2d(CUtensorMap* map, const void* base, CUtensorMapDataType dtype, size_t elem_bytes,
                          uint64_t rows, uint64_t cols, uint64_t ld, uint32_t box_rows, uint32_t box_cols) {
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
        else
            cudaGetLastError();
    });
    if (!encode) return false;
    const cuuint64_t dims[2] = {rows, cols};
    const cuuint64_t strides[1] = {ld * elem_bytes};
    const cuuint32_t box[2] = {box_rows, box_cols};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = encode(map, dtype, 2, const_cast<void*>(base), dims, strides, box, estr,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

namespace {

template <typename T>
struct TmaType;
template <>
struct TmaType<float> {
    static constexpr CUtensorMapDataType kType = CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
};
template <>
struct TmaType<double> {
    static constexpr CUtensorMapDataType kType = CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
};

// Band coefficients in the element type of the tiled kernel.  In FP32, b - 1
// comes from expm1 so that it keeps full relative precision near b = 1.
template <typename T>
void band_coefficients(const std::vector<double>& b, const std::vector<double>& bm1, std::vector<T>& ob,
                       std::vector<T>& obm1) {
    ob.resize(b.size());
    obm1.resize(b.size());
    for (size_t k = 0; k < b.size(); ++k) {
        ob[k] = static_cast<T>(b[k]);
        if constexpr (std::is_same<T, float>::value) {
            // b = exp(-d dt) was computed in double; log recovers -d dt exactly enough
            obm1[k] = static_cast<float>(std::expm1(std::log(b[k])));
        } else {
            obm1[k] = bm1[k];
        }
    }
}

// Composed second-derivative coefficients a_0..a_l of D-(D+ .) for weights w.
void composed(const double* w, int N, double* a) {
    const int L = 2 * N - 1;
    for (int m = 0; m <= L; ++m) a[m] = 0.0;
    for (int k = 0; k < N; ++k)
        for (int n = 0; n < N; ++n) {
            const double ww = w[k] * w[n];
            a[k + n + 1] += ww;  // +P(i+k+n+1) (and its mirror +P(i-1-k-n))
            // -P(i+k-n) and -P(i-k+n): over ordered pairs each |k-n| > 0 is met
            // twice (once per sign), while k = n puts both terms on P(i)
            const int d = k - n;
            a[d < 0 ? -d : d] -= (d == 0 ? 2.0 : 1.0) * ww;
        }
}

}  // namespace

template <typename T>
Tile2d<T>::Tile2d(const double* v, int64_t nz, int64_t nx, int N, int nB, double dz, double dx, double dt,
                  bool strict, cudaStream_t stream)
    : nz_(nz), nx_(nx), N_(N), L_(2 * N - 1), nB_(nB), stream_(stream) {
    SSSI_REQUIRE(!strict, SSSI_ERR_INTERNAL, "the tiled kernel has no strict arithmetic");
    SSSI_REQUIRE(N >= 1 && N <= kMaxOrder, SSSI_ERR_ARG, "nDiffOrder must be in 1..%d (got %d)", kMaxOrder, N);
    SSSI_REQUIRE(nz >= 1 && nx >= 1, SSSI_ERR_ARG, "empty model (%lld x %lld)", (long long)nz, (long long)nx);
    SSSI_REQUIRE(nB >= 0 && nB <= nz && 2 * (int64_t)nB <= nx, SSSI_ERR_ARG,
                 "nBoundary %d does not fit the model (%lld x %lld): need nBoundary <= nz and 2*nBoundary <= nx", nB,
                 (long long)nz, (long long)nx);
    SSSI_REQUIRE(nz < (1LL << 30) && nx < (1LL << 30), SSSI_ERR_ARG, "model too large");
    using Sh = TileShape<T>;
    const int HZ = tile_halo_rows(N);
    constexpr int al = Scalar<T>::kAlign;
    oz_ = (std::max(L_, HZ) + al - 1) / al * al;
    const int64_t nz_alloc = (nz + Sh::TZ - 1) / Sh::TZ * Sh::TZ;
    ldp_ = (oz_ + nz_alloc + HZ + al - 1) / al * al;
    origin_ = oz_ + (int64_t)L_ * ldp_;
    const int64_t cols = nx + 2 * L_;
    const size_t pbytes = sizeof(T) * (size_t)ldp_ * (size_t)cols;
    for (auto& b : P_) b.allocate(pbytes);
    vdt2_.allocate(pbytes);
    err_.allocate(sizeof(int));

    // (v dt)^2 in the padded layout (the TMA copies tiles of it like the fields)
    {
        const int64_t n = nz * nx;
        std::vector<T> h(n);
        for (int64_t q = 0; q < n; ++q) h[q] = static_cast<T>((v[q] * dt) * (v[q] * dt));
        vdt2_.zero(stream);
        SSSI_CHECK_CUDA(cudaMemcpy2DAsync(vdt2_.as<T>() + origin_, sizeof(T) * ldp_, h.data(), sizeof(T) * nz,
                                          sizeof(T) * nz, nx, cudaMemcpyHostToDevice, stream));
        SSSI_CHECK_CUDA(cudaStreamSynchronize(stream));
    }

    // coefficients
    double c[kMaxOrder], wz[kMaxOrder], wx[kMaxOrder], az[16], ax[16];
    staggered_coefficients(N, c);
    for (int k = 0; k < N; ++k) {
        wz[k] = c[k] / dz;
        wx[k] = c[k] / dx;
    }
    composed(wz, N, az);
    composed(wx, N, ax);
    for (int k = 0; k < 8; ++k) {
        tmpl_.wz[k] = k < N ? static_cast<T>(wz[k]) : T(0);
        tmpl_.wx[k] = k < N ? static_cast<T>(wx[k]) : T(0);
    }
    for (int m = 0; m < 16; ++m) {
        tmpl_.az[m] = m <= L_ ? static_cast<T>(az[m]) : T(0);
        tmpl_.ax[m] = m <= L_ ? static_cast<T>(ax[m]) : T(0);
    }

    // damping bands
    Bands2D bands = damping_bands_2d(v, nz, nx, nB, dz, dx, dt);
    auto upload = [&](DeviceBuffer& buf, const std::vector<T>& h) {
        buf.allocate(sizeof(T) * std::max<size_t>(h.size(), 1));
        if (!h.empty())
            SSSI_CHECK_CUDA(cudaMemcpyAsync(buf.get(), h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, stream));
        SSSI_CHECK_CUDA(cudaStreamSynchronize(stream));
    };
    std::vector<T> b, bm1;
    band_coefficients<T>(bands.zb, bands.zbm1, b, bm1);
    upload(zb_, b);
    upload(zbm1_, bm1);
    band_coefficients<T>(bands.xb, bands.xbm1, b, bm1);
    upload(xb_, b);
    upload(xbm1_, bm1);
    const size_t zbytes = sizeof(M) * std::max<size_t>((size_t)nB * nx, 1);
    const size_t xbytes = sizeof(M) * std::max<size_t>((size_t)nz * 2 * nB, 1);
    zphi_[0].allocate(zbytes);
    zphi_[1].allocate(zbytes);
    zpsi_.allocate(zbytes);
    xphi_[0].allocate(xbytes);
    xphi_[1].allocate(xbytes);
    xpsi_.allocate(xbytes);

    // tensor maps: P box of each field, tile box of each field, tile box of (v dt)^2
    const uint32_t box_rows = Sh::TZ + 2 * HZ, box_cols = Sh::TX + 2 * L_;
    for (int k = 0; k < 2; ++k) {
        SSSI_REQUIRE(encode_tensor_map_2d(&tm_box_[k], P_[k].get(), TmaType<T>::kType, sizeof(T), ldp_, cols, ldp_,
                                          box_rows, box_cols),
                     SSSI_ERR_CUDA, "cuTensorMapEncodeTiled failed for the field halo box");
        SSSI_REQUIRE(encode_tensor_map_2d(&tm_tile_[k], P_[k].get(), TmaType<T>::kType, sizeof(T), ldp_, cols, ldp_,
                                          Sh::TZ, Sh::TX),
                     SSSI_ERR_CUDA, "cuTensorMapEncodeTiled failed for the field tile box");
    }
    SSSI_REQUIRE(encode_tensor_map_2d(&tm_v_, vdt2_.get(), TmaType<T>::kType, sizeof(T), ldp_, cols, ldp_, Sh::TZ,
                                      Sh::TX),
                 SSSI_ERR_CUDA, "cuTensorMapEncodeTiled failed for (v dt)^2");

    tmpl_.nz = (int)nz;
    tmpl_.nx = (int)nx;
    tmpl_.nB = nB;
    tmpl_.ntz = (int)((nz + Sh::TZ - 1) / Sh::TZ);
    tmpl_.ntx = (int)((nx + Sh::TX - 1) / Sh::TX);
    tmpl_.oz = (int)oz_;
    tmpl_.ldp = ldp_;
    tmpl_.zb = zb_.as<T>();
    tmpl_.zbm1 = zbm1_.as<T>();
    tmpl_.zpsi = zpsi_.as<M>();
    tmpl_.xb = xb_.as<T>();
    tmpl_.xbm1 = xbm1_.as<T>();
    tmpl_.xpsi = xpsi_.as<M>();
    tmpl_.err = err_.as<int>();
    int sms = 0, dev = 0;
    SSSI_CHECK_CUDA(cudaGetDevice(&dev));
    SSSI_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int ntiles = tmpl_.ntz * tmpl_.ntx;
    grid_ = std::max(1, std::min(ntiles, sms * tile2d_ctas_per_sm<T>(N)));
    reset();
}

template <typename T>
void Tile2d<T>::reset() {
    for (auto& b : P_) b.zero(stream_);
    for (auto* b : {&zphi_[0], &zphi_[1], &zpsi_, &xphi_[0], &xphi_[1], &xpsi_, &err_}) b->zero(stream_);
    cur_ = 0;
    phase_ = 0;
}

template <typename T>
void Tile2d<T>::set_point_sources(int nsrc, const int64_t* iz, const int64_t* ix, const T* d_wavelet, int nt) {
    SSSI_REQUIRE(nsrc >= 0 && nsrc <= kMaxPointSources, SSSI_ERR_ARG, "at most %d point sources (got %d)",
                 kMaxPointSources, nsrc);
    tmpl_.nsrc = nsrc;
    for (int s = 0; s < nsrc; ++s) {
        SSSI_REQUIRE(iz[s] >= 0 && iz[s] < nz_ && ix[s] >= 0 && ix[s] < nx_, SSSI_ERR_ARG,
                     "point source %d at (%lld, %lld) outside the %lld x %lld model", s, (long long)iz[s],
                     (long long)ix[s], (long long)nz_, (long long)nx_);
        tmpl_.src_iz[s] = (int)iz[s];
        tmpl_.src_ix[s] = (int)ix[s];
    }
    tmpl_.src_wavelet = d_wavelet;
    tmpl_.nt = nt;
}

template <typename T>
void Tile2d<T>::step(const StepIO<T>& io) {
    TileStep<T> p = tmpl_;
    p.t = io.t;
    p.Pnew = field(1 - cur_);
    p.zphi_in = zphi_[phase_].template as<M>();
    p.zphi_out = zphi_[1 - phase_].template as<M>();
    p.xphi_in = xphi_[phase_].template as<M>();
    p.xphi_out = xphi_[1 - phase_].template as<M>();
    p.src_dense = io.src_dense;
    p.src_row = io.src_row;
    p.rec = io.rec;
    p.snap = io.snap;
    p.pack = io.pack;
    p.pack_amax = io.pack_amax;
    p.pack_inv_scale_out = io.pack_inv_scale_out;
    p.amax = io.amax;
    p.img_f64 = io.img_f64;
    p.img_f16 = io.img_f16;
    p.img_inv_scale = io.img_inv_scale;
    p.img_m = io.img_m;
    p.img_s2 = io.img_s2;
    p.img_m2 = io.img_m2;
    p.img_s22 = io.img_s22;
    if (p.nsrc == 0) p.src_wavelet = nullptr;
    launch_tile2d<T>(N_, tm_box_[cur_], tm_tile_[1 - cur_], tm_v_, p, grid_, stream_);
    cur_ = 1 - cur_;
    phase_ = 1 - phase_;
}

template <typename T>
void Tile2d<T>::check_errors() {
    int h = 0;
    SSSI_CHECK_CUDA(cudaMemcpyAsync(&h, err_.get(), sizeof(int), cudaMemcpyDeviceToHost, stream_));
    SSSI_CHECK_CUDA(cudaStreamSynchronize(stream_));
    SSSI_REQUIRE(h == 0, SSSI_ERR_INTERNAL, "a tile copy did not arrive within the wait limit (kernel aborted)");
}

template <typename T>
void launch_tile2d(int N, const CUtensorMap& tm_cur, const CUtensorMap& tm_old, const CUtensorMap& tm_v,
                   const TileStep<T>& p, int grid, cudaStream_t stream) {
    switch (N) {
        case 1: launch_tile2d_n<T, 1>(tm_cur, tm_old, tm_v, p, grid, stream); break;
        case 2: launch_tile2d_n<T, 2>(tm_cur, tm_old, tm_v, p, grid, stream); break;
        case 3: launch_tile2d_n<T, 3>(tm_cur, tm_old, tm_v, p, grid, stream); break;
        case 4: launch_tile2d_n<T, 4>(tm_cur, tm_old, tm_v, p, grid, stream); break;
        case 5: launch_tile2d_n<T, 5>(tm_cur, tm_old, tm_v, p, grid, stream); break;
        case 6: launch_tile2d_n<T, 6>(tm_cur, tm_old, tm_v, p, grid, stream); break;
        case 7: launch_tile2d_n<T, 7>(tm_cur, tm_old, tm_v, p, grid, stream); break;
        case 8: launch_tile2d_n<T, 8>(tm_cur, tm_old, tm_v, p, grid, stream); break;
        default: SSSI_REQUIRE(false, SSSI_ERR_ARG, "nDiffOrder %d out of range 1..8", N);
    }
}

template <typename T>
int tile2d_ctas_per_sm(int N) {
    switch (N) {
        case 1: return tile2d_occupancy_n<T, 1>();
        case 2: return tile2d_occupancy_n<T, 2>();
        case 3: return tile2d_occupancy_n<T, 3>();
        case 4: return tile2d_occupancy_n<T, 4>();
        case 5: return tile2d_occupancy_n<T, 5>();
        case 6: return tile2d_occupancy_n<T, 6>();
        case 7: return tile2d_occupancy_n<T, 7>();
        default: return tile2d_occupancy_n<T, 8>();
    }
}

template class Tile2d<float>;
template class Tile2d<double>;

}  // namespace sssi
