// Host side of the batched 2D CPML step: shot state, descriptors, launches.
#include <cudaTypedefs.h>

#include <algorithm>

#include <cmath>
#include <mutex>
#include <functional>

#include "batch2d.cuh"

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
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
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

}  // namespace

template <typename T>
Batch2d<T>::Batch2d(int N, double dz, double dx, cudaStream_t stream)
    : N_(N), L_(2 * N - 1), dz_(dz), dx_(dx), stream_(stream) {
    SSSI_REQUIRE(N >= 1 && N <= kMaxOrder, SSSI_ERR_ARG, "nDiffOrder must be in 1..%d (got %d)", kMaxOrder, N);
    SSSI_REQUIRE(dz > 0 && dx > 0, SSSI_ERR_ARG, "dz and dx must be positive");
    double c[kMaxOrder], wz[kMaxOrder], wx[kMaxOrder], az[16], ax[16];
    staggered_coefficients(N, c);
    for (int k = 0; k < N; ++k) {
        wz[k] = c[k] / dz;
        wx[k] = c[k] / dx;
    }
    composed_coefficients(wz, N, az);
    composed_coefficients(wx, N, ax);
    for (int k = 0; k < 8; ++k) {
        bc_.wz[k] = k < N ? static_cast<T>(wz[k]) : T(0);
        bc_.wx[k] = k < N ? static_cast<T>(wx[k]) : T(0);
    }
    for (int m = 0; m < 16; ++m) {
        bc_.az[m] = m <= L_ ? static_cast<T>(az[m]) : T(0);
        bc_.ax[m] = m <= L_ ? static_cast<T>(ax[m]) : T(0);
        const float fz = static_cast<float>(bc_.az[m]), fx = static_cast<float>(bc_.ax[m]);
        bc_.az2[m] = make_float2(fz, fz);
        bc_.ax2[m] = make_float2(fx, fx);
    }
    d_ctr_.allocate(4 * sizeof(int));  // graph step base, zero, error flag, spare
    d_ctr_.zero(stream);
    bc_.step_base = d_ctr_.template as<int>() + 1;
    bc_.step_offset = 0;
    bc_.err = d_ctr_.template as<int>() + 2;
    bc_.wait_limit = kDefaultWaitLimit;
    bc_.debug_step = -1;
    {
        int step = -1;
        unsigned limit = 0;
        debug_withhold(&step, &limit);
        set_debug(step, limit);
    }
    int dev = 0;
    SSSI_CHECK_CUDA(cudaGetDevice(&dev));
    SSSI_CHECK_CUDA(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, dev));
    for (int v = 0; v < kBatchShapes<T>; ++v) ctas_per_sm_[v] = batch2d_ctas_per_sm<T>(N, v, false);
    if (kBatchShapes<T> > 1) ctas_per_sm_pair_ = batch2d_ctas_per_sm<T>(N, 1, true);
}

template <typename T>
int Batch2d<T>::add_shot(const double* v, int64_t nz, int64_t nx, int nB, double dt, int nt, int t_start,
                         bool reverse) {
    SSSI_REQUIRE(nz >= 1 && nx >= 1, SSSI_ERR_ARG, "empty model (%lld x %lld)", (long long)nz, (long long)nx);
    SSSI_REQUIRE(nB >= 0 && nB <= nz && 2 * (int64_t)nB <= nx, SSSI_ERR_ARG,
                 "nBoundary %d does not fit the model (%lld x %lld): need nBoundary <= nz and 2*nBoundary <= nx", nB,
                 (long long)nz, (long long)nx);
    SSSI_REQUIRE(nz <= 65535LL * 32 && nx <= 65535LL * 32, SSSI_ERR_ARG,
                 "model too large (%lld x %lld): at most %lld x %lld", (long long)nz, (long long)nx, 65535LL * 32,
                 65535LL * 32);
    SSSI_REQUIRE(dt > 0 && nt >= 0, SSSI_ERR_ARG, "dt must be positive and nt >= 0");
    const int slot = take_slot();
    stale_ = true;
    try {
        return add_shot_in(slot, v, -1, nz, nx, nB, dt, nt, t_start, reverse);
    } catch (...) {
        remove_shot(slot);
        throw;
    }
}

template <typename T>
int Batch2d<T>::add_shot_like(int k, int nt, int t_start, bool reverse) {
    SSSI_REQUIRE(k >= 0 && k < (int)shots_.size() && !shots_[k].free, SSSI_ERR_ARG, "no shot %d", k);
    SSSI_REQUIRE(nt >= 0, SSSI_ERR_ARG, "nt must be >= 0");
    const ShotTail<T> q = shots_[k].desc.s;
    const int slot = take_slot();
    stale_ = true;
    try {
        return add_shot_in(slot, nullptr, k, q.nz, q.nx, q.nB, 0.0, nt, t_start, reverse);
    } catch (...) {
        remove_shot(slot);
        throw;
    }
}

template <typename T>
int Batch2d<T>::add_pair_shot(const double* vp, const double* vq, int64_t nz, int64_t nx, int nB, double dt, int nt,
                              int t_start) {
    SSSI_REQUIRE((std::is_same<T, float>::value), SSSI_ERR_INTERNAL, "residual pairs are FP32 only");
    SSSI_REQUIRE(vp && vq, SSSI_ERR_ARG, "a residual pair needs both models");
    SSSI_REQUIRE(nz >= 1 && nx >= 1, SSSI_ERR_ARG, "empty model (%lld x %lld)", (long long)nz, (long long)nx);
    SSSI_REQUIRE(nB >= 0 && nB <= nz && 2 * (int64_t)nB <= nx, SSSI_ERR_ARG,
                 "nBoundary %d does not fit the model (%lld x %lld): need nBoundary <= nz and 2*nBoundary <= nx", nB,
                 (long long)nz, (long long)nx);
    SSSI_REQUIRE(nz <= 65535LL * 32 && nx <= 65535LL * 16, SSSI_ERR_ARG,
                 "model too large for a residual pair (%lld x %lld)", (long long)nz, (long long)nx);
    SSSI_REQUIRE(dt > 0 && nt >= 0, SSSI_ERR_ARG, "dt must be positive and nt >= 0");
    const int slot = take_slot();
    stale_ = true;
    try {
        return add_shot_in(slot, vp, -1, nz, nx, nB, dt, nt, t_start, false, vq);
    } catch (...) {
        remove_shot(slot);
        throw;
    }
}

template <typename T>
int Batch2d<T>::pairs_enabled() const {
    int n = 0;
    for (const Shot& S : shots_) n += (!S.free && S.enabled && S.desc.s.dcol > 0) ? 1 : 0;
    return n;
}

template <typename T>
int Batch2d<T>::take_slot() {
    for (int q = 0; q < (int)shots_.size(); ++q)
        if (shots_[q].free) {
            shots_[q].free = false;
            return q;
        }
    SSSI_REQUIRE(shots_.size() < (1u << 24), SSSI_ERR_ARG, "too many shots in one batch");
    shots_.emplace_back();
    return (int)shots_.size() - 1;
}

namespace {

// (vq dt)^2 - (vp dt)^2 in FP64, rounded once to T: the residual's source
// weight, exact to the last bit of T even where the two models nearly agree.
template <typename T>
__global__ void vdt2_diff_kernel(const double* vp, const double* vq, int64_t nz, int64_t nx, double dt, T* out,
                                 int64_t ldz) {
    const int64_t n = nz * nx;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const double a = vq[q] * dt, b = vp[q] * dt;
        out[(q % nz) + (q / nz) * ldz] = static_cast<T>(a * a - b * b);
    }
}

}  // namespace

template <typename T>
int Batch2d<T>::add_shot_in(int slot, const double* v, int like, int64_t nz, int64_t nx, int nB, double dt, int nt,
                            int t_start, bool reverse, const double* vq) {
    using Sh = TileShape<T>;
    shots_[slot] = Shot{};
    Shot& S = shots_[slot];
    ShotTail<T>& d = S.desc.s;
    const bool pair = vq != nullptr;
    const int HZ = tile_halo_rows(N_);
    constexpr int al = Scalar<T>::kAlign;
    const int64_t oz = (std::max(L_, HZ) + al - 1) / al * al;
    const int64_t nz_alloc = (nz + Sh::TZ - 1) / Sh::TZ * Sh::TZ;
    const int64_t ldp = (oz + nz_alloc + HZ + al - 1) / al * al;
    S.origin = oz + (int64_t)L_ * ldp;
    const int64_t cols = nx + 2 * L_;
    // a residual pair keeps D in the same buffers, dcol columns to the right of
    // P, past 8 zero columns (a tile box of D that starts left of D's padded
    // grid, as shifted tile columns do by up to 8 columns, reads zeros), and the
    // low part of P another dcol columns on
    const int64_t dcol = pair ? cols + 8 : 0;
    const int64_t cols_all = pair ? 2 * dcol + cols : cols;
    const size_t pbytes = sizeof(T) * (size_t)ldp * (size_t)cols_all;
    const int64_t nzb = (int64_t)nB * nx, nxb = nz * 2 * (int64_t)nB;  // band sizes (pair: per field)
    for (auto& b : S.P) b.allocate(pbytes);
    if (like >= 0) {
        // the same model as shot `like`: copy its (v dt)^2 and band coefficients
        auto copy = [&](DeviceBuffer& dst, const DeviceBuffer& src) {
            dst.allocate(src.bytes());
            SSSI_CHECK_CUDA(cudaMemcpyAsync(dst.get(), src.get(), src.bytes(), cudaMemcpyDeviceToDevice, up()));
        };
        const Shot& Q = shots_[like];
        SSSI_REQUIRE(Q.desc.s.dcol == 0, SSSI_ERR_INTERNAL, "a shot cannot copy a residual pair's model");
        copy(S.vdt2, Q.vdt2);
        copy(S.zb, Q.zb);
        copy(S.zbm1, Q.zbm1);
        copy(S.xb, Q.xb);
        copy(S.xbm1, Q.xbm1);
    } else {
        // (v dt)^2 on the device, from v where it lies (host models go up once
        // as doubles); the damping bands on the host, from the band strips of v
        const int64_t n = nz * nx;
        S.vdt2.allocate(pbytes);
        S.vdt2.zero(up());
        auto on_device = [&](const double* m, DeviceBuffer& tmp) {
            if (is_device_pointer(m)) return m;
            tmp.allocate(sizeof(double) * n);
            SSSI_CHECK_CUDA(cudaMemcpyAsync(tmp.get(), m, sizeof(double) * n, cudaMemcpyHostToDevice, up()));
            return static_cast<const double*>(tmp.template as<double>());
        };
        auto bands_of = [&](const double* m) {
            if (!is_device_pointer(m)) return damping_bands_2d(m, nz, nx, nB, dz_, dx_, dt);
            std::vector<double> bottom((size_t)nB * nx), sides((size_t)nz * 2 * nB);
            if (nB > 0) {
                SSSI_CHECK_CUDA(cudaMemcpy2DAsync(bottom.data(), sizeof(double) * nB, m + (nz - nB),
                                                  sizeof(double) * nz, sizeof(double) * nB, nx,
                                                  cudaMemcpyDeviceToHost, up()));
                SSSI_CHECK_CUDA(cudaMemcpyAsync(sides.data(), m, sizeof(double) * nz * nB, cudaMemcpyDeviceToHost,
                                                up()));
                SSSI_CHECK_CUDA(cudaMemcpyAsync(sides.data() + nz * nB, m + (nx - nB) * nz, sizeof(double) * nz * nB,
                                                cudaMemcpyDeviceToHost, up()));
            }
            SSSI_CHECK_CUDA(cudaStreamSynchronize(up()));
            return damping_bands_2d_strips(bottom.data(), sides.data(), nz, nx, nB, dz_, dx_, dt);
        };
        DeviceBuffer vd, vqd;
        const double* vdev = on_device(v, vd);
        launch_vdt2<T>(vdev, nz, nx, 1, dt, S.vdt2.template as<T>() + S.origin, ldp, ldp * cols_all, up());
        Bands2D bands = bands_of(v);
        std::vector<T> zb, zbm1, xb, xbm1;
        band_coefficients<T>(bands.zb, bands.zbm1, zb, zbm1);
        band_coefficients<T>(bands.xb, bands.xbm1, xb, xbm1);
        if (pair) {
            // D's (v dt)^2 column block holds (vq dt)^2 - (vp dt)^2 and its band
            // factors b_Q - b_P follow P's b: the residual uses P's rounded factors
            // plus these exact differences
            const double* vqdev = on_device(vq, vqd);
            vdt2_diff_kernel<T><<<152 * 4, 256, 0, up()>>>(vdev, vqdev, nz, nx, dt,
                                                          S.vdt2.template as<T>() + S.origin + dcol * ldp, ldp);
            count_launch();
            SSSI_CHECK_CUDA(cudaGetLastError());
            const Bands2D bq = bands_of(vq);
            for (size_t k = 0; k < bq.zb.size(); ++k) zb.push_back(static_cast<T>(bq.zb[k] - bands.zb[k]));
            for (size_t k = 0; k < bq.xb.size(); ++k) xb.push_back(static_cast<T>(bq.xb[k] - bands.xb[k]));
        }
        auto upload = [&](DeviceBuffer& buf, const std::vector<T>& h) {
            buf.allocate(sizeof(T) * std::max<size_t>(h.size(), 1));
            if (!h.empty())
                SSSI_CHECK_CUDA(cudaMemcpyAsync(buf.get(), h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice,
                                                up()));
        };
        upload(S.zb, zb);
        upload(S.zbm1, zbm1);
        upload(S.xb, xb);
        upload(S.xbm1, xbm1);
        SSSI_CHECK_CUDA(cudaStreamSynchronize(up()));  // vd and the host vectors go out of scope
    }
    const size_t fields = pair ? 2 : 1;  // memory variables of P, then D's
    const size_t zbytes = sizeof(M) * std::max<size_t>(fields * (size_t)nzb, 1);
    const size_t xbytes = sizeof(M) * std::max<size_t>(fields * (size_t)nxb, 1);
    for (auto* bf : {&S.zphi[0], &S.zphi[1], &S.zpsi}) bf->allocate(zbytes);
    for (auto* bf : {&S.xphi[0], &S.xphi[1], &S.xpsi}) bf->allocate(xbytes);

    for (int v = 0; v < kBatchShapes<T>; ++v) {  // boxes of every tile shape
        const uint32_t tz = (uint32_t)tile_z(v), tx = (uint32_t)tile_x(v);
        const uint32_t box_rows = tz + 2 * HZ, box_cols = tx + 2 * L_;
        for (int k = 0; k < 2; ++k) {
            SSSI_REQUIRE(encode_tensor_map_2d(&S.desc.tm_box[v][k], S.P[k].get(), TmaType<T>::kType, sizeof(T), ldp,
                                              cols_all, ldp, box_rows, box_cols),
                         SSSI_ERR_CUDA, "cuTensorMapEncodeTiled failed for the field halo box");
            SSSI_REQUIRE(encode_tensor_map_2d(&S.desc.tm_tile[v][k], S.P[k].get(), TmaType<T>::kType, sizeof(T), ldp,
                                              cols_all, ldp, tz, tx),
                         SSSI_ERR_CUDA, "cuTensorMapEncodeTiled failed for the field tile box");
        }
        SSSI_REQUIRE(encode_tensor_map_2d(&S.desc.tm_v[v], S.vdt2.get(), TmaType<T>::kType, sizeof(T), ldp, cols_all,
                                          ldp, tz, tx),
                     SSSI_ERR_CUDA, "cuTensorMapEncodeTiled failed for (v dt)^2");
    }
    d.field[0] = S.P[0].template as<T>() + S.origin;
    d.field[1] = S.P[1].template as<T>() + S.origin;
    d.zb = S.zb.template as<T>();
    d.zbm1 = S.zbm1.template as<T>();
    d.zphi[0] = S.zphi[0].template as<M>();
    d.zphi[1] = S.zphi[1].template as<M>();
    d.zpsi = S.zpsi.template as<M>();
    d.xb = S.xb.template as<T>();
    d.xbm1 = S.xbm1.template as<T>();
    d.xphi[0] = S.xphi[0].template as<M>();
    d.xphi[1] = S.xphi[1].template as<M>();
    d.xpsi = S.xpsi.template as<M>();
    d.ldp = ldp;
    d.nz = (int)nz;
    d.nx = (int)nx;
    d.nB = nB;
    d.ntz = (int)((nz + Sh::TZ - 1) / Sh::TZ);
    d.ntx = (int)((nx + Sh::TX - 1) / Sh::TX);
    d.oz = (int)oz;
    d.t_start = t_start;
    d.nt = nt;
    d.reverse = reverse ? 1 : 0;
    d.stride = 1;
    d.dcol = (int)dcol;
    reset_shot(slot);
    return slot;
}

template <typename T>
void Batch2d<T>::remove_shot(int k) {
    SSSI_REQUIRE(k >= 0 && k < (int)shots_.size() && !shots_[k].free, SSSI_ERR_ARG, "no shot %d", k);
    shots_[k] = Shot{};  // buffers go back to the pool
    shots_[k].enabled = false;
    shots_[k].free = true;
    stale_ = true;
}

template <typename T>
int Batch2d<T>::active_shots() const {
    int n = 0;
    for (const Shot& S : shots_) n += (!S.free && S.enabled) ? 1 : 0;
    return n;
}

template <typename T>
void Batch2d<T>::set_point_sources(int k, int nsrc, const int64_t* iz, const int64_t* ix, const T* d_wavelet) {
    SSSI_REQUIRE(nsrc >= 0 && nsrc <= kMaxPointSources, SSSI_ERR_ARG, "at most %d point sources (got %d)",
                 kMaxPointSources, nsrc);
    ShotTail<T>& d = shots_[k].desc.s;
    d.nsrc = nsrc;
    stale_ = true;  // point sources are part of the work items' flags
    for (int s = 0; s < nsrc; ++s) {
        SSSI_REQUIRE(iz[s] >= 0 && iz[s] < d.nz && ix[s] >= 0 && ix[s] < d.nx, SSSI_ERR_ARG,
                     "point source %d at (%lld, %lld) outside the %d x %d model", s, (long long)iz[s],
                     (long long)ix[s], d.nz, d.nx);
        d.src_iz[s] = (int)iz[s];
        d.src_ix[s] = (int)ix[s];
    }
    d.src_wavelet = nsrc ? d_wavelet : nullptr;
}

template <typename T>
void Batch2d<T>::reset_shot(int k) {
    clear_status(k);
    Shot& S = shots_[k];
    for (auto& b : S.P) b.zero(up());
    for (auto* b : {&S.zphi[0], &S.zphi[1], &S.zpsi, &S.xphi[0], &S.xphi[1], &S.xpsi}) b->zero(up());
}

template <typename T>
Batch2d<T>::~Batch2d() {
    drop_graph();
}

template <typename T>
void Batch2d<T>::drop_graph() {
    if (graph_) cudaGraphExecDestroy(graph_);
    graph_ = nullptr;
}

template <typename T>
int Batch2d<T>::tile_z(int shape) const {
    if constexpr (kBatchShapes<T> > 2) {
        if (shape == 1) return BatchShape<T, 1>::TZ;
        if (shape == 2) return BatchShape<T, 2>::TZ;
    }
    return TileShape<T>::TZ;
}

template <typename T>
int Batch2d<T>::tile_x(int shape) const {
    if constexpr (kBatchShapes<T> > 2) {
        if (shape == 1) return BatchShape<T, 1>::TX;
        if (shape == 2) return BatchShape<T, 2>::TX;
    }
    return TileShape<T>::TX;
}

template <typename T>
void Batch2d<T>::finalize() {
    // residual pairs run in the pair variant of the step, 32 x 32 whole tiles,
    // for every shot of the batch while any pair is enabled
    const bool was_pair = pair_;
    pair_ = pairs_enabled() > 0;
    if (pair_) {
        if (!was_pair) shape_free_ = shape_;
        schedule(1);
        use_shape(1);
        stale_ = false;
        return;
    }
    if (was_pair) shape_ = shape_free_;  // the shape in use before the pairs
    // the first large schedule (at least four whole tiles' worth per block) is
    // worth tuning the tile shape for, and one grown eightfold since
    int64_t tiles = 0;
    for (const Shot& S : shots_)
        if (S.enabled)
            tiles += ((int64_t)(S.desc.s.nz + TileShape<T>::TZ - 1) / TileShape<T>::TZ) *
                     ((S.desc.s.nx + TileShape<T>::TX - 1) / TileShape<T>::TX);
    const int forced = forced_tile_shape();
    if (forced >= 0 && forced < kBatchShapes<T>) {  // test knob: a fixed shape, no tuning
        tune_ = false;
        shape_ = forced;
    } else if (kBatchShapes<T> > 1 && tiles >= 4LL * sms_ * ctas_per_sm_[0] && tiles > 8LL * tuned_tiles_) {
        tune_ = true;
        tuned_tiles_ = (int)std::min<int64_t>(tiles, 1 << 30);
    }
    if (tune_)
        for (int v = 0; v < kBatchShapes<T>; ++v) schedule(v);  // every shape, for the tuner
    else
        schedule(shape_);
    use_shape(shape_);
    stale_ = false;
}

template <typename T>
void Batch2d<T>::use_shape(int shape) {
    shape_ = shape;
    grid_ = grid_s_[shape];
    ntiles_ = ntiles_s_[shape];
    split_ = split_s_[shape];
    bc_.nshots = (int)shots_.size();
    bc_.ntiles = ntiles_;
    bc_.cta_begin = d_cta_begin_[shape].template as<int>();
    bc_.work = d_work_[shape].template as<int2>();
}

template <typename T>
void Batch2d<T>::schedule(int shape) {
    const int TZs = tile_z(shape), TXs = tile_x(shape);
    // tiles of the enabled shots with an estimated cost: tiles whose stencil
    // reaches a damped band add a cooperative first-derivative pass and the
    // memory-variable traffic
    struct Item {
        int shot, z0, x0;
        unsigned flags;  // step-independent, and the half (1 left, 2 right) << 3 of a split tile
        float cost;
    };
    // a tile (or a half of width TX/2 at x0) with its step-independent flags and cost:
    // a tile next to a band costs more per banded direction (the cooperative pass and
    // the memory variables), partial tiles cost in proportion to their cells.  The
    // extra cost, measured: 1.2 interior tiles when the batch is small (its fields
    // stay in L2), 2.0 when it streams from HBM (at least 8 tiles per block), where
    // the memory variables' own bytes weigh more (the 64-shot batch and 4096^2
    // single grids step 0.7-0.8 % faster with 2.0; a two-shot 620 x 1240 forward
    // phase 4 % slower).
    float band_w = 1.2f;
    {
        int64_t n = 0;
        for (const Shot& S : shots_)
            if (S.enabled) n += (int64_t)((S.desc.s.nz + TZs - 1) / TZs) * ((S.desc.s.nx + TXs - 1) / TXs);
        if (n >= 8LL * sms_ * ctas_per_sm_[shape]) band_w = 2.0f;
    }
    const int cps = pair_ ? ctas_per_sm_pair_ : ctas_per_sm_[shape];  // resident blocks per SM
    auto tile_item = [&](int k, int z0, int x0, int width) {
        const ShotTail<T>& d = shots_[k].desc.s;
        unsigned f = tile_band_flags(N_, TZs, width, d.nz, d.nx, d.nB, z0, x0);
        const bool bz = f & kBandZ, bx = f & kBandX;
        for (int s = 0; s < d.nsrc; ++s)
            if (d.src_iz[s] >= z0 && d.src_iz[s] < z0 + TZs && d.src_ix[s] >= x0 && d.src_ix[s] < x0 + width)
                f |= kSource;
        const int rows = std::min(z0 + TZs, d.nz) - std::max(z0, 0);
        const int cols = std::max(0, std::min(x0 + width, d.nx) - std::max(x0, 0));
        const float fill = (float)(rows * cols) / (float)(TZs * TXs);
        const float pair_w = d.dcol > 0 ? 2.0f : 1.0f;  // a residual pair's tile advances two fields
        return Item{k, z0, x0, f,
                    pair_w * (0.3f + 0.7f * fill) * (1.0f + (bz ? band_w : 0.0f) + (bx ? band_w : 0.0f))};
    };
    // Tile rows of a shot start at row -zs (0 <= zs < TZs, a multiple of one
    // 32-byte sector of rows, so that the tiles' copies stay sector-aligned; the
    // rows above the grid are not computed).  The lowest rows whose second z
    // derivative reaches the damped band (zb0 - N + 1 on, zb0 = nz - nB) take
    // the two-stage form; a shift that puts them into one tile row instead of
    // two, with no more tile rows in all, saves a row of band tiles.  zs is a
    // function of the shot's grid and the tile shape only, so every cell of a
    // shot uses the same formula whichever shots share the batch.
    auto row_shift = [&](const ShotTail<T>& d) {
        const int cut = d.nz - d.nB - N_ + 1;
        if (d.nB <= 0 || cut < 0) return 0;
        auto cost = [&](int zs) {
            float c = 0.0f;
            for (int z0 = -zs; z0 < d.nz; z0 += TZs) {
                const int rows = std::min(z0 + TZs, d.nz) - std::max(z0, 0);
                const bool bz = tile_band_flags(N_, TZs, TXs, d.nz, d.nx, d.nB, z0, TXs) & kBandZ;
                c += (0.3f + 0.7f * (float)rows / (float)TZs) * (bz ? 2.2f : 1.0f);
            }
            return c;
        };
        constexpr int kSector = 32 / (int)sizeof(T);  // rows per 32-byte sector
        const int zs = (TZs - (cut / kSector * kSector) % TZs) % TZs;
        return (zs > 0 && cost(zs) < cost(0) - 1e-3f) ? zs : 0;
    };
    // Likewise tile columns start at column -xs (0 <= xs <= 8, even, so that a
    // thread's two columns are on one side of column 0): the shift with the
    // least estimated cost, which mostly means the columns reaching the right
    // band in one tile column instead of two (larger shifts would push the left
    // band's columns into a second tile column for the usual band widths).
    auto col_shift = [&](const ShotTail<T>& d) {
        if (d.nB <= 0) return 0;
        auto cost = [&](int xs) {
            float c = 0.0f;
            for (int x0 = -xs; x0 < d.nx; x0 += TXs) {
                const int cols = std::min(x0 + TXs, d.nx) - std::max(x0, 0);
                const bool bx = tile_band_flags(N_, TZs, TXs, d.nz, d.nx, d.nB, 0, x0) & kBandX;
                c += (0.3f + 0.7f * (float)cols / (float)TXs) * (bx ? 2.2f : 1.0f);
            }
            return c;
        };
        int best = 0;
        float cbest = cost(0);
        for (int xs = 2; xs <= 8; xs += 2) {
            const float c = cost(xs);
            if (c < cbest - 1e-3f) {
                best = xs;
                cbest = c;
            }
        }
        return best;
    };
    std::vector<Item> items;
    {
        size_t n = 0;
        for (const Shot& S : shots_)
            if (S.enabled) n += (size_t)((S.desc.s.nz + 2 * TZs - 1) / TZs) * ((S.desc.s.nx + 2 * TXs - 1) / TXs);
        items.reserve(n);
    }
    for (int k = 0; k < (int)shots_.size(); ++k) {
        if (!shots_[k].enabled) continue;
        const ShotTail<T>& d = shots_[k].desc.s;
        const int zs = row_shift(d), xs = col_shift(d);
        const int ntz = (d.nz + zs + TZs - 1) / TZs, ntx = (d.nx + xs + TXs - 1) / TXs;
        SSSI_REQUIRE((ntz - 1) * TZs - zs <= kMaxTileRow && (ntx - 1) * TXs - xs <= kMaxTileCol, SSSI_ERR_ARG,
                     "grid of %d x %d cells too large for the batched step", d.nz, d.nx);
        for (int q = 0; q < ntz * ntx; ++q) {
            const int z0 = (q % ntz) * TZs - zs, x0 = (q / ntz) * TXs - xs;
            items.push_back(tile_item(k, z0, x0, TXs));
        }
    }
    // A band tile takes several times as long as an interior one.  When a block
    // has less than two tiles' worth of work on average (small grids), one band
    // tile sets the length of the step: split the band tiles into two halves of
    // TX/2 columns (measured: a 620 x 1240 shot with 20-cell bands steps in 6.6
    // instead of 8.4 us; with two such shots, 2.9 tiles per block, splitting
    // loses 8 %).
    {
        float total = 0.0f;
        for (const Item& it : items) total += it.cost;
        const int blocks = std::max(1, std::min((int)items.size(), sms_ * cps));
        // FP64 tiles are bound by the FP64 pipe, so a band tile's extra work weighs
        // more against the step: split up to four tiles' worth per block.  A half
        // tile runs on half the block's threads and costs FP64 throughput, so
        // interior tiles are split only when the whole tiles do not reach every SM
        // (measured on C2's schedules: 7 % slower; on 77 tiles: 6.5 % faster).
        constexpr bool kF64 = std::is_same<T, double>::value;
        const float split_below = kF64 ? 4.0f : 2.0f;
        const bool split_interior = kF64 && (int)items.size() < sms_;
        split_s_[shape] = !pair_ && total < split_below * (float)blocks;  // the pair variant takes whole tiles only
        if (split_s_[shape]) {
            std::vector<Item> split;
            split.reserve(items.size() + items.size() / 4);
            for (const Item& it : items) {
                const ShotTail<T>& d = shots_[it.shot].desc.s;
                if ((!split_interior && !(it.flags & (kBandZ | kBandX))) || d.nx - it.x0 <= TXs / 2) {
                    split.push_back(it);
                    continue;
                }
                for (int h = 0; h < 2; ++h) {
                    // the half keeps the whole tile's band flags, so that every cell is
                    // computed by the same formula as in the unsplit tile (results do
                    // not depend on which shots share the batch)
                    Item hi = tile_item(it.shot, it.z0, it.x0 + h * (TXs / 2), TXs / 2);
                    const float band = (it.flags & kBandZ ? band_w : 0.0f) + (it.flags & kBandX ? band_w : 0.0f);
                    const float own = (hi.flags & kBandZ ? band_w : 0.0f) + (hi.flags & kBandX ? band_w : 0.0f);
                    hi.cost *= (1.0f + band) / (1.0f + own);
                    hi.flags = (hi.flags & ~(kBandZ | kBandX)) | (it.flags & (kBandZ | kBandX));
                    hi.x0 = it.x0;  // the work item keeps the tile position; the half selects the columns
                    hi.flags |= (unsigned)(h + 1) << 3;
                    split.push_back(hi);
                }
            }
            items.swap(split);
        }
    }
    const int ntiles = (int)items.size();
    const int grid = std::max(1, std::min(ntiles, sms_ * cps));
    ntiles_s_[shape] = ntiles;
    grid_s_[shape] = grid;
    // longest processing time first onto the least loaded CTA
    std::stable_sort(items.begin(), items.end(), [](const Item& a, const Item& b) { return a.cost > b.cost; });
    std::vector<int> owner(items.size());
    std::vector<int> begin(grid + 1, 0);
    {
        // Longest processing time first onto the least loaded block (a heap), except
        // for the longest run of equal costs (the whole interior tiles), which is
        // spread to level the loads directly: the same assignment up to ties, in
        // time linear in the tiles, so large batches reschedule quickly.
        using P = std::pair<float, int>;
        std::vector<P> heap;  // min-heap on load
        heap.reserve(grid);
        for (int c = 0; c < grid; ++c) heap.push_back({0.0f, c});
        const auto cmp = std::greater<P>();
        auto lpt = [&](size_t a, size_t b) {
            for (size_t q = a; q < b; ++q) {
                std::pop_heap(heap.begin(), heap.end(), cmp);
                P& top = heap.back();
                owner[q] = top.second;
                top.first += items[q].cost;
                std::push_heap(heap.begin(), heap.end(), cmp);
            }
        };
        size_t ra = 0, rb = 0;  // the longest run of equal costs
        for (size_t q = 0; q < items.size();) {
            size_t e = q;
            while (e < items.size() && items[e].cost == items[q].cost) ++e;
            if (e - q > rb - ra) {
                ra = q;
                rb = e;
            }
            q = e;
        }
        lpt(0, ra);
        if (rb > ra) {
            const float c = items[ra].cost;
            const int64_t m = (int64_t)(rb - ra);
            std::vector<double> load(grid);
            double sum = 0;
            for (const P& h : heap) {
                load[h.second] = h.first;
                sum += h.first;
            }
            const double level = (sum + (double)m * c) / grid;
            std::vector<int64_t> cnt(grid);
            int64_t given = 0;
            for (int b = 0; b < grid; ++b) {
                cnt[b] = std::max<int64_t>(0, (int64_t)std::floor((level - load[b]) / c));
                given += cnt[b];
            }
            if (given > m) {  // rounding: take back from the most loaded
                std::vector<int> order(grid);
                for (int b = 0; b < grid; ++b) order[b] = b;
                std::sort(order.begin(), order.end(),
                          [&](int x, int y) { return load[x] + cnt[x] * c > load[y] + cnt[y] * c; });
                for (int k = 0; given > m; k = (k + 1) % grid)
                    if (cnt[order[k]] > 0) {
                        --cnt[order[k]];
                        --given;
                    }
            }
            if (given < m) {  // the rest one each to the least loaded
                std::vector<int> order(grid);
                for (int b = 0; b < grid; ++b) order[b] = b;
                std::sort(order.begin(), order.end(),
                          [&](int x, int y) { return load[x] + cnt[x] * c < load[y] + cnt[y] * c; });
                for (int k = 0; given < m; k = (k + 1) % grid) {
                    ++cnt[order[k]];
                    ++given;
                }
            }
            // deal the run out block by block in turn, so that neighbouring tiles
            // go to different blocks
            size_t q = ra;
            for (int64_t round = 0; q < rb; ++round)
                for (int b = 0; b < grid && q < rb; ++b)
                    if (cnt[b] > round) owner[q++] = b;
            for (P& h : heap) h.first = (float)(load[h.second] + cnt[h.second] * c);
            std::make_heap(heap.begin(), heap.end(), cmp);
        }
        lpt(rb, items.size());
        for (size_t q = 0; q < items.size(); ++q) ++begin[owner[q] + 1];
    }
    for (int c = 0; c < grid; ++c) begin[c + 1] += begin[c];
    std::vector<int2> work(items.size());
    {
        std::vector<int> fill(begin.begin(), begin.end() - 1);
        for (size_t q = 0; q < items.size(); ++q) {
            const Item& it = items[q];
            work[fill[owner[q]]++] = pack_work_item(it.shot, it.flags, it.z0, it.x0);
        }
    }

    // descriptors of every slot in one copy
    const size_t nd = std::max<size_t>(shots_.size(), 1);
    if (d_desc_.bytes() < nd * sizeof(ShotDesc<T>)) d_desc_.allocate(nd * sizeof(ShotDesc<T>));
    ensure_status();
    std::vector<ShotDesc<T>> hdesc(shots_.size());
    for (int k = 0; k < (int)shots_.size(); ++k) {
        ShotTail<T>& d = shots_[k].desc.s;
        SSSI_REQUIRE(d.stride < (1 << 22), SSSI_ERR_ARG, "snapshot stride %d too large", d.stride);
        d.sched = sched_word(d);
        hdesc[k] = shots_[k].desc;
    }
    update_lean();
    if (!hdesc.empty())
        SSSI_CHECK_CUDA(cudaMemcpyAsync(d_desc_.get(), hdesc.data(), sizeof(ShotDesc<T>) * hdesc.size(),
                                        cudaMemcpyHostToDevice, stream_));
    DeviceBuffer& d_begin = d_cta_begin_[shape];
    DeviceBuffer& d_work = d_work_[shape];
    if (d_begin.bytes() < sizeof(int) * begin.size()) d_begin.allocate(sizeof(int) * begin.size());
    if (d_work.bytes() < sizeof(int2) * std::max<size_t>(work.size(), 1))
        d_work.allocate(sizeof(int2) * std::max<size_t>(work.size(), 1));
    SSSI_CHECK_CUDA(cudaMemcpyAsync(d_begin.get(), begin.data(), sizeof(int) * begin.size(),
                                    cudaMemcpyHostToDevice, stream_));
    if (!work.empty())
        SSSI_CHECK_CUDA(cudaMemcpyAsync(d_work.get(), work.data(), sizeof(int2) * work.size(),
                                        cudaMemcpyHostToDevice, stream_));
    SSSI_CHECK_CUDA(cudaStreamSynchronize(stream_));
}

template <typename T>
void Batch2d<T>::sync_desc(int k) {
    ShotTail<T>& d = shots_[k].desc.s;
    SSSI_REQUIRE(d.stride < (1 << 22), SSSI_ERR_ARG, "snapshot stride %d too large", d.stride);
    d.sched = sched_word(d);
    update_lean();
    SSSI_CHECK_CUDA(cudaMemcpyAsync(d_desc_.template as<ShotDesc<T>>() + k, &shots_[k].desc, sizeof(ShotDesc<T>),
                                    cudaMemcpyHostToDevice, stream_));
}

template <typename T>
void Batch2d<T>::update_lean() {
    // the variant without rare outputs takes whole single-field tiles; a batch
    // whose enabled shots write no snapshots, packs, maxima or imaging sums
    // runs it (the descriptors' sched words are current: called on upload)
    bool rare = false;
    for (const Shot& S : shots_)
        if (!S.free && S.enabled) rare |= (S.desc.s.sched & kSchedRareOut) != 0u;
    lean_ = !rare;
}

template <typename T>
void Batch2d<T>::set_step(int step) {
    step_ = step;
}

template <typename T>
void Batch2d<T>::launch_step(const int* base, int offset, cudaStream_t stream) {
    BatchConst<T> bc = bc_;
    bc.step_base = base;
    bc.step_offset = offset;
    launch_batch2d<T>(N_, d_desc_.template as<ShotDesc<T>>(), bc, grid_, split_, shape_, pair_, lean_, stream);
}

template <typename T>
void Batch2d<T>::run(int nsteps) {
    SSSI_REQUIRE(grid_ > 0 && !stale_, SSSI_ERR_INTERNAL, "Batch2d::run: the schedule is out of date (finalize)");
    int q = 0;
    if (tune_ && !pair_ && nsteps >= kTuneMinRun) {
        // tile-shape tuning: kTuneSteps steps with each shape, timed with events,
        // then the faster shape's schedule for the rest (the per-cell arithmetic
        // does not depend on the tiling, so the results do not either)
        tune_ = false;
        cudaEvent_t ev[2 * kMaxBatchShapes] = {};
        float ms[kMaxBatchShapes] = {};
        cudaError_t e = cudaSuccess;
        for (auto& x : ev)
            if (e == cudaSuccess) e = cudaEventCreate(&x);
        for (int v = 0; v < kBatchShapes<T> && e == cudaSuccess; ++v) {
            use_shape(v);
            e = cudaEventRecord(ev[2 * v], stream_);
            for (int i = 0; i < kTuneSteps && e == cudaSuccess; ++i) launch_step(bc_.step_base, step_ + q + i, stream_);
            q += kTuneSteps;
            if (e == cudaSuccess) e = cudaEventRecord(ev[2 * v + 1], stream_);
        }
        if (e == cudaSuccess) e = cudaEventSynchronize(ev[2 * kBatchShapes<T> - 1]);
        for (int v = 0; v < kBatchShapes<T> && e == cudaSuccess; ++v) e = cudaEventElapsedTime(&ms[v], ev[2 * v], ev[2 * v + 1]);
        for (auto& x : ev)
            if (x) cudaEventDestroy(x);
        SSSI_CHECK_CUDA(e);
        int best = 0;
        for (int v = 1; v < kBatchShapes<T>; ++v)
            if (ms[v] < ms[best]) best = v;
        use_shape(best);
        for (int v = 0; v < kBatchShapes<T>; ++v) tuned_ms_[v] = ms[v];
    }
    if (nsteps - q >= kGraphSteps) {
        int* base = d_ctr_.template as<int>();
        if (graph_ && !(graph_key_ == current_key())) drop_graph();
        if (!graph_) {
            graph_key_ = current_key();
            // steps base .. base+K-1, then base += K
            std::lock_guard<std::mutex> lock(capture_mutex());
            cudaStream_t cs = capture_stream();
            cudaGraph_t g = nullptr;
            SSSI_CHECK_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
            cudaError_t e = cudaSuccess;
            try {
                for (int k = 0; k < kGraphSteps; ++k) launch_step(base, k, cs);
                launch_add_int(base, kGraphSteps, cs);
            } catch (...) {
                cudaStreamEndCapture(cs, &g);  // leave the capture stream usable
                if (g) cudaGraphDestroy(g);
                throw;
            }
            count_launch(-kGraphSteps);  // recorded, not run
            const cudaError_t ee = cudaStreamEndCapture(cs, &g);
            if (e == cudaSuccess) e = ee;
            if (e == cudaSuccess) e = cudaGraphInstantiate(&graph_, g, 0);
            if (g) cudaGraphDestroy(g);
            if (e != cudaSuccess) graph_ = nullptr;
            SSSI_CHECK_CUDA(e);
        }
        launch_store_int(base, step_ + q, stream_);
        count_launch();
        for (; q + kGraphSteps <= nsteps; q += kGraphSteps) {
            SSSI_CHECK_CUDA(cudaGraphLaunch(graph_, stream_));
            count_launch(kGraphSteps + 1);
        }
    }
    for (; q < nsteps; ++q) launch_step(bc_.step_base, step_ + q, stream_);
    step_ += nsteps;
}

template <typename T>
const T* Batch2d<T>::current_field(int k) const {
    const ShotTail<T>& d = shots_[k].desc.s;
    int done = step_ - d.t_start;
    done = std::max(0, std::min(done, d.nt));
    return d.field[done & 1];
}

template <typename T>
void Batch2d<T>::check_errors() {
    int h = 0;
    SSSI_CHECK_CUDA(cudaMemcpyAsync(&h, bc_.err, sizeof(int), cudaMemcpyDeviceToHost, stream_));
    SSSI_CHECK_CUDA(cudaStreamSynchronize(stream_));
    if (h != 0) SSSI_CHECK_CUDA(cudaMemsetAsync(bc_.err, 0, sizeof(int), stream_));  // the batch stays usable
    SSSI_REQUIRE(h == 0, SSSI_ERR_INTERNAL,
                 "a tile copy did not arrive within the wait limit: the step was aborted and the fields of its "
                 "shots are incomplete");
}

template <typename T>
void Batch2d<T>::ensure_status() {
    // one status word per slot; the descriptors point at theirs
    const size_t need = sizeof(int) * std::max<size_t>(shots_.size(), 1);
    if (d_status_.bytes() < need) {
        DeviceBuffer fresh(need * 2);
        fresh.zero(stream_);
        if (d_status_.bytes())
            SSSI_CHECK_CUDA(cudaMemcpyAsync(fresh.get(), d_status_.get(), d_status_.bytes(), cudaMemcpyDeviceToDevice,
                                            stream_));
        d_status_ = std::move(fresh);
    }
    for (int k = 0; k < (int)shots_.size(); ++k) shots_[k].desc.s.status = d_status_.template as<int>() + k;
}

template <typename T>
std::vector<int> Batch2d<T>::statuses() {
    // slots added since the last schedule have not stepped yet: they read as SSSI_OK
    std::vector<int> h(shots_.size(), 0);
    const size_t n = std::min(h.size(), d_status_.bytes() / sizeof(int));
    if (n) {
        SSSI_CHECK_CUDA(cudaMemcpyAsync(h.data(), d_status_.get(), sizeof(int) * n, cudaMemcpyDeviceToHost, stream_));
        SSSI_CHECK_CUDA(cudaStreamSynchronize(stream_));
    }
    return h;
}

template <typename T>
void Batch2d<T>::clear_status(int k) {
    if (d_status_.bytes() >= sizeof(int) * (size_t)(k + 1))
        SSSI_CHECK_CUDA(cudaMemsetAsync(d_status_.template as<int>() + k, 0, sizeof(int), stream_));
}

template <typename T>
void Batch2d<T>::set_debug(int step, unsigned wait_limit) {
    bc_.debug_step = step;
    bc_.wait_limit = step >= 0 && wait_limit ? wait_limit : kDefaultWaitLimit;
}

template <typename T>
void launch_batch2d(int N, const ShotDesc<T>* shots, const BatchConst<T>& bc, int grid, bool split, int shape,
                    bool pair, bool lean, cudaStream_t stream) {
    switch (N) {
        case 1: launch_batch2d_n<T, 1>(shots, bc, grid, split, shape, pair, lean, stream); break;
        case 2: launch_batch2d_n<T, 2>(shots, bc, grid, split, shape, pair, lean, stream); break;
        case 3: launch_batch2d_n<T, 3>(shots, bc, grid, split, shape, pair, lean, stream); break;
        case 4: launch_batch2d_n<T, 4>(shots, bc, grid, split, shape, pair, lean, stream); break;
        case 5: launch_batch2d_n<T, 5>(shots, bc, grid, split, shape, pair, lean, stream); break;
        case 6: launch_batch2d_n<T, 6>(shots, bc, grid, split, shape, pair, lean, stream); break;
        case 7: launch_batch2d_n<T, 7>(shots, bc, grid, split, shape, pair, lean, stream); break;
        case 8: launch_batch2d_n<T, 8>(shots, bc, grid, split, shape, pair, lean, stream); break;
        default: SSSI_REQUIRE(false, SSSI_ERR_ARG, "nDiffOrder %d out of range 1..8", N);
    }
}

template <typename T>
int batch2d_ctas_per_sm(int N, int shape, bool pair) {
    switch (N) {
        case 1: return batch2d_occupancy_n<T, 1>(shape, pair);
        case 2: return batch2d_occupancy_n<T, 2>(shape, pair);
        case 3: return batch2d_occupancy_n<T, 3>(shape, pair);
        case 4: return batch2d_occupancy_n<T, 4>(shape, pair);
        case 5: return batch2d_occupancy_n<T, 5>(shape, pair);
        case 6: return batch2d_occupancy_n<T, 6>(shape, pair);
        case 7: return batch2d_occupancy_n<T, 7>(shape, pair);
        default: return batch2d_occupancy_n<T, 8>(shape, pair);
    }
}

template class Batch2d<float>;
template class Batch2d<double>;

}  // namespace sssi
