// Host side of the 3D CPML propagation: grids, damping, descriptors, launches.
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <mutex>

#include "prop3d.cuh"

namespace sssi {

bool encode_tensor_map_3d(CUtensorMap* map, const void* base, CUtensorMapDataType dtype, size_t elem_bytes,
                          uint64_t d0, uint64_t d1, uint64_t d2, uint64_t ld0, uint64_t ld1, uint32_t b0, uint32_t b1,
                          uint32_t b2) {
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
    const cuuint64_t dims[3] = {d0, d1, d2};
    const cuuint64_t strides[2] = {ld0 * elem_bytes, ld1 * elem_bytes};
    const cuuint32_t box[3] = {b0, b1, b2};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = encode(map, dtype, 3, const_cast<void*>(base), dims, strides, box, estr,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

namespace {

template <typename T>
constexpr CUtensorMapDataType tma_type() {
    return std::is_same<T, float>::value ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
}

// (v dt)^2 into the padded layout (interior origin `org`, strides ldz, ldxy).
template <typename T>
__global__ void vdt2_kernel(const double* v, int64_t nz, int64_t nx, int64_t ny, double dt, T* out, int64_t ldz,
                            int64_t ldxy) {
    const int64_t n = nz * nx * ny;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = q % nz, j = (q / nz) % nx, k = q / (nz * nx);
        const double a = v[q] * dt;
        out[i + j * ldz + k * ldxy] = static_cast<T>(a * a);
    }
}

template <typename T>
void launch_prop3d(int N, const Desc3<T>* d, const Const3<T>& c, int grid, cudaStream_t s) {
    switch (N) {
        case 1: launch_prop3d_n<T, 1>(d, c, grid, s); break;
        case 2: launch_prop3d_n<T, 2>(d, c, grid, s); break;
        case 3: launch_prop3d_n<T, 3>(d, c, grid, s); break;
        case 4: launch_prop3d_n<T, 4>(d, c, grid, s); break;
        case 5: launch_prop3d_n<T, 5>(d, c, grid, s); break;
        case 6: launch_prop3d_n<T, 6>(d, c, grid, s); break;
        case 7: launch_prop3d_n<T, 7>(d, c, grid, s); break;
        case 8: launch_prop3d_n<T, 8>(d, c, grid, s); break;
        default: SSSI_REQUIRE(false, SSSI_ERR_ARG, "nDiffOrder %d out of range 1..8", N);
    }
}

template <typename T>
int prop3d_occupancy(int N) {
    switch (N) {
        case 1: return prop3d_occupancy_n<T, 1>();
        case 2: return prop3d_occupancy_n<T, 2>();
        case 3: return prop3d_occupancy_n<T, 3>();
        case 4: return prop3d_occupancy_n<T, 4>();
        case 5: return prop3d_occupancy_n<T, 5>();
        case 6: return prop3d_occupancy_n<T, 6>();
        case 7: return prop3d_occupancy_n<T, 7>();
        default: return prop3d_occupancy_n<T, 8>();
    }
}

}  // namespace

template <typename T>
void launch_vdt2(const double* v, int64_t nz, int64_t nx, int64_t ny, double dt, T* out, int64_t ldz, int64_t ldxy,
                 cudaStream_t s) {
    if (nz * nx * ny == 0) return;
    vdt2_kernel<T><<<152 * 4, 256, 0, s>>>(v, nz, nx, ny, dt, out, ldz, ldxy);
    count_launch();
    SSSI_CHECK_CUDA(cudaGetLastError());
}
template void launch_vdt2<float>(const double*, int64_t, int64_t, int64_t, double, float*, int64_t, int64_t,
                                 cudaStream_t);
template void launch_vdt2<double>(const double*, int64_t, int64_t, int64_t, double, double*, int64_t, int64_t,
                                  cudaStream_t);

template <typename T>
Prop3d<T>::Prop3d(const double* v, int64_t nz, int64_t nx, int64_t ny, int N, int nB, double dz, double dx,
                  double dy, double dt, int nt, cudaStream_t stream)
    : N_(N), stream_(stream) {
    using S = Shape3D<T>;
    SSSI_REQUIRE(N >= 1 && N <= kMaxOrder, SSSI_ERR_ARG, "nDiffOrder must be in 1..%d (got %d)", kMaxOrder, N);
    SSSI_REQUIRE(nz > 0 && nx > 0 && ny > 0, SSSI_ERR_ARG, "bad 3D sizes");
    SSSI_REQUIRE(nB >= 0 && 2 * (int64_t)nB <= std::min(nx, ny) && nB <= nz, SSSI_ERR_ARG,
                 "nBoundary %d does not fit the grid", nB);
    SSSI_REQUIRE(dz > 0 && dx > 0 && dy > 0 && dt > 0, SSSI_ERR_ARG, "dz, dx, dy, dt must be positive");
    SSSI_REQUIRE(nz * nx * ny < (int64_t(1) << 40), SSSI_ERR_ARG, "grid too large");
    const int L = 2 * N - 1, HZ = tile_halo_rows(N);
    const int64_t Nzp = (nz + 2 * HZ + 3) / 4 * 4, Nxp = nx + 2 * L, Nyp = ny + 2 * L;
    const int64_t np = Nzp * Nxp * Nyp, org = HZ + L * Nzp + L * Nzp * Nxp;
    SSSI_REQUIRE(np < (int64_t(1) << 40), SSSI_ERR_ARG, "grid too large");

    // coefficients
    double c[kMaxOrder], wz[kMaxOrder], wx[kMaxOrder], az[16], ax[16];
    staggered_coefficients(N, c);
    for (int k = 0; k < N; ++k) {
        wz[k] = c[k] / dz;
        wx[k] = c[k] / dx;
    }
    composed_coefficients(wz, N, az);
    composed_coefficients(wx, N, ax);
    for (int k = 0; k < 8; ++k) {
        cc_.wz[k] = k < N ? static_cast<T>(wz[k]) : T(0);
        cc_.wx[k] = k < N ? static_cast<T>(wx[k]) : T(0);
        cc_.wy[k] = k < N ? static_cast<T>(c[k] / dy) : T(0);
    }
    for (int m = 0; m < 16; ++m) {
        cc_.az[m] = m <= L ? static_cast<T>(az[m]) : T(0);
        cc_.ax[m] = m <= L ? static_cast<T>(ax[m]) : T(0);
    }
    // at queue position u the slot of A_y(y + k) is (u + N + 1 + k) mod 2N (weight
    // w_k), the slot of A_y(y - 1 - k) is (u + N - k) mod 2N (weight -w_k)
    for (int u = 0; u < 16; ++u)
        for (int q = 0; q < 16; ++q) cc_.wyq[u * 16 + q] = T(0);
    for (int u = 0; u < 2 * N; ++u)
        for (int k = 0; k < N; ++k) {
            cc_.wyq[u * 16 + (u + N + 1 + k) % (2 * N)] = cc_.wy[k];
            cc_.wyq[u * 16 + (u + N - k) % (2 * N)] = -cc_.wy[k];
        }
    auto pair = [](T c) { return make_float2(static_cast<float>(c), static_cast<float>(c)); };
    for (int m = 0; m < 16; ++m) {
        cc_.az2[m] = pair(cc_.az[m]);
        cc_.ax2[m] = pair(cc_.ax[m]);
    }
    for (int k = 0; k < 8; ++k) cc_.wy2[k] = pair(cc_.wy[k]);
    for (int q = 0; q < 16 * 16; ++q) cc_.wyq2[q] = pair(cc_.wyq[q]);

    // fields and (v dt)^2 in the padded layout (the padding stays zero)
    for (auto& b : P_) {
        b.allocate(sizeof(T) * np);
        b.zero(stream_);
    }
    vdt2_.allocate(sizeof(T) * np);
    vdt2_.zero(stream_);
    const int64_t n = nz * nx * ny;
    {
        DeviceBuffer vd;
        const double* vdev = v;
        if (!is_device_pointer(v)) {
            vd.allocate(sizeof(double) * n);
            SSSI_CHECK_CUDA(cudaMemcpyAsync(vd.get(), v, sizeof(double) * n, cudaMemcpyHostToDevice, stream_));
            vdev = vd.template as<double>();
        }
        launch_vdt2<T>(vdev, nz, nx, ny, dt, vdt2_.template as<T>() + org, Nzp, Nzp * Nxp, stream_);
        SSSI_CHECK_CUDA(cudaStreamSynchronize(stream_));  // vd is released at the end of this scope
    }

    // damping: the profiles read v on the y = 0 slice and the top row only
    std::vector<double> vslice((size_t)(nz * nx)), vtop((size_t)(nx * ny));
    if (is_device_pointer(v)) {
        SSSI_CHECK_CUDA(cudaMemcpyAsync(vslice.data(), v, sizeof(double) * nz * nx, cudaMemcpyDeviceToHost, stream_));
        SSSI_CHECK_CUDA(cudaMemcpy2DAsync(vtop.data(), sizeof(double), v, sizeof(double) * nz, sizeof(double),
                                          (size_t)(nx * ny), cudaMemcpyDeviceToHost, stream_));
        SSSI_CHECK_CUDA(cudaStreamSynchronize(stream_));
    } else {
        std::copy(v, v + nz * nx, vslice.begin());
        for (int64_t q = 0; q < nx * ny; ++q) vtop[q] = v[q * nz];
    }
    const Bands3D bands = damping_bands_3d(vslice.data(), vtop.data(), nz, nx, ny, nB, dt);
    auto upload = [&](DeviceBuffer& buf, const std::vector<T>& h) {
        buf.allocate(sizeof(T) * std::max<size_t>(h.size(), 1));
        if (!h.empty())
            SSSI_CHECK_CUDA(cudaMemcpyAsync(buf.get(), h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, stream_));
    };
    std::vector<T> b, bm1;
    band_coefficients<T>(bands.zb, bands.zbm1, b, bm1);
    upload(zb_, b);
    upload(zbm1_, bm1);
    band_coefficients<T>(bands.xb, bands.xbm1, b, bm1);
    upload(xb_, b);
    upload(xbm1_, bm1);
    band_coefficients<T>(bands.yb, bands.ybm1, b, bm1);
    upload(yb_, b);
    upload(ybm1_, bm1);
    SSSI_CHECK_CUDA(cudaStreamSynchronize(stream_));  // host staging vectors go out of scope
    auto mem = [&](DeviceBuffer& buf, int64_t count) {
        buf.allocate(sizeof(M) * std::max<int64_t>(count, 1));
        buf.zero(stream_);
    };
    const int64_t mz = (int64_t)nB * nx * ny, mx = nz * 2 * (int64_t)nB * ny, my = nz * nx * 2 * (int64_t)nB;
    mem(zphi_[0], mz);
    mem(zphi_[1], mz);
    mem(zpsi_, mz);
    mem(xphi_[0], mx);
    mem(xphi_[1], mx);
    mem(xpsi_, mx);
    mem(yphi_[0], my);
    mem(yphi_[1], my);
    mem(ypsi_, my);

    // descriptor
    Desc3<T>& d = desc_;
    const uint32_t box_rows = S::TZ + 2 * HZ, box_cols = S::TX + 2 * L;
    for (int k = 0; k < 2; ++k) {
        SSSI_REQUIRE(encode_tensor_map_3d(&d.tm_plane[k], P_[k].get(), tma_type<T>(), sizeof(T), Nzp, Nxp, Nyp, Nzp,
                                          Nzp * Nxp, box_rows, box_cols, 1),
                     SSSI_ERR_CUDA, "cuTensorMapEncodeTiled failed for the 3D field");
        SSSI_REQUIRE(encode_tensor_map_3d(&d.tm_tile[k], P_[k].get(), tma_type<T>(), sizeof(T), Nzp, Nxp, Nyp, Nzp,
                                          Nzp * Nxp, S::TZ, S::TX, 1),
                     SSSI_ERR_CUDA, "cuTensorMapEncodeTiled failed for the 3D field");
        d.field[k] = P_[k].template as<T>() + org;
    }
    SSSI_REQUIRE(encode_tensor_map_3d(&d.tm_v, vdt2_.get(), tma_type<T>(), sizeof(T), Nzp, Nxp, Nyp, Nzp, Nzp * Nxp,
                                      S::TZ, S::TX, 1),
                 SSSI_ERR_CUDA, "cuTensorMapEncodeTiled failed for (v dt)^2");
    d.vdt2 = vdt2_.template as<T>() + org;
    d.ldz = Nzp;
    d.ldxy = Nzp * Nxp;
    d.nz = (int)nz;
    d.nx = (int)nx;
    d.ny = (int)ny;
    d.nB = nB;
    d.nt = nt;
    // Tile rows start at row -zs (whole 32-byte sectors of rows): the rows whose z
    // second derivative reaches the bottom band (nz - nB - N + 1 on) then fall in
    // one tile row instead of two, when that does not add a tile row.  Rows above
    // the grid are not computed.
    d.zs = 0;
    {
        const int64_t cut = nz - nB - N + 1;
        if (nB > 0 && cut >= 0) {
            constexpr int kSector = 32 / (int)sizeof(T);
            const int zs = (int)((S::TZ - (cut / kSector * kSector) % S::TZ) % S::TZ);
            auto band_rows = [&](int s0) {
                int n = 0;
                for (int64_t z0 = -s0; z0 < nz; z0 += S::TZ) n += z0 + S::TZ + N - 1 > nz - nB;
                return n;
            };
            if (zs > 0 && (nz + zs + S::TZ - 1) / S::TZ == (nz + S::TZ - 1) / S::TZ && band_rows(zs) < band_rows(0))
                d.zs = zs;
        }
    }
    d.ntz = (int)((nz + d.zs + S::TZ - 1) / S::TZ);
    d.ntx = (int)((nx + S::TX - 1) / S::TX);
    int dev = 0, sms = 1;
    SSSI_CHECK_CUDA(cudaGetDevice(&dev));
    SSSI_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int slots = sms * prop3d_occupancy<T>(N);
    d.zb = zb_.template as<T>();
    d.zbm1 = zbm1_.template as<T>();
    d.xb = xb_.template as<T>();
    d.xbm1 = xbm1_.template as<T>();
    d.yb = yb_.template as<T>();
    d.ybm1 = ybm1_.template as<T>();
    for (int k = 0; k < 2; ++k) {
        d.zphi[k] = zphi_[k].template as<M>();
        d.xphi[k] = xphi_[k].template as<M>();
        d.yphi[k] = yphi_[k].template as<M>();
    }
    d.zpsi = zpsi_.template as<M>();
    d.xpsi = xpsi_.template as<M>();
    d.ypsi = ypsi_.template as<M>();
    d_desc_.allocate(sizeof(Desc3<T>));

    d_ctr_.allocate(4 * sizeof(int));  // graph step base, zero, error flag, spare
    d_ctr_.zero(stream_);
    cc_.step_base = d_ctr_.template as<int>() + 1;
    cc_.step_offset = 0;
    cc_.err = d_ctr_.template as<int>() + 2;
    // Candidate schedules of work items, each item a (z, x) tile and a chunk of
    // planes; the dynamic schedule takes the most expensive first.  Cost model
    // (plane times measured on 256^3-288^3 grids): a plane costs 1, 2.6 in a
    // tile next to a z or an x band (cooperative pass per plane), 4 next to
    // both, +0.5 in a y band (memory-variable traffic); every chunk also fills
    // its queues from 2N-1 planes (0.4 each).
    //   0:       even chunks along y, about three items per resident block,
    //            8 to 64 planes;
    //   1, 2, 3: each tile's planes cut into chunks of about equal estimated
    //            cost (tiles next to a band get shorter chunks, each tile ends
    //            with a shorter one), about three, two or four items per
    //            resident block, 4 to 64 planes.
    // Fewer, longer chunks fill the queues less often; more chunks, and short
    // ones last, balance the blocks better.
    {
        SSSI_REQUIRE(ny < 65536, SSSI_ERR_ARG, "ny must be below 65536");
        const int ntile = d.ntz * d.ntx;
        auto plane_cost = [&](int band_zx, int y) {
            static const float kTile[3] = {1.0f, 2.6f, 4.0f};
            return kTile[band_zx] + ((nB > 0 && (y < nB || y >= ny - nB)) ? 0.5f : 0.0f);
        };
        std::vector<char> bzx(ntile);  // 0: no z / x band work, 1: z or x, 2: both
        double total = 0;
        for (int t = 0; t < ntile; ++t) {
            const int z0 = (t % d.ntz) * S::TZ - d.zs, x0 = (t / d.ntz) * S::TX;
            const bool bz = nB > 0 && z0 + S::TZ + N - 1 > nz - nB;
            const bool bx = nB > 0 && (x0 - N < nB || x0 + S::TX + N - 2 >= nx - nB);
            bzx[t] = (char)(bz + bx);
            for (int y = 0; y < ny; ++y) total += plane_cost(bzx[t], y);
        }
        const float warm = 0.4f * (2 * N - 1);
        struct It {
            int2 item;
            float cost;
        };
        for (int c = 0; c < kSchedules3; ++c) {
            std::vector<It> its;
            static const int kPer[kSchedules3] = {3, 3, 2, 4};  // items per resident block
            const int64_t per = kPer[c];
            auto chunk = [&](int t, int y0, int y1) {
                float cost = warm;
                for (int y = y0; y < y1; ++y) cost += plane_cost(bzx[t], y);
                its.push_back({make_int2(t, y0 | (y1 << 16)), cost});
            };
            if (c == 0) {
                int64_t yc = std::max<int64_t>(8, (ny * ntile + per * slots - 1) / (per * (int64_t)slots));
                yc = std::min<int64_t>(yc, 64);
                const int64_t nch = (ny + yc - 1) / yc;
                const int ychunk = (int)((ny + nch - 1) / nch);  // even chunks
                for (int t = 0; t < ntile; ++t)
                    for (int y0 = 0; y0 < ny; y0 += ychunk) chunk(t, y0, (int)std::min<int64_t>(y0 + ychunk, ny));
            } else {
                const float target = std::max(4.0f, (float)(total / ((double)per * slots)));
                for (int t = 0; t < ntile; ++t) {
                    int y0 = 0;
                    while (y0 < ny) {
                        float cost = 0;
                        int y1 = y0;
                        while (y1 < ny && (y1 - y0 < 4 || (cost < target && y1 - y0 < 64)))
                            cost += plane_cost(bzx[t], y1++);
                        if (ny - y1 < 4) y1 = (int)ny;  // no short tail chunk
                        chunk(t, y0, y1);
                        y0 = y1;
                    }
                }
            }
            // most expensive first; among equal costs by first plane, then tile, so that
            // blocks running at the same time work on nearby planes (L2 reuse of halos)
            std::sort(its.begin(), its.end(), [](const It& a, const It& b) {
                if (a.cost != b.cost) return a.cost > b.cost;
                const int ya = a.item.y & 0xffff, yb = b.item.y & 0xffff;
                return ya != yb ? ya < yb : a.item.x < b.item.x;
            });
            std::vector<int2> order(its.size());
            for (size_t q = 0; q < its.size(); ++q) order[q] = its[q].item;
            d_order_[c].allocate(sizeof(int2) * std::max<size_t>(order.size(), 1));
            SSSI_CHECK_CUDA(cudaMemcpyAsync(d_order_[c].get(), order.data(), sizeof(int2) * order.size(),
                                            cudaMemcpyHostToDevice, stream_));
            SSSI_CHECK_CUDA(cudaStreamSynchronize(stream_));
            d.order[c] = d_order_[c].template as<int2>();
            nitems_[c] = (int)its.size();
            grid_c_[c] = std::max(1, std::min(nitems_[c], slots));
        }
        d_next_.allocate(2 * sizeof(int));
        d_next_.zero(stream_);
        d.next = d_next_.template as<int>();
        use_schedule(0);
        if (nt < kTuneMinSteps) tune_ = kTuneDone;  // short runs keep schedule 0
        for (auto& e : tev_) SSSI_CHECK_CUDA(cudaEventCreate(&e));
    }
    sync_desc();
}

template <typename T>
Prop3d<T>::~Prop3d() {
    if (graph_) cudaGraphExecDestroy(graph_);
    for (auto& e : tev_)
        if (e) cudaEventDestroy(e);
}

template <typename T>
void Prop3d<T>::use_schedule(int c) {
    if (cc_.sched == c && grid_ == grid_c_[c] && cc_.nitems == nitems_[c]) return;
    cc_.sched = c;
    cc_.nitems = nitems_[c];
    grid_ = grid_c_[c];
    if (graph_) cudaGraphExecDestroy(graph_);  // launch parameters change
    graph_ = nullptr;
}

template <typename T>
void Prop3d<T>::set_point_sources(int nsrc, const int64_t* iz, const int64_t* ix, const int64_t* iy,
                                  const T* d_wavelet) {
    SSSI_REQUIRE(nsrc >= 0 && nsrc <= kMaxPointSources, SSSI_ERR_ARG, "at most %d point sources (got %d)",
                 kMaxPointSources, nsrc);
    for (int s = 0; s < nsrc; ++s)
        SSSI_REQUIRE(iz[s] >= 0 && iz[s] < desc_.nz && ix[s] >= 0 && ix[s] < desc_.nx && iy[s] >= 0 &&
                         iy[s] < desc_.ny,
                     SSSI_ERR_ARG, "point source %d outside the grid", s);
    desc_.nsrc = nsrc;
    for (int s = 0; s < nsrc; ++s) {
        desc_.src_iz[s] = (int)iz[s];
        desc_.src_ix[s] = (int)ix[s];
        desc_.src_iy[s] = (int)iy[s];
    }
    desc_.src_wavelet = d_wavelet;
}

template <typename T>
void Prop3d<T>::sync_desc() {
    SSSI_CHECK_CUDA(cudaMemcpyAsync(d_desc_.get(), &desc_, sizeof(Desc3<T>), cudaMemcpyHostToDevice, stream_));
    SSSI_CHECK_CUDA(cudaStreamSynchronize(stream_));  // desc_ may change on the host next
}

template <typename T>
void Prop3d<T>::launch_step(const int* base, int offset, cudaStream_t s) {
    Const3<T> c = cc_;
    c.step_base = base;
    c.step_offset = offset;
    launch_prop3d<T>(N_, d_desc_.template as<Desc3<T>>(), c, grid_, s);
}

template <typename T>
void Prop3d<T>::run(int nsteps) {
    int q = 0;
    // schedule tuning (single launches, events around the timed runs)
    while (q < nsteps && tune_ < kTuneWait) {
        if (tune_left_ == (tune_ == 0 ? 2 : kTuneSteps)) {
            // a timed run must lie within this call: the caller may queue other
            // work on the stream between calls
            if (tune_ > 0 && nsteps - q < kTuneSteps) break;
            use_schedule(tune_ > 0 ? tune_ - 1 : 0);
            if (tune_ > 0) SSSI_CHECK_CUDA(cudaEventRecord(tev_[2 * (tune_ - 1)], stream_));  // start
        }
        const int k = std::min(nsteps - q, tune_left_);
        for (int i = 0; i < k; ++i) launch_step(cc_.step_base, step_ + q + i, stream_);
        q += k;
        tune_left_ -= k;
        if (tune_left_ == 0) {
            if (tune_ > 0) SSSI_CHECK_CUDA(cudaEventRecord(tev_[2 * (tune_ - 1) + 1], stream_));  // end
            ++tune_;
            tune_left_ = kTuneSteps;
        }
    }
    if (tune_ == kTuneWait) {
        // steps left in this call: wait for the timings (once per propagation),
        // else look without waiting and decide at a later call
        cudaEvent_t last = tev_[2 * kSchedules3 - 1];
        const cudaError_t e = q < nsteps ? cudaEventSynchronize(last) : cudaEventQuery(last);
        if (e == cudaSuccess) {
            int best = 0;
            for (int c = 0; c < kSchedules3; ++c) {
                SSSI_CHECK_CUDA(cudaEventElapsedTime(&tune_ms_[c], tev_[2 * c], tev_[2 * c + 1]));
                if (tune_ms_[c] < tune_ms_[best]) best = c;
            }
            use_schedule(best);
            record_schedule3d(best, tune_ms_, kSchedules3);
            tune_ = kTuneDone;
        } else if (e != cudaErrorNotReady) {
            SSSI_CHECK_CUDA(e);
        } else {
            cudaGetLastError();
        }
    }
    nsteps -= q;
    step_ += q;
    q = 0;
    if (nsteps >= kGraphSteps) {
        int* base = d_ctr_.template as<int>();
        if (!graph_) {
            std::lock_guard<std::mutex> lock(capture_mutex());
            cudaStream_t cs = capture_stream();
            cudaGraph_t g = nullptr;
            SSSI_CHECK_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
            try {
                for (int k = 0; k < kGraphSteps; ++k) launch_step(base, k, cs);
                launch_add_int(base, kGraphSteps, cs);
            } catch (...) {
                cudaStreamEndCapture(cs, &g);
                if (g) cudaGraphDestroy(g);
                throw;
            }
            count_launch(-kGraphSteps);  // recorded, not run
            cudaError_t e = cudaStreamEndCapture(cs, &g);
            if (e == cudaSuccess) e = cudaGraphInstantiate(&graph_, g, 0);
            if (g) cudaGraphDestroy(g);
            if (e != cudaSuccess) graph_ = nullptr;
            SSSI_CHECK_CUDA(e);
        }
        launch_store_int(base, step_, stream_);
        count_launch();
        for (; q + kGraphSteps <= nsteps; q += kGraphSteps) {
            SSSI_CHECK_CUDA(cudaGraphLaunch(graph_, stream_));
            count_launch(kGraphSteps + 1);
        }
    }
    for (; q < nsteps; ++q) launch_step(cc_.step_base, step_ + q, stream_);
    step_ += nsteps;
}

template <typename T>
void Prop3d<T>::check_errors() {
    int h = 0;
    SSSI_CHECK_CUDA(cudaMemcpyAsync(&h, cc_.err, sizeof(int), cudaMemcpyDeviceToHost, stream_));
    SSSI_CHECK_CUDA(cudaStreamSynchronize(stream_));
    SSSI_REQUIRE(h == 0, SSSI_ERR_INTERNAL, "a plane copy did not arrive within the wait limit (kernel aborted)");
}

template class Prop3d<float>;
template class Prop3d<double>;

}  // namespace sssi
