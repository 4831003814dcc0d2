// 2D acoustic propagation with the sponge absorbing boundary: forward
// modelling, reverse propagation and the RTM shot of
//   src/fwdTimeSpongeFor2dAw.m:36-101, src/rvsTimeSpongeFor2dAw.m:36-103,
//   applications/rtm_2d_acoustic/mainRtmTimeSpongeFor2dAw.m:160-161,247-268,310.
//
// The reference (MATLAB) advances a zero-bordered field with the second-order
// five-point update
//     fdm3 = b .* fdm2 - fdm1 + ax .* (right + left) + az .* (down + up) - vdtSq .* source
// (b = 2 - 2ax - 2az, ax = (v dt/dx)^2, az = (v dt/dz)^2, vdtSq = (v dt)^2),
// rotates (fdm1 <- fdm2, fdm2 <- fdm3) and then multiplies BOTH the new past
// and the new present by the sponge factors of the left / right columns
// (rows above the bottom band) and of the bottom rows (every column):
//     boundary(k) = exp(-(alpha (nB - k + 1))^2)^10,  alpha = 0.015.
// The past of the next step is therefore s .* (present of this step), which
// this kernel forms at the cell itself when it reads its previous value: one
// pair of field buffers, each step reading the present and overwriting the
// previous present of its own cell with s .* fdm3.  No cell is read by a
// neighbour after it is overwritten (neighbours read only the present).
//
// GB300 layout and launch: each field is (ldp rows) x (nx + 2 columns) with a
// zero border (row -1 and row nz, columns -1 and nx), every column's interior
// starting on a 32-element boundary; the coefficient arrays share the layout.
// A block of 8 warps takes a tile of 32 rows x 8 columns (one warp per
// column, coalesced along z) so that the x neighbours of the inner columns
// come from L1; tiles run z-fastest over a persistent grid.  One step
// is one launch; runs of kSpGraphSteps steps replay a CUDA graph that reads the
// step number and the chunked hooks (sources, snapshots) from device memory.
//
// Arithmetic: SSSI_MODE_FP64_STRICT rounds every operation as the MATLAB
// expression is written (left to right, no fused multiply-add); SSSI_MODE_FP64
// fuses b*present - past, ax*(.) and az*(.) into multiply-adds; SSSI_MODE_FP32
// keeps the field in FP32 and derives ax, az, b from (v dt)^2 in the kernel
// (16 bytes of HBM traffic per cell and step).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "api_util.cuh"
#include "sssi_internal.h"

namespace sssi {
namespace {

using namespace api;

constexpr int kSpRows = 32, kSpCols = 8;  // a tile: one warp per column
constexpr int kSpThreads = kSpRows * kSpCols;
constexpr int kSpOrgRow = 32;             // interior row 0 within a column (row -1 is zero padding)
constexpr int kSpGraphSteps = 32;
constexpr double kSpongeAlpha = 0.015;    // src/fwdTimeSpongeFor2dAw.m:45

// Per-chunk hooks, read from device memory by every launch (a captured graph
// keeps its launch parameters; these change between chunks).
template <typename T>
struct SpongeHooks {
    const T* src_dense;  // nz x nx slices (pitch nz), slice of step t at src_dense + (t - dense_t0) * nz * nx
    T* snap;             // the same layout for snapshots
    const T* fsnap;      // forward snapshots for imaging (t - fsnap_t0)
    int dense_t0, snap_t0, fsnap_t0, pad;
};

template <typename T>
struct SpongeParams {
    T* field[2];                // ping-pong fields (interior origin applied)
    const T* cb;                // FP64 modes: b, ax, az, (v dt)^2 (interior origin applied)
    const T* cax;
    const T* caz;
    const T* cvdt2;             // all modes: (v dt)^2
    const T* bnd;               // sponge factors, nB entries
    const SpongeHooks<T>* hooks;
    const int* step_base;       // device step counter (graph replays); the step is *step_base + step_offset
    int step_offset;
    int nz, nx, nB, nt;
    int64_t ldp;
    int ntz, ntiles;
    int reverse;                // time runs nt-1 .. 0 and row 0 takes src_row
    T kx, kz;                   // FP32: 1/dx^2, 1/dz^2 (ax = vdt2 kx, az = vdt2 kz)
    // point sources (forward): cell (src_iz[k], src_ix[k]) adds wavelets[k * nt + t]
    int nsrc;
    const int* src_iz;
    const int* src_ix;
    const T* wavelets;
    const T* src_row;           // reverse: data, nx x nt (row 0 source of step t at src_row + t * nx)
    T* rec;                     // data, nx x nt: row 0 of the new present
    double* im;                 // imaging sums (FP64 fused RTM): M and S2, nz x nx (pitch nz)
    double* is2;
};

// The sponge factors of cell (i, j) applied to x in the order of the
// reference's loop (src/fwdTimeSpongeFor2dAw.m:80-90): for ixb = 2..nB+1 the
// left column ixb, the right column nx-nB+ixb, the bottom row nz-nB+ixb.  A
// cell is hit by the bottom rows alone or by the side columns of its row;
// both side columns hit it only when nx < 2 nB (the right one first unless
// nx == nB).
template <typename T, int kMode>
__device__ __forceinline__ T sponge(T x, int i, int j, const SpongeParams<T>& p) {
    const int nB = p.nB;
    if (i >= p.nz - nB) return kMode == SSSI_MODE_FP32 ? x * p.bnd[p.nz - 1 - i] : __dmul_rn(p.bnd[p.nz - 1 - i], x);
    const bool left = j < nB, right = j >= p.nx - nB;
    if (!(left | right)) return x;
    auto mul = [](T a, T b) -> T {
        if constexpr (kMode == SSSI_MODE_FP32)
            return a * b;
        else
            return __dmul_rn(a, b);
    };
    if (left && right) {
        const T bl = p.bnd[j], br = p.bnd[p.nx - 1 - j];
        return p.nx > nB ? mul(bl, mul(br, x)) : mul(br, mul(bl, x));
    }
    return mul(p.bnd[left ? j : p.nx - 1 - j], x);
}

template <typename T, int kMode>
__global__ void __launch_bounds__(kSpThreads) sponge2d_step_kernel(const __grid_constant__ SpongeParams<T> p) {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const int step = *reinterpret_cast<volatile const int*>(p.step_base) + p.step_offset;
    const int t = p.reverse ? p.nt - 1 - step : step;
    const T* __restrict__ cur = p.field[step & 1];
    T* __restrict__ nxt = p.field[(step & 1) ^ 1];
    const SpongeHooks<T> h = *p.hooks;
    const int64_t n = (int64_t)p.nz * p.nx;
    const T* src_dense = h.src_dense ? h.src_dense + (int64_t)(t - h.dense_t0) * n : nullptr;
    T* snap = h.snap ? h.snap + (int64_t)(t - h.snap_t0) * n : nullptr;
    const T* fsnap = h.fsnap ? h.fsnap + (int64_t)(t - h.fsnap_t0) * n : nullptr;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t ldp = p.ldp;
    for (int tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x) {
        const int tz = tile % p.ntz, tx = tile / p.ntz;
        const int i = tz * kSpRows + lane, j = tx * kSpCols + w;
        if (i >= p.nz || j >= p.nx) continue;
        const int64_t q = i + (int64_t)j * ldp;
        const T c = __ldg(cur + q), up = __ldg(cur + q - 1), dn = __ldg(cur + q + 1);
        const T lf = __ldg(cur + q - ldp), rt = __ldg(cur + q + ldp);
        const T past = sponge<T, kMode>(nxt[q], i, j, p);
        const T vdt2 = __ldg(p.cvdt2 + q);
        // the injected value of the cell at step t (dense slice, point sources, or row 0)
        T src = T(0);
        bool has_src = false;
        if (src_dense) {
            src = src_dense[i + (int64_t)j * p.nz];
            has_src = true;
        }
        if (p.src_row && i == 0) {
            src = p.src_row[j + (int64_t)t * p.nx];
            has_src = true;
        }
        for (int k = 0; k < p.nsrc; ++k)
            if (p.src_iz[k] == i && p.src_ix[k] == j) {
                src = has_src ? src + p.wavelets[(int64_t)k * p.nt + t] : p.wavelets[(int64_t)k * p.nt + t];
                has_src = true;
            }
        T r;
        if constexpr (kMode == SSSI_MODE_FP64_STRICT) {
            r = __dsub_rn(__dmul_rn(__ldg(p.cb + q), c), past);
            r = __dadd_rn(r, __dmul_rn(__ldg(p.cax + q), __dadd_rn(rt, lf)));
            r = __dadd_rn(r, __dmul_rn(__ldg(p.caz + q), __dadd_rn(dn, up)));
            if (has_src) r = __dsub_rn(r, __dmul_rn(vdt2, src));
        } else if constexpr (kMode == SSSI_MODE_FP64) {
            r = fma(__ldg(p.cb + q), c, -past);
            r = fma(__ldg(p.cax + q), rt + lf, r);
            r = fma(__ldg(p.caz + q), dn + up, r);
            if (has_src) r = fma(-vdt2, src, r);
        } else {
            const T ax = vdt2 * p.kx, az = vdt2 * p.kz;
            const T b = (T(2) - T(2) * ax) - T(2) * az;
            r = fmaf(b, c, -past);
            r = fmaf(ax, rt + lf, r);
            r = fmaf(az, dn + up, r);
            if (has_src) r = fmaf(-vdt2, src, r);
        }
        const T out = sponge<T, kMode>(r, i, j, p);
        nxt[q] = out;
        const int64_t qd = i + (int64_t)j * p.nz;
        if (p.rec && i == 0) p.rec[j + (int64_t)t * p.nx] = out;
        if (snap) snap[qd] = out;
        if constexpr (kMode == SSSI_MODE_FP64) {
            if (fsnap) {
                const double f = fsnap[qd];
                p.im[qd] = fma(f, (double)out, p.im[qd]);
                p.is2[qd] = fma(f, f, p.is2[qd]);
            }
        }
    }
}

template <typename T, int kMode>
void launch_sponge_step(const SpongeParams<T>& p, int grid, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kSpThreads);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    SSSI_CHECK_CUDA(cudaLaunchKernelEx(&cfg, sponge2d_step_kernel<T, kMode>, p));
    count_launch();
}

// The sponge profile boundary(1..nB) of src/fwdTimeSpongeFor2dAw.m:43-46,
// evaluated as written: (exp(-(alpha (nB - iz))^2))^10 for iz = 0..nB-1.
std::vector<double> sponge_profile(int nB) {
    std::vector<double> b((size_t)nB);
    for (int iz = 0; iz < nB; ++iz) {
        const double a = kSpongeAlpha * (double)(nB - iz);
        b[(size_t)iz] = std::pow(std::exp(-(a * a)), 10.0);
    }
    return b;
}

// One propagation (forward or reverse) of one shot: fields, coefficients,
// hooks and the step loop (graphs of kSpGraphSteps steps).
template <typename T>
class Sponge2d {
  public:
    Sponge2d(const double* v, int64_t nz, int64_t nx, int nB, double dz, double dx, double dt, int mode, int64_t nt,
             bool reverse, cudaStream_t s)
        : nz_((int)nz), nx_((int)nx), mode_(mode), s_(s) {
        ldp_ = ((int64_t)kSpOrgRow + nz + 1 + 31) / 32 * 32;
        const int64_t cols = nx + 2;
        const size_t cells = (size_t)(ldp_ * cols);
        org_ = kSpOrgRow + ldp_;  // interior (0, 0): row kSpOrgRow of column 1
        for (auto& f : F_) {
            f.allocate(cells * sizeof(T));
            f.zero(s);
        }
        // coefficients as the reference forms them (src/fwdTimeSpongeFor2dAw.m:51-55)
        const bool fp64 = mode != SSSI_MODE_FP32;
        std::vector<T> hb, hax, haz, hv(cells, T(0));
        if (fp64) {
            hb.assign(cells, T(0));
            hax.assign(cells, T(0));
            haz.assign(cells, T(0));
        }
        for (int64_t j = 0; j < nx; ++j)
            for (int64_t i = 0; i < nz; ++i) {
                const double vv = v[i + j * nz];
                const double vdt = vv * dt;
                const double ax = (vdt / dx) * (vdt / dx), az = (vdt / dz) * (vdt / dz);
                const size_t q = (size_t)(org_ + i + j * ldp_);
                hv[q] = (T)(vdt * vdt);
                if (fp64) {
                    hax[q] = (T)ax;
                    haz[q] = (T)az;
                    hb[q] = (T)((2.0 - 2.0 * ax) - 2.0 * az);
                }
            }
        auto upload = [&](DeviceBuffer& d, const std::vector<T>& h) {
            d.allocate(cells * sizeof(T));
            SSSI_CHECK_CUDA(cudaMemcpyAsync(d.get(), h.data(), cells * sizeof(T), cudaMemcpyHostToDevice, s));
        };
        upload(vdt2_, hv);
        if (fp64) {
            upload(b_, hb);
            upload(ax_, hax);
            upload(az_, haz);
        }
        const std::vector<double> prof = sponge_profile(nB);
        std::vector<T> hp(prof.begin(), prof.end());
        bnd_.allocate(std::max<size_t>(hp.size(), 1) * sizeof(T));
        if (!hp.empty())
            SSSI_CHECK_CUDA(cudaMemcpyAsync(bnd_.get(), hp.data(), hp.size() * sizeof(T), cudaMemcpyHostToDevice, s));
        hooks_dev_.allocate(sizeof(SpongeHooks<T>));
        ctr_.allocate(sizeof(int));
        ctr_.zero(s);

        p_ = SpongeParams<T>{};
        p_.field[0] = F_[0].template as<T>() + org_;
        p_.field[1] = F_[1].template as<T>() + org_;
        p_.cvdt2 = vdt2_.template as<T>() + org_;
        if (fp64) {
            p_.cb = b_.template as<T>() + org_;
            p_.cax = ax_.template as<T>() + org_;
            p_.caz = az_.template as<T>() + org_;
        }
        p_.bnd = bnd_.template as<T>();
        p_.hooks = hooks_dev_.template as<SpongeHooks<T>>();
        p_.step_base = ctr_.template as<int>();
        p_.nz = nz_;
        p_.nx = nx_;
        p_.nB = nB;
        p_.nt = (int)nt;
        p_.ldp = ldp_;
        p_.ntz = (nz_ + kSpRows - 1) / kSpRows;
        p_.ntiles = p_.ntz * ((nx_ + kSpCols - 1) / kSpCols);
        p_.reverse = reverse ? 1 : 0;
        p_.kx = (T)(1.0 / (dx * dx));
        p_.kz = (T)(1.0 / (dz * dz));
        int dev = 0, sms = 0;
        SSSI_CHECK_CUDA(cudaGetDevice(&dev));
        SSSI_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        grid_ = std::max(1, std::min(p_.ntiles, sms * 8));  // 8 blocks of 256 threads per SM
        set_hooks(SpongeHooks<T>{});
    }
    ~Sponge2d() {
        if (graph_) cudaGraphExecDestroy(graph_);
    }
    SpongeParams<T>& params() { return p_; }
    void set_hooks(const SpongeHooks<T>& h) {
        SSSI_CHECK_CUDA(cudaMemcpyAsync(hooks_dev_.get(), &h, sizeof(h), cudaMemcpyHostToDevice, s_));
        SSSI_CHECK_CUDA(cudaStreamSynchronize(s_));  // the host copy may go out of scope
    }
    // The present field after `done` steps (interior origin, pitch ldp).
    const T* present(int done) const { return p_.field[done & 1]; }
    int64_t ldp() const { return ldp_; }
    // Steps step_ .. step_ + nsteps - 1 (params() must not change while a graph is live).
    void run(int nsteps) {
        int q = 0;
        if (nsteps >= kSpGraphSteps) {
            int* base = ctr_.template as<int>();
            if (!graph_) {
                std::lock_guard<std::mutex> lock(capture_mutex());
                cudaStream_t cs = capture_stream();
                cudaGraph_t g = nullptr;
                SSSI_CHECK_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
                try {
                    for (int k = 0; k < kSpGraphSteps; ++k) launch(k, cs);
                    launch_add_int(base, kSpGraphSteps, cs);
                } catch (...) {
                    cudaStreamEndCapture(cs, &g);
                    if (g) cudaGraphDestroy(g);
                    throw;
                }
                count_launch(-kSpGraphSteps);  // recorded, not run
                cudaError_t e = cudaStreamEndCapture(cs, &g);
                if (e == cudaSuccess) e = cudaGraphInstantiate(&graph_, g, 0);
                if (g) cudaGraphDestroy(g);
                if (e != cudaSuccess) graph_ = nullptr;
                SSSI_CHECK_CUDA(e);
            }
            launch_store_int(base, step_, s_);
            count_launch();
            for (; q + kSpGraphSteps <= nsteps; q += kSpGraphSteps) {
                SSSI_CHECK_CUDA(cudaGraphLaunch(graph_, s_));
                count_launch(kSpGraphSteps + 1);
            }
        }
        if (q < nsteps) {
            launch_store_int(ctr_.template as<int>(), step_ + q, s_);
            count_launch();
            for (int k = 0; q + k < nsteps; ++k) launch(k, s_);
        }
        step_ += nsteps;
    }

  private:
    void launch(int offset, cudaStream_t s) {
        SpongeParams<T> p = p_;
        p.step_offset = offset;
        if constexpr (std::is_same<T, float>::value) {
            launch_sponge_step<T, SSSI_MODE_FP32>(p, grid_, s);
        } else {
            if (mode_ == SSSI_MODE_FP64_STRICT)
                launch_sponge_step<T, SSSI_MODE_FP64_STRICT>(p, grid_, s);
            else
                launch_sponge_step<T, SSSI_MODE_FP64>(p, grid_, s);
        }
    }
    int nz_, nx_, mode_;
    cudaStream_t s_;
    int64_t ldp_ = 0, org_ = 0;
    DeviceBuffer F_[2], b_, ax_, az_, vdt2_, bnd_, hooks_dev_, ctr_;
    SpongeParams<T> p_{};
    int grid_ = 1, step_ = 0;
    cudaGraphExec_t graph_ = nullptr;
};

void check_sponge(int64_t nz, int64_t nx, int64_t nt, int nB, double dz, double dx, double dt, int mode) {
    SSSI_REQUIRE(nz > 0 && nx > 0 && nt >= 0, SSSI_ERR_ARG, "bad sizes nz=%lld nx=%lld nt=%lld", (long long)nz,
                 (long long)nx, (long long)nt);
    SSSI_REQUIRE(nz < (1 << 30) && nx < (1 << 30) && nt < (1 << 30) && nz * nx < (int64_t(1) << 40), SSSI_ERR_ARG,
                 "grid too large");
    SSSI_REQUIRE(nB >= 0 && nB <= nz && nB <= nx, SSSI_ERR_ARG,
                 "nBoundary must be in 0..min(nz, nx) (got %d): the sponge rows and columns lie inside the grid", nB);
    SSSI_REQUIRE(dz > 0 && dx > 0 && dt > 0, SSSI_ERR_ARG, "dz, dx, dt must be positive");
    SSSI_REQUIRE(mode == SSSI_MODE_FP64_STRICT || mode == SSSI_MODE_FP64 || mode == SSSI_MODE_FP32, SSSI_ERR_ARG,
                 "unknown mode %d", mode);
}

// Forward modelling (dense source and/or point sources).  data: nx x nt (row 0
// of every step), snapshot: nz x nx x nt; either may be NULL.
template <typename T>
void sponge_fwd(const double* v, const double* source, int64_t nz, int64_t nx, int64_t nt, int nB, double dz,
                double dx, double dt, int mode, int nsrc, const int64_t* src_iz, const int64_t* src_ix,
                const double* wavelets, double* data, double* snapshot) {
    cudaStream_t s = current_stream();
    const int64_t n = nz * nx;
    std::vector<double> vh = host_copy(v, (size_t)n, s);
    Sponge2d<T> P(vh.data(), nz, nx, nB, dz, dx, dt, mode, nt, false, s);
    Staged<T> rec(data, (size_t)(nx * nt), false, s);
    Staged<T> wav(wavelets, (size_t)(nsrc * nt), true, s);
    DeviceBuffer d_iz, d_ix;
    if (nsrc > 0) {
        std::vector<int> hz((size_t)nsrc), hx((size_t)nsrc);
        for (int k = 0; k < nsrc; ++k) {
            SSSI_REQUIRE(src_iz[k] >= 0 && src_iz[k] < nz && src_ix[k] >= 0 && src_ix[k] < nx, SSSI_ERR_ARG,
                         "point source %d at (%lld, %lld) lies outside the %lld x %lld grid", k, (long long)src_iz[k],
                         (long long)src_ix[k], (long long)nz, (long long)nx);
            hz[(size_t)k] = (int)src_iz[k];
            hx[(size_t)k] = (int)src_ix[k];
        }
        d_iz.allocate(sizeof(int) * nsrc);
        d_ix.allocate(sizeof(int) * nsrc);
        SSSI_CHECK_CUDA(cudaMemcpyAsync(d_iz.get(), hz.data(), sizeof(int) * nsrc, cudaMemcpyHostToDevice, s));
        SSSI_CHECK_CUDA(cudaMemcpyAsync(d_ix.get(), hx.data(), sizeof(int) * nsrc, cudaMemcpyHostToDevice, s));
        P.params().nsrc = nsrc;
        P.params().src_iz = d_iz.template as<int>();
        P.params().src_ix = d_ix.template as<int>();
        P.params().wavelets = wav.ptr;
    }
    P.params().rec = rec.ptr;
    const int64_t K = (source || snapshot) ? chunk_steps(nt, n) : std::max<int64_t>(nt, 1);
    SliceStream<T> src(const_cast<double*>(source), n, K), snap(snapshot, n, K);
    timing_begin(s);
    for (int64_t t0 = 0; t0 < nt; t0 += K) {
        const int64_t kk = std::min(K, nt - t0);
        src.load(t0, kk, s);
        SpongeHooks<T> h{};
        h.src_dense = source ? src.slice(t0, t0) : nullptr;
        h.dense_t0 = (int)t0;
        h.snap = snapshot ? snap.slice(t0, t0) : nullptr;
        h.snap_t0 = (int)t0;
        P.set_hooks(h);
        P.run((int)kk);
        snap.store(t0, kk, s);
    }
    timing_end(s);
    rec.download(data, s);
    SSSI_CHECK_CUDA(cudaStreamSynchronize(s));
}

// Copies the interior of a padded field into a dense nz x nx array of doubles.
template <typename T>
__global__ void sponge_interior_kernel(const T* f, int64_t ldp, int nz, int nx, double* out) {
    const int64_t n = (int64_t)nz * nx;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = q % nz, j = q / nz;
        out[q] = (double)f[i + j * ldp];
    }
}

// Reverse propagation of data (nx x nt) injected on row 0, t = nt-1 .. 0.
// model: nz x nx, the present field after the last step (t = 0); the
// reference's rvsTimeSpongeFor2dAw.m never assigns its `model` output.
template <typename T>
void sponge_rvs(const double* v, const double* data, int64_t nz, int64_t nx, int64_t nt, int nB, double dz,
                double dx, double dt, int mode, double* model, double* snapshot) {
    cudaStream_t s = current_stream();
    const int64_t n = nz * nx;
    std::vector<double> vh = host_copy(v, (size_t)n, s);
    Sponge2d<T> P(vh.data(), nz, nx, nB, dz, dx, dt, mode, nt, true, s);
    Staged<T> rows(data, (size_t)(nx * nt), true, s);
    P.params().src_row = data ? rows.ptr : nullptr;
    const int64_t K = snapshot ? chunk_steps(nt, n) : std::max<int64_t>(nt, 1);
    SliceStream<T> snap(snapshot, n, K);
    timing_begin(s);
    for (int64_t t_hi = nt; t_hi > 0; t_hi -= K) {
        const int64_t t0 = std::max<int64_t>(0, t_hi - K);
        SpongeHooks<T> h{};
        h.snap = snapshot ? snap.slice(t0, t0) : nullptr;
        h.snap_t0 = (int)t0;
        P.set_hooks(h);
        P.run((int)(t_hi - t0));
        snap.store(t0, t_hi - t0, s);
    }
    timing_end(s);
    if (model) {
        DeviceView out(model, (size_t)n, false, s);
        sponge_interior_kernel<T><<<152 * 4, 256, 0, s>>>(P.present((int)nt), P.ldp(), (int)nz, (int)nx, out.ptr);
        count_launch();
        SSSI_CHECK_CUDA(cudaGetLastError());
        out.download(model, (size_t)n, s);
    }
    SSSI_CHECK_CUDA(cudaStreamSynchronize(s));
}

// One RTM shot (FP64 modes): forward in v (dataTrue) and vs (dataSmooth, the
// forward snapshots), reverse of dataTrue - dataSmooth in v, and
//     image = M ./ s2,  M = sum_t f_t .* r_t,  s2 = epsilon + sum_t f_t.^2
// (mainRtmTimeSpongeFor2dAw.m:247-268,310).  Strict: every snapshot kept in FP64
// and the sums formed in the reference's order (t ascending) after the
// reverse pass; fused: the sums accumulate inside the reverse step.
void sponge_rtm(const double* v, const double* vs, int64_t nz, int64_t nx, int64_t nt, int nB, double dz, double dx,
                double dt, const double* wavelet, int64_t siz, int64_t six, double eps, int mode, double* image,
                double* data_true, double* data_smooth) {
    SSSI_REQUIRE(siz >= 0 && siz < nz && six >= 0 && six < nx, SSSI_ERR_ARG, "source (%lld, %lld) outside the grid",
                 (long long)siz, (long long)six);
    cudaStream_t s = current_stream();
    const int64_t n = nz * nx;
    std::vector<double> vh = host_copy(v, (size_t)n, s), vsh = host_copy(vs, (size_t)n, s);
    Staged<double> wav(wavelet, (size_t)nt, true, s);
    DeviceBuffer d_src(2 * sizeof(int));
    const int hsrc[2] = {(int)siz, (int)six};
    SSSI_CHECK_CUDA(cudaMemcpyAsync(d_src.get(), hsrc, sizeof(hsrc), cudaMemcpyHostToDevice, s));
    DeviceBuffer rec_true((size_t)(nx * std::max<int64_t>(nt, 1)) * sizeof(double)),
        rec_smooth((size_t)(nx * std::max<int64_t>(nt, 1)) * sizeof(double));
    DeviceBuffer fsnap((size_t)(n * std::max<int64_t>(nt, 1)) * sizeof(double));
    const bool strict = mode == SSSI_MODE_FP64_STRICT;
    timing_begin(s);
    for (int pass = 0; pass < 2; ++pass) {
        Sponge2d<double> P(pass == 0 ? vh.data() : vsh.data(), nz, nx, nB, dz, dx, dt, mode, nt, false, s);
        SpongeParams<double>& p = P.params();
        p.nsrc = 1;
        p.src_iz = d_src.as<int>();
        p.src_ix = d_src.as<int>() + 1;
        p.wavelets = wav.ptr;
        p.rec = (pass == 0 ? rec_true : rec_smooth).as<double>();
        SpongeHooks<double> h{};
        if (pass == 1) h.snap = fsnap.as<double>();
        P.set_hooks(h);
        P.run((int)nt);
    }
    timing_mark(s);
    DeviceBuffer delta((size_t)(nx * std::max<int64_t>(nt, 1)) * sizeof(double));
    diff_kernel<double><<<152 * 4, 256, 0, s>>>(rec_true.as<double>(), rec_smooth.as<double>(), delta.as<double>(),
                                               nx * nt);
    count_launch();
    SSSI_CHECK_CUDA(cudaGetLastError());
    DeviceView img(image, (size_t)n, false, s);
    {
        Sponge2d<double> R(vh.data(), nz, nx, nB, dz, dx, dt, mode, nt, true, s);
        R.params().src_row = delta.as<double>();
        DeviceBuffer rsnap, msum, ssum;
        SpongeHooks<double> h{};
        if (strict) {
            rsnap.allocate((size_t)(n * std::max<int64_t>(nt, 1)) * sizeof(double));
            h.snap = rsnap.as<double>();
        } else {
            msum.allocate((size_t)n * sizeof(double));
            ssum.allocate((size_t)n * sizeof(double));
            msum.zero(s);
            ssum.zero(s);
            h.fsnap = fsnap.as<double>();
            R.params().im = msum.as<double>();
            R.params().is2 = ssum.as<double>();
        }
        R.set_hooks(h);
        R.run((int)nt);
        if (strict) {
            image_ascending_kernel<<<152 * 4, 256, 0, s>>>(fsnap.as<double>(), rsnap.as<double>(), n, nt, eps, img.ptr);
        } else {
            image_finish_kernel<<<152 * 4, 256, 0, s>>>(msum.as<double>(), ssum.as<double>(), n, 1.0, eps, img.ptr);
        }
        count_launch();
        SSSI_CHECK_CUDA(cudaGetLastError());
    }
    timing_end(s);
    img.download(image, (size_t)n, s);
    if (data_true)
        SSSI_CHECK_CUDA(cudaMemcpyAsync(data_true, rec_true.get(), sizeof(double) * nx * nt, cudaMemcpyDefault, s));
    if (data_smooth)
        SSSI_CHECK_CUDA(
            cudaMemcpyAsync(data_smooth, rec_smooth.get(), sizeof(double) * nx * nt, cudaMemcpyDefault, s));
    SSSI_CHECK_CUDA(cudaStreamSynchronize(s));
}

}  // namespace
}  // namespace sssi

using namespace sssi;

extern "C" {

int sssi_fwdTimeSpongeFor2dAw(const double* v, const double* source, int64_t nz, int64_t nx, int64_t nt,
                              int nBoundary, double dz, double dx, double dt, double* data, double* snapshot,
                              int mode) {
    return guarded([&] {
        check_sponge(nz, nx, nt, nBoundary, dz, dx, dt, mode);
        SSSI_REQUIRE(v && source, SSSI_ERR_ARG, "v and source are required");
        ensure_device();
        if (nt == 0) return;
        if (mode == SSSI_MODE_FP32)
            sponge_fwd<float>(v, source, nz, nx, nt, nBoundary, dz, dx, dt, mode, 0, nullptr, nullptr, nullptr, data,
                              snapshot);
        else
            sponge_fwd<double>(v, source, nz, nx, nt, nBoundary, dz, dx, dt, mode, 0, nullptr, nullptr, nullptr, data,
                               snapshot);
    });
}

int sssi_fwdTimeSpongeFor2dAwPoint(const double* v, int64_t nz, int64_t nx, int64_t nt, int nBoundary, double dz,
                                   double dx, double dt, int nsrc, const int64_t* src_iz, const int64_t* src_ix,
                                   const double* wavelets, double* data, double* snapshot, int mode) {
    return guarded([&] {
        check_sponge(nz, nx, nt, nBoundary, dz, dx, dt, mode);
        SSSI_REQUIRE(v, SSSI_ERR_ARG, "v is required");
        SSSI_REQUIRE(nsrc >= 0 && nsrc <= 64, SSSI_ERR_ARG, "nsrc must be in 0..64 (got %d)", nsrc);
        SSSI_REQUIRE(nsrc == 0 || (src_iz && src_ix && wavelets), SSSI_ERR_ARG, "point sources need positions and wavelets");
        ensure_device();
        if (nt == 0) return;
        if (mode == SSSI_MODE_FP32)
            sponge_fwd<float>(v, nullptr, nz, nx, nt, nBoundary, dz, dx, dt, mode, nsrc, src_iz, src_ix, wavelets,
                              data, snapshot);
        else
            sponge_fwd<double>(v, nullptr, nz, nx, nt, nBoundary, dz, dx, dt, mode, nsrc, src_iz, src_ix, wavelets,
                               data, snapshot);
    });
}

int sssi_rvsTimeSpongeFor2dAw(const double* v, const double* data, int64_t nz, int64_t nx, int64_t nt,
                              int nBoundary, double dz, double dx, double dt, double* model, double* snapshot,
                              int mode) {
    return guarded([&] {
        check_sponge(nz, nx, nt, nBoundary, dz, dx, dt, mode);
        SSSI_REQUIRE(v && data, SSSI_ERR_ARG, "v and data are required");
        ensure_device();
        if (nt == 0) {
            if (model) {
                cudaStream_t s = current_stream();
                DeviceView out(model, (size_t)(nz * nx), false, s);
                fill(out.ptr, nz * nx, 0.0, s);
                out.download(model, (size_t)(nz * nx), s);
                SSSI_CHECK_CUDA(cudaStreamSynchronize(s));
            }
            return;
        }
        if (mode == SSSI_MODE_FP32)
            sponge_rvs<float>(v, data, nz, nx, nt, nBoundary, dz, dx, dt, mode, model, snapshot);
        else
            sponge_rvs<double>(v, data, nz, nx, nt, nBoundary, dz, dx, dt, mode, model, snapshot);
    });
}

int sssi_rtmTimeSpongeFor2dAw(const double* v, const double* vs, int64_t nz, int64_t nx, int64_t nt, int nBoundary,
                              double dz, double dx, double dt, const double* wavelet, int64_t src_iz, int64_t src_ix,
                              double epsilon, int mode, double* image, double* data_true, double* data_smooth) {
    return guarded([&] {
        check_sponge(nz, nx, nt, nBoundary, dz, dx, dt, mode);
        SSSI_REQUIRE(v && vs && wavelet && image, SSSI_ERR_ARG, "v, vs, wavelet and image are required");
        SSSI_REQUIRE(nt >= 1, SSSI_ERR_ARG, "nt must be at least 1");
        SSSI_REQUIRE(mode != SSSI_MODE_FP32, SSSI_ERR_ARG,
                     "the sponge RTM shot runs in FP64 (SSSI_MODE_FP64 or SSSI_MODE_FP64_STRICT)");
        ensure_device();
        sponge_rtm(v, vs, nz, nx, nt, nBoundary, dz, dx, dt, wavelet, src_iz, src_ix, epsilon, mode, image, data_true,
                   data_smooth);
    });
}

}  // extern "C"
