// 2D elastic propagation with the simplified PML of src/fwdTimeSpmlFor2dEw.m:38-103
// (MATLAB only in the reference), on the device.
//
// The file advances the velocity split into P and S parts through two
// potentials: per step
//   A_x = rx .* A_x + sx .* Dx-(Vx),   A_z = rz .* A_z + sz .* Dz-(Vz),   A = A_x + A_z
//   B_z = rz .* B_z + sz .* Dz+(Vx),   B_x = rx .* B_x - sx .* Dx+(Vz),   B = B_z + B_x
//   Vzp = rz .* Vzp + kzp .* Dz+(A) + sz .* src      Vxp = rx .* Vxp + kxp .* Dx+(A) + sx .* src
//   Vzs = rx .* Vzs - kzs .* Dx-(B)                  Vxs = rz .* Vxs + kxs .* Dz-(B)
//   Vx = Vxp + Vxs,  Vz = Vzp + Vzs
// with r = (1 - 0.5 d dt) ./ (1 + 0.5 d dt), s = dt ./ (1 + 0.5 d dt) from the
// damping d of each axis (dampPml in cell units: only the side columns damp x,
// only the bottom rows damp z), kzp = 0.25 (4-point average of vp^2) dt ./ den_z,
// kxp = vp^2 dt ./ den_x, kzs = vs^2 dt ./ den_x, kxs = 0.25 (4-point average of
// vs^2) dt ./ den_z, and the staggered derivatives of diffOperator on the
// zero-padded fields:  D-(f)(i) = sum_k c_k (f(i+k) - f(i-1-k)) / d  and
// D+(f)(i) = sum_k c_k (f(i+1+k) - f(i-k)) / d  (the slices the file hands to
// diffOperator: `Vx(iz, 1:end-1)` is D-, `Vx(2:end, ix)` is D+, ...).
//
// GB300 form: two launches per step (phase 1 writes A and B, whose stencils
// phase 2 needs whole), one thread per cell on 32 x 8 block tiles (one warp per
// column, coalesced along z; the x neighbours of a tile's inner columns come
// from L1), a persistent grid, runs of steps replayed as CUDA graphs that read
// the step number and the chunked hooks from device memory.  Outside the bands
// r = 1, s = dt and the divisions by den = 1 are exact no-ops, so the band
// coefficients live in two small arrays (side columns nz x 2nB, bottom rows
// nB x nx), the interior takes the constants and forms no product with r.
// The velocity updates' coefficients kzp, kxs, kxp, kzs do not change in
// time: they are formed once per run, with the step's operations, and loaded.
//
// Arithmetic: SSSI_MODE_FP64_STRICT rounds as the file (and diffOperator_mex,
// src/fd_cmex/diffOperator_mex.c:81-92: c_k*(a-b)/d per term, summed from zero)
// do, with no fused multiply-add; SSSI_MODE_FP64 folds c_k/d and fuses;
// SSSI_MODE_FP32 does the fused form in FP32.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "api_util.cuh"
#include "elastic_common.cuh"
#include "sssi_internal.h"

namespace sssi {
namespace {

using namespace api;
using namespace elastic;

constexpr int kElMaxOrder = 8;
constexpr int kElRows = 32, kElCols = 8, kElThreads = kElRows * kElCols;
constexpr int kElOrgRow = 32;       // interior row 0 within a padded column (>= nDiffOrder)
constexpr int kElGraphSteps = 16;   // steps per graph (two launches each)

template <typename T>
struct ElHooks {
    const T* src_dense;  // nz x nx slices (pitch nz): slice of step t at src_dense + (t - dense_t0) * nz * nx
    T* snap[4];          // Vzp, Vxp, Vzs, Vxs snapshots, same layout (t - snap_t0)
    int dense_t0, snap_t0;
};

template <typename T>
struct ElParams {
    // padded fields (interior origin applied, pitch ldp)
    T* Vx;
    T* Vz;
    T* A;
    T* B;
    T* Ax;
    T* Az;
    T* Bz;
    T* Bx;
    T* Vzp;
    T* Vxp;
    T* Vzs;
    T* Vxs;
    const T* vpSq;  // vp.^2 and vs.^2 padded by edge replication (padarray 'replicate')
    const T* vsSq;
    // the velocity updates' coefficients kzp, kxs, kxp, kzs (constant in time,
    // formed once by el_coef_kernel), padded layout
    const T* kzp;
    const T* kxs;
    const T* kxp;
    const T* kzs;
    // band coefficients: side columns (nz x 2 nB, pitch nz; column j < nB, or
    // nB + j - (nx - nB)), bottom rows (nB x nx, pitch nB; row i - (nz - nB))
    const T* xr;
    const T* xs;
    const T* xden;
    const T* zr;
    const T* zs;
    const T* zden;
    T dt;
    T c[kElMaxOrder];   // strict: coefficients, divided by dz / dx per term
    T wz[kElMaxOrder];  // fused: c_k / dz, c_k / dx
    T wx[kElMaxOrder];
    Divisor<T> dz, dx;  // strict: the spacings the terms are divided by
    int nz, nx, nB, nt;
    int64_t ldp;
    int ntz, ntiles;
    const ElHooks<T>* hooks;
    const int* step_base;
    int step_offset;
    int nsrc;  // point sources: cell (src_iz[k], src_ix[k]) takes wavelets[k * nt + t]
    const int* src_iz;
    const int* src_ix;
    const T* wavelets;
};

// Damping factors of cell (i, j): x from the side columns, z from the bottom rows.
template <typename T>
__device__ __forceinline__ void el_factors(const ElParams<T>& p, int i, int j, T& rx, T& sx, T& dnx, T& rz, T& sz,
                                           T& dnz) {
    rx = T(1);
    sx = p.dt;
    dnx = T(1);
    rz = T(1);
    sz = p.dt;
    dnz = T(1);
    const int nB = p.nB;
    if (j < nB || j >= p.nx - nB) {
        const int64_t b = i + (int64_t)(j < nB ? j : nB + j - (p.nx - nB)) * p.nz;
        rx = __ldg(p.xr + b);
        sx = __ldg(p.xs + b);
        dnx = __ldg(p.xden + b);
    }
    if (i >= p.nz - nB) {
        const int64_t b = (i - (p.nz - nB)) + (int64_t)j * nB;
        rz = __ldg(p.zr + b);
        sz = __ldg(p.zs + b);
        dnz = __ldg(p.zden + b);
    }
}

template <typename T>
__device__ __forceinline__ int el_step(const ElParams<T>& p) {
    return *reinterpret_cast<volatile const int*>(p.step_base) + p.step_offset;
}

// Phase 1: the potentials' split parts and sums from the velocities' derivatives.
template <typename T, int N, int kMode>
__global__ void __launch_bounds__(kElThreads) elastic2d_phase1_kernel(const __grid_constant__ ElParams<T> p) {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t ldp = p.ldp;
    T c[N], wz[N], wx[N];
#pragma unroll
    for (int k = 0; k < N; ++k) {
        c[k] = p.c[k];
        wz[k] = p.wz[k];
        wx[k] = p.wx[k];
    }
    const Divisor<T> dz = p.dz, dx = p.dx;
    for (int tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x) {
        const int i = (tile % p.ntz) * kElRows + lane, j = (tile / p.ntz) * kElCols + w;
        if (i >= p.nz || j >= p.nx) continue;
        const int64_t q = i + (int64_t)j * ldp;
        T rx, sx, dnx, rz, sz, dnz;
        el_factors(p, i, j, rx, sx, dnx, rz, sz, dnz);
        const T dVxx = el_diff<T, N, kMode, false>(p.Vx, q, ldp, c, wx, dx);  // Vx(iz, 1:end-1), dim 2
        const T dVzz = el_diff<T, N, kMode, false>(p.Vz, q, 1, c, wz, dz);    // Vz(1:end-1, ix), dim 1
        const T dVxz = el_diff<T, N, kMode, true>(p.Vx, q, 1, c, wz, dz);     // Vx(2:end, ix), dim 1
        const T dVzx = el_diff<T, N, kMode, true>(p.Vz, q, ldp, c, wx, dx);   // Vz(iz, 2:end), dim 2
        const bool xb = j < p.nB || j >= p.nx - p.nB, zb = i >= p.nz - p.nB;  // damped along x / z
        const T ax = el_raxpby<T, kMode, true>(xb, rx, p.Ax[q], sx, dVxx);
        const T az = el_raxpby<T, kMode, true>(zb, rz, p.Az[q], sz, dVzz);
        const T bz = el_raxpby<T, kMode, true>(zb, rz, p.Bz[q], sz, dVxz);
        const T bx = el_sub<T, kMode>(el_rx<T, kMode, true>(xb, rx, p.Bx[q]), el_mul<T, kMode>(sx, dVzx));
        p.Ax[q] = ax;
        p.Az[q] = az;
        p.Bz[q] = bz;
        p.Bx[q] = bx;
        p.A[q] = el_add<T, kMode>(ax, az);
        p.B[q] = el_add<T, kMode>(bz, bx);
    }
}

// Phase 2: the velocities from the potentials' derivatives, sources, snapshots.
template <typename T, int N, int kMode>
__global__ void __launch_bounds__(kElThreads) elastic2d_phase2_kernel(const __grid_constant__ ElParams<T> p) {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const int t = el_step(p);
    const ElHooks<T> h = *p.hooks;
    const int64_t n = (int64_t)p.nz * p.nx;
    const T* src_dense = h.src_dense ? h.src_dense + (int64_t)(t - h.dense_t0) * n : nullptr;
    T* snap[4];
#pragma unroll
    for (int s = 0; s < 4; ++s) snap[s] = h.snap[s] ? h.snap[s] + (int64_t)(t - h.snap_t0) * n : nullptr;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t ldp = p.ldp;
    T c[N], wz[N], wx[N];
#pragma unroll
    for (int k = 0; k < N; ++k) {
        c[k] = p.c[k];
        wz[k] = p.wz[k];
        wx[k] = p.wx[k];
    }
    const Divisor<T> dz = p.dz, dx = p.dx;
    for (int tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x) {
        const int i = (tile % p.ntz) * kElRows + lane, j = (tile / p.ntz) * kElCols + w;
        if (i >= p.nz || j >= p.nx) continue;
        const int64_t q = i + (int64_t)j * ldp;
        T rx, sx, dnx, rz, sz, dnz;
        el_factors(p, i, j, rx, sx, dnx, rz, sz, dnz);
        const T dAz = el_diff<T, N, kMode, true>(p.A, q, 1, c, wz, dz);     // A(2:end, ix), dim 1
        const T dAx = el_diff<T, N, kMode, true>(p.A, q, ldp, c, wx, dx);   // A(iz, 2:end), dim 2
        const T dBx = el_diff<T, N, kMode, false>(p.B, q, ldp, c, wx, dx);  // B(iz, 1:end-1), dim 2
        const T dBz = el_diff<T, N, kMode, false>(p.B, q, 1, c, wz, dz);    // B(1:end-1, ix), dim 1
        const T kzp = __ldg(p.kzp + q), kxs = __ldg(p.kxs + q), kxp = __ldg(p.kxp + q), kzs = __ldg(p.kzs + q);
        const bool xb = j < p.nB || j >= p.nx - p.nB, zb = i >= p.nz - p.nB;  // damped along x / z
        T src = T(0);
        bool has_src = false;
        if (src_dense) {
            src = src_dense[i + (int64_t)j * p.nz];
            has_src = true;
        }
        for (int k = 0; k < p.nsrc; ++k)
            if (p.src_iz[k] == i && p.src_ix[k] == j) {
                const T wv = p.wavelets[(int64_t)k * p.nt + t];
                src = has_src ? src + wv : wv;
                has_src = true;
            }
        T vzp = el_raxpby<T, kMode, true>(zb, rz, p.Vzp[q], kzp, dAz);
        T vxp = el_raxpby<T, kMode, true>(xb, rx, p.Vxp[q], kxp, dAx);
        if (has_src) {
            vzp = el_add<T, kMode>(vzp, el_mul<T, kMode>(sz, src));
            vxp = el_add<T, kMode>(vxp, el_mul<T, kMode>(sx, src));
        }
        const T vzs = el_sub<T, kMode>(el_rx<T, kMode, true>(xb, rx, p.Vzs[q]), el_mul<T, kMode>(kzs, dBx));
        const T vxs = el_raxpby<T, kMode, true>(zb, rz, p.Vxs[q], kxs, dBz);
        p.Vzp[q] = vzp;
        p.Vxp[q] = vxp;
        p.Vzs[q] = vzs;
        p.Vxs[q] = vxs;
        p.Vx[q] = el_add<T, kMode>(vxp, vxs);
        p.Vz[q] = el_add<T, kMode>(vzp, vzs);
        const int64_t qd = i + (int64_t)j * p.nz;
        if (snap[0]) snap[0][qd] = vzp;
        if (snap[1]) snap[1][qd] = vxp;
        if (snap[2]) snap[2][qd] = vzs;
        if (snap[3]) snap[3][qd] = vxs;
    }
}

template <typename T>
void el_launch(void (*kernel)(ElParams<T>), const ElParams<T>& p, int grid, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kElThreads);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    SSSI_CHECK_CUDA(cudaLaunchKernelEx(&cfg, kernel, p));
    count_launch();
}

template <typename T, int N>
void el_launch_step(const ElParams<T>& p, int mode, int grid, cudaStream_t s) {
    if constexpr (std::is_same<T, float>::value) {
        el_launch<T>(elastic2d_phase1_kernel<T, N, SSSI_MODE_FP32>, p, grid, s);
        el_launch<T>(elastic2d_phase2_kernel<T, N, SSSI_MODE_FP32>, p, grid, s);
    } else if (mode == SSSI_MODE_FP64_STRICT) {
        el_launch<T>(elastic2d_phase1_kernel<T, N, SSSI_MODE_FP64_STRICT>, p, grid, s);
        el_launch<T>(elastic2d_phase2_kernel<T, N, SSSI_MODE_FP64_STRICT>, p, grid, s);
    } else {
        el_launch<T>(elastic2d_phase1_kernel<T, N, SSSI_MODE_FP64>, p, grid, s);
        el_launch<T>(elastic2d_phase2_kernel<T, N, SSSI_MODE_FP64>, p, grid, s);
    }
}

template <typename T>
void el_launch_step_n(int N, const ElParams<T>& p, int mode, int grid, cudaStream_t s) {
    switch (N) {
        case 1: el_launch_step<T, 1>(p, mode, grid, s); break;
        case 2: el_launch_step<T, 2>(p, mode, grid, s); break;
        case 3: el_launch_step<T, 3>(p, mode, grid, s); break;
        case 4: el_launch_step<T, 4>(p, mode, grid, s); break;
        case 5: el_launch_step<T, 5>(p, mode, grid, s); break;
        case 6: el_launch_step<T, 6>(p, mode, grid, s); break;
        case 7: el_launch_step<T, 7>(p, mode, grid, s); break;
        default: el_launch_step<T, 8>(p, mode, grid, s); break;
    }
}

// vp.^2, vs.^2 padded by nDiffOrder with edge replication (padarray 'replicate'),
// into the padded layout (interior origin applied to the outputs).
template <typename T>
__global__ void el_square_kernel(const double* vp, const double* vs, int nz, int nx, int N, int64_t ldp, T* vp2,
                                 T* vs2) {
    const int64_t rows = nz + 2 * N, cols = nx + 2 * N, n = rows * cols;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const int ip = (int)(q % rows) - N, jp = (int)(q / rows) - N;
        const int i = min(max(ip, 0), nz - 1), j = min(max(jp, 0), nx - 1);
        const double a = vp[i + (int64_t)j * nz], b = vs[i + (int64_t)j * nz];
        const int64_t o = ip + (int64_t)jp * ldp;
        vp2[o] = (T)__dmul_rn(a, a);
        vs2[o] = (T)__dmul_rn(b, b);
    }
}

// The velocity updates' coefficients, constant in time, in the step's
// operation order: kzp = 0.25 (vpSq(iz,ix) + vpSq(iz+1,ix) + vpSq(iz+1,ix-1) +
// vpSq(iz,ix-1)) dt ./ den_z, kxs = 0.25 (vsSq(iz,ix) + vsSq(iz,ix+1) +
// vsSq(iz-1,ix+1) + vsSq(iz-1,ix)) dt ./ den_z, kxp = vpSq dt ./ den_x,
// kzs = vsSq dt ./ den_x (den = 1 outside the bands: the division is exact
// there and skipped).
template <typename T, int kMode>
__global__ void el_coef_kernel(const ElParams<T> p, T* kzp_out, T* kxs_out, T* kxp_out, T* kzs_out) {
    const int64_t n = (int64_t)p.nz * p.nx, ldp = p.ldp;
    const T dt = p.dt;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(c % p.nz), j = (int)(c / p.nz);
        const int64_t q = i + (int64_t)j * ldp;
        T rx, sx, dnx, rz, sz, dnz;
        el_factors(p, i, j, rx, sx, dnx, rz, sz, dnz);
        const T p00 = p.vpSq[q], s00 = p.vsSq[q];
        const T s4p = el_add<T, kMode>(el_add<T, kMode>(el_add<T, kMode>(p00, p.vpSq[q + 1]), p.vpSq[q + 1 - ldp]),
                                       p.vpSq[q - ldp]);
        const T s4s = el_add<T, kMode>(el_add<T, kMode>(el_add<T, kMode>(s00, p.vsSq[q + ldp]), p.vsSq[q - 1 + ldp]),
                                       p.vsSq[q - 1]);
        T kzp = el_mul<T, kMode>(el_mul<T, kMode>(T(0.25), s4p), dt);
        T kxs = el_mul<T, kMode>(el_mul<T, kMode>(T(0.25), s4s), dt);
        T kxp = el_mul<T, kMode>(p00, dt);
        T kzs = el_mul<T, kMode>(s00, dt);
        if (dnz != T(1)) {
            kzp = el_div<T, kMode>(kzp, dnz);
            kxs = el_div<T, kMode>(kxs, dnz);
        }
        if (dnx != T(1)) {
            kxp = el_div<T, kMode>(kxp, dnx);
            kzs = el_div<T, kMode>(kzs, dnx);
        }
        kzp_out[q] = kzp;
        kxs_out[q] = kxs;
        kxp_out[q] = kxp;
        kzs_out[q] = kzs;
    }
}

template <typename T>
class Elastic2d {
  public:
    // vp, vs: host arrays (nz x nx doubles); dvp, dvs: the same on the device
    Elastic2d(const double* vp, const double* dvp, const double* dvs, int64_t nz, int64_t nx, int64_t nt, int N,
              int nB, double dz, double dx, double dt, int mode, cudaStream_t s)
        : N_(N), mode_(mode), s_(s) {
        ldp_ = (int64_t)kElOrgRow + (nz + 31) / 32 * 32 + 32;
        const int64_t cols = nx + 2 * N;
        const size_t cells = (size_t)(ldp_ * cols);
        org_ = kElOrgRow + (int64_t)N * ldp_;
        for (auto& f : F_) {
            f.allocate(cells * sizeof(T));
            f.zero(s);
        }
        for (auto& f : V2_) {
            f.allocate(cells * sizeof(T));
            f.zero(s);
        }
        el_square_kernel<T><<<152 * 4, 256, 0, s>>>(dvp, dvs, (int)nz, (int)nx, N, ldp_, V2_[0].template as<T>() + org_,
                                                    V2_[1].template as<T>() + org_);
        count_launch();
        SSSI_CHECK_CUDA(cudaGetLastError());
        // band coefficients (src/fwdTimeSpmlFor2dEw.m:47-55): x from the side
        // columns (u = nB..1 on the left, 1..nB on the right), z from the bottom
        // rows (u = 1..nB), velocity vp of the cell, L = nB cells
        const size_t nxb = (size_t)std::max<int64_t>(nz * 2 * nB, 1), nzb = (size_t)std::max<int64_t>((int64_t)nB * nx, 1);
        std::vector<T> hxr(nxb), hxs(nxb), hxd(nxb), hzr(nzb), hzs(nzb), hzd(nzb);
        const double L = (double)nB;
        for (int b = 0; b < 2 * nB; ++b) {
            const int64_t j = b < nB ? b : nx - nB + (b - nB);
            const double u = b < nB ? (double)(nB - b) : (double)(b - nB + 1);
            for (int64_t i = 0; i < nz; ++i) {
                double r, sv, den;
                el_band(vp[i + j * nz], u, L, dt, r, sv, den);
                hxr[(size_t)(i + b * nz)] = (T)r;
                hxs[(size_t)(i + b * nz)] = (T)sv;
                hxd[(size_t)(i + b * nz)] = (T)den;
            }
        }
        for (int64_t j = 0; j < nx; ++j)
            for (int b = 0; b < nB; ++b) {
                const int64_t i = nz - nB + b;
                double r, sv, den;
                el_band(vp[i + j * nz], (double)(b + 1), L, dt, r, sv, den);
                hzr[(size_t)(b + j * nB)] = (T)r;
                hzs[(size_t)(b + j * nB)] = (T)sv;
                hzd[(size_t)(b + j * nB)] = (T)den;
            }
        auto upload = [&](DeviceBuffer& d, const std::vector<T>& h) {
            d.allocate(h.size() * sizeof(T));
            SSSI_CHECK_CUDA(cudaMemcpyAsync(d.get(), h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s));
        };
        upload(band_[0], hxr);
        upload(band_[1], hxs);
        upload(band_[2], hxd);
        upload(band_[3], hzr);
        upload(band_[4], hzs);
        upload(band_[5], hzd);
        hooks_dev_.allocate(sizeof(ElHooks<T>));
        ctr_.allocate(sizeof(int));
        ctr_.zero(s);

        p_ = ElParams<T>{};
        T* f[12];
        for (int k = 0; k < 12; ++k) f[k] = F_[k].template as<T>() + org_;
        p_.Vx = f[0];
        p_.Vz = f[1];
        p_.A = f[2];
        p_.B = f[3];
        p_.Ax = f[4];
        p_.Az = f[5];
        p_.Bz = f[6];
        p_.Bx = f[7];
        p_.Vzp = f[8];
        p_.Vxp = f[9];
        p_.Vzs = f[10];
        p_.Vxs = f[11];
        p_.vpSq = V2_[0].template as<T>() + org_;
        p_.vsSq = V2_[1].template as<T>() + org_;
        p_.xr = band_[0].template as<T>();
        p_.xs = band_[1].template as<T>();
        p_.xden = band_[2].template as<T>();
        p_.zr = band_[3].template as<T>();
        p_.zs = band_[4].template as<T>();
        p_.zden = band_[5].template as<T>();
        p_.dt = (T)dt;
        std::vector<double> cf(N);
        staggered_coefficients(N, cf.data());
        for (int k = 0; k < N; ++k) {
            p_.c[k] = (T)cf[k];
            p_.wz[k] = (T)(cf[k] / dz);
            p_.wx[k] = (T)(cf[k] / dx);
        }
        p_.dz = make_divisor<T>(dz);
        p_.dx = make_divisor<T>(dx);
        p_.nz = (int)nz;
        p_.nx = (int)nx;
        p_.nB = nB;
        p_.nt = (int)nt;
        p_.ldp = ldp_;
        p_.ntz = (int)((nz + kElRows - 1) / kElRows);
        p_.ntiles = p_.ntz * (int)((nx + kElCols - 1) / kElCols);
        p_.hooks = hooks_dev_.template as<ElHooks<T>>();
        p_.step_base = ctr_.template as<int>();
        int dev = 0, sms = 0;
        SSSI_CHECK_CUDA(cudaGetDevice(&dev));
        SSSI_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        grid_ = std::max(1, std::min(p_.ntiles, sms * 4));
        // the velocity updates' coefficients, once
        T* k[4];
        for (int c = 0; c < 4; ++c) {
            K_[c].allocate(cells * sizeof(T));
            k[c] = K_[c].template as<T>() + org_;
        }
        p_.kzp = k[0];
        p_.kxs = k[1];
        p_.kxp = k[2];
        p_.kzs = k[3];
        if constexpr (std::is_same<T, float>::value)
            el_coef_kernel<T, SSSI_MODE_FP32><<<sms * 4, 256, 0, s>>>(p_, k[0], k[1], k[2], k[3]);
        else if (mode == SSSI_MODE_FP64_STRICT)
            el_coef_kernel<T, SSSI_MODE_FP64_STRICT><<<sms * 4, 256, 0, s>>>(p_, k[0], k[1], k[2], k[3]);
        else
            el_coef_kernel<T, SSSI_MODE_FP64><<<sms * 4, 256, 0, s>>>(p_, k[0], k[1], k[2], k[3]);
        count_launch();
        SSSI_CHECK_CUDA(cudaGetLastError());
        set_hooks(ElHooks<T>{});
    }
    ~Elastic2d() {
        if (graph_) cudaGraphExecDestroy(graph_);
    }
    ElParams<T>& params() { return p_; }
    void set_hooks(const ElHooks<T>& h) {
        SSSI_CHECK_CUDA(cudaMemcpyAsync(hooks_dev_.get(), &h, sizeof(h), cudaMemcpyHostToDevice, s_));
        SSSI_CHECK_CUDA(cudaStreamSynchronize(s_));
    }
    void run(int nsteps) {
        int q = 0;
        int* base = ctr_.template as<int>();
        if (nsteps >= kElGraphSteps) {
            if (!graph_) {
                std::lock_guard<std::mutex> lock(capture_mutex());
                cudaStream_t cs = capture_stream();
                cudaGraph_t g = nullptr;
                SSSI_CHECK_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
                try {
                    for (int k = 0; k < kElGraphSteps; ++k) launch(k, cs);
                    launch_add_int(base, kElGraphSteps, cs);
                } catch (...) {
                    cudaStreamEndCapture(cs, &g);
                    if (g) cudaGraphDestroy(g);
                    throw;
                }
                count_launch(-2 * kElGraphSteps);  // recorded, not run
                cudaError_t e = cudaStreamEndCapture(cs, &g);
                if (e == cudaSuccess) e = cudaGraphInstantiate(&graph_, g, 0);
                if (g) cudaGraphDestroy(g);
                if (e != cudaSuccess) graph_ = nullptr;
                SSSI_CHECK_CUDA(e);
            }
            launch_store_int(base, step_, s_);
            count_launch();
            for (; q + kElGraphSteps <= nsteps; q += kElGraphSteps) {
                SSSI_CHECK_CUDA(cudaGraphLaunch(graph_, s_));
                count_launch(2 * kElGraphSteps + 1);
            }
        }
        if (q < nsteps) {
            launch_store_int(base, step_ + q, s_);
            count_launch();
            for (int k = 0; q + k < nsteps; ++k) launch(k, s_);
        }
        step_ += nsteps;
    }

  private:
    void launch(int offset, cudaStream_t s) {
        ElParams<T> p = p_;
        p.step_offset = offset;
        el_launch_step_n<T>(N_, p, mode_, grid_, s);
    }
    int N_, mode_;
    cudaStream_t s_;
    int64_t ldp_ = 0, org_ = 0;
    DeviceBuffer F_[12], V2_[2], K_[4], band_[6], hooks_dev_, ctr_;
    ElParams<T> p_{};
    int grid_ = 1, step_ = 0;
    cudaGraphExec_t graph_ = nullptr;
};

void check_elastic(int64_t nz, int64_t nx, int64_t nt, int N, int nB, double dz, double dx, double dt, int mode) {
    SSSI_REQUIRE(nz > 0 && nx > 0 && nt >= 0, SSSI_ERR_ARG, "bad sizes nz=%lld nx=%lld nt=%lld", (long long)nz,
                 (long long)nx, (long long)nt);
    SSSI_REQUIRE(nz < (1 << 30) && nx < (1 << 30) && nt < (1 << 30) && nz * nx < (int64_t(1) << 40), SSSI_ERR_ARG,
                 "grid too large");
    SSSI_REQUIRE(N >= 1 && N <= kElMaxOrder, SSSI_ERR_ARG, "nDiffOrder must be in 1..%d (got %d)", kElMaxOrder, N);
    SSSI_REQUIRE(nB >= 0 && 2 * (int64_t)nB <= nx && nB <= nz, SSSI_ERR_ARG,
                 "nBoundary must be in 0..min(nz, nx/2) (got %d): the side bands may not overlap", nB);
    SSSI_REQUIRE(dz > 0 && dx > 0 && dt > 0, SSSI_ERR_ARG, "dz, dx, dt must be positive");
    SSSI_REQUIRE(mode == SSSI_MODE_FP64_STRICT || mode == SSSI_MODE_FP64 || mode == SSSI_MODE_FP32, SSSI_ERR_ARG,
                 "unknown mode %d", mode);
}

template <typename T>
void elastic_fwd(const double* vp, const double* vs, const double* source, int64_t nz, int64_t nx, int64_t nt, int N,
                 int nB, double dz, double dx, double dt, int mode, int nsrc, const int64_t* src_iz,
                 const int64_t* src_ix, const double* wavelets, double* snaps[4]) {
    cudaStream_t s = current_stream();
    const int64_t n = nz * nx;
    std::vector<double> vph = host_copy(vp, (size_t)n, s);
    DeviceView dvp(vp, (size_t)n, true, s), dvs(vs, (size_t)n, true, s);
    Elastic2d<T> E(vph.data(), dvp.ptr, dvs.ptr, nz, nx, nt, N, nB, dz, dx, dt, mode, s);
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
        E.params().nsrc = nsrc;
        E.params().src_iz = d_iz.template as<int>();
        E.params().src_ix = d_ix.template as<int>();
        E.params().wavelets = wav.ptr;
    }
    bool any_snap = false;
    for (int k = 0; k < 4; ++k) any_snap |= snaps[k] != nullptr;
    const int64_t K = (source || any_snap) ? chunk_steps(nt, n) : std::max<int64_t>(nt, 1);
    SliceStream<T> src(const_cast<double*>(source), n, K);
    SliceStream<T> sn0(snaps[0], n, K), sn1(snaps[1], n, K), sn2(snaps[2], n, K), sn3(snaps[3], n, K);
    SliceStream<T>* sn[4] = {&sn0, &sn1, &sn2, &sn3};
    timing_begin(s);
    for (int64_t t0 = 0; t0 < nt; t0 += K) {
        const int64_t kk = std::min(K, nt - t0);
        src.load(t0, kk, s);
        ElHooks<T> h{};
        h.src_dense = source ? src.slice(t0, t0) : nullptr;
        h.dense_t0 = (int)t0;
        for (int k = 0; k < 4; ++k) h.snap[k] = snaps[k] ? sn[k]->slice(t0, t0) : nullptr;
        h.snap_t0 = (int)t0;
        E.set_hooks(h);
        E.run((int)kk);
        for (int k = 0; k < 4; ++k) sn[k]->store(t0, kk, s);
    }
    timing_end(s);
    SSSI_CHECK_CUDA(cudaStreamSynchronize(s));
}

}  // namespace
}  // namespace sssi

using namespace sssi;

extern "C" {

int sssi_fwdTimeSpmlFor2dEw(const double* vp, const double* vs, const double* source, int64_t nz, int64_t nx,
                            int64_t nt, int nDiffOrder, int nBoundary, double dz, double dx, double dt,
                            double* snapshotVzp, double* snapshotVxp, double* snapshotVzs, double* snapshotVxs,
                            int mode) {
    return guarded([&] {
        check_elastic(nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, mode);
        SSSI_REQUIRE(vp && vs && source, SSSI_ERR_ARG, "vp, vs and source are required");
        ensure_device();
        if (nt == 0) return;
        double* snaps[4] = {snapshotVzp, snapshotVxp, snapshotVzs, snapshotVxs};
        if (mode == SSSI_MODE_FP32)
            elastic_fwd<float>(vp, vs, source, nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, mode, 0, nullptr,
                               nullptr, nullptr, snaps);
        else
            elastic_fwd<double>(vp, vs, source, nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, mode, 0, nullptr,
                                nullptr, nullptr, snaps);
    });
}

int sssi_fwdTimeSpmlFor2dEwPoint(const double* vp, const double* vs, int64_t nz, int64_t nx, int64_t nt,
                                 int nDiffOrder, int nBoundary, double dz, double dx, double dt, int nsrc,
                                 const int64_t* src_iz, const int64_t* src_ix, const double* wavelets,
                                 double* snapshotVzp, double* snapshotVxp, double* snapshotVzs, double* snapshotVxs,
                                 int mode) {
    return guarded([&] {
        check_elastic(nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, mode);
        SSSI_REQUIRE(vp && vs, SSSI_ERR_ARG, "vp and vs are required");
        SSSI_REQUIRE(nsrc >= 0 && nsrc <= 64, SSSI_ERR_ARG, "nsrc must be in 0..64 (got %d)", nsrc);
        SSSI_REQUIRE(nsrc == 0 || (src_iz && src_ix && wavelets), SSSI_ERR_ARG,
                     "point sources need positions and wavelets");
        ensure_device();
        if (nt == 0) return;
        double* snaps[4] = {snapshotVzp, snapshotVxp, snapshotVzs, snapshotVxs};
        if (mode == SSSI_MODE_FP32)
            elastic_fwd<float>(vp, vs, nullptr, nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, mode, nsrc, src_iz,
                               src_ix, wavelets, snaps);
        else
            elastic_fwd<double>(vp, vs, nullptr, nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, mode, nsrc, src_iz,
                                src_ix, wavelets, snaps);
    });
}

}  // extern "C"
