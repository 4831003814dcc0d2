// 3D elastic propagation with the simplified PML of src/fwdTimeSpmlFor3dEw.m:40-236
// (MATLAB only in the reference), on the device.
//
// Per step (r, s, den of each axis as in the 2D file, dampPml in cell units;
// x and z profiles from the y = 1 slice of vp, y profiles from its top row):
//   phase 1, the potentials from the velocities' staggered derivatives
//     A_x = rx A_x + sx Dx-(Vx)   A_y = ry A_y + sy Dy-(Vy)   A_z = rz A_z + sz Dz-(Vz)   A = A_x + A_y + A_z
//     B1_y = ry B1_y + sy Dy+(Vz)   B1_z = rz B1_z - sz Dz+(Vy)   B1 = B1_y + B1_z
//     B2_z = rz B2_z + sz Dz+(Vx)   B2_x = rx B2_x - sx Dx+(Vz)   B2 = B2_z + B2_x
//     B3_x = rx B3_x + sx Dx+(Vy)   B3_y = ry B3_y - sy Dy+(Vx)   B3 = B3_x + B3_y
//   phase 2, the P and S velocities from the potentials' derivatives
//     Vxp = rx Vxp + (0.25 Szy(vp^2) dt / den_x) Dx+(A) + sx src_x    (and Vyp, Vzp alike)
//     Vxs_y = ry Vxs_y - (0.25 Szy(vs^2) dt / den_y) Dy-(B3)   Vxs_z = rz Vxs_z + (... / den_z) Dz-(B2)
//     Vys_x = rx Vys_x + (0.25 Szx(vs^2) dt / den_x) Dx-(B3)   Vys_z = rz Vys_z - (... / den_z) Dz-(B1)
//     Vzs_x = rx Vzs_x - (0.25 Sxy(vs^2) dt / den_x) Dx-(B2)   Vzs_y = ry Vzs_y + (... / den_y) Dy-(B1)
//     Vxs = Vxs_y + Vxs_z, ..., Vx = Vxp + Vxs, ...
// with the 4-point sums Szy(f) = f + f(z-1) + f(z-1, y-1) + f(y-1),
// Szx(f) = f + f(x-1) + f(z-1, x-1) + f(z-1), Sxy(f) = f + f(x-1) + f(x-1, y-1) + f(y-1)
// in that order, and the derivative slices the file hands to diffOperator.
//
// GB300 form: as the 2D propagator (elastic2d.cu), with 32 x 8 block tiles on
// each y plane; the y derivatives read whole planes apart, coalesced along z.
// The six 0.25 S dt products are constant in time: FP64 forms them once per
// run and loads them (its step is bound by the FP64 pipe); FP32 forms them per
// step from the cached neighbours.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "api_util.cuh"
#include "elastic_common.cuh"
#include "sssi_internal.h"

namespace sssi {
namespace {

using namespace api;
using namespace elastic;

constexpr int kE3MaxOrder = 8;
constexpr int kE3Rows = 32, kE3Cols = 8, kE3Threads = kE3Rows * kE3Cols;
constexpr int kE3OrgRow = 32;
constexpr int kE3GraphSteps = 8;

template <typename T>
struct E3Hooks {
    const T* src[3];  // x, y, z sources: nz x nx x ny slices, slice of step t at + (t - dense_t0) * n
    T* snap[6];       // Vzp, Vxp, Vyp, Vzs, Vxs, Vys snapshots (t - snap_t0)
    int dense_t0, snap_t0;
};

// the fields: 0..6 carry a halo (their derivatives are taken), 7.. own-cell recursions
enum E3Field {
    kVx, kVy, kVz, kA, kB1, kB2, kB3,
    kAx, kAy, kAz, kB1y, kB1z, kB2z, kB2x, kB3x, kB3y,
    kVxp, kVxsy, kVxsz, kVyp, kVysx, kVysz, kVzp, kVzsx, kVzsy,
    kE3Fields
};

template <typename T>
struct E3Params {
    T* f[kE3Fields];  // padded layout, interior origin applied
    const T* vpSq;
    const T* vsSq;
    // 0.25 S dt of the six 4-point sums of vp^2 (pzy, pzx, pxy) and vs^2 (szy,
    // szx, sxy), constant in time (formed once by e3_coef_kernel), padded layout
    const T* kc[6];
    const T* xb[3];  // x band (r, s, den): nz x 2nB, pitch nz (column j < nB, or nB + j - (nx - nB))
    const T* yb[3];  // y band: nx x 2nB, pitch nx (plane k < nB, or nB + k - (ny - nB))
    const T* zb[3];  // z band: nB x nx, pitch nB (row i - (nz - nB))
    T dt;
    T c[kE3MaxOrder];
    T wz[kE3MaxOrder];
    T wx[kE3MaxOrder];
    T wy[kE3MaxOrder];
    Divisor<T> dz, dx, dy;  // strict: the spacings the terms are divided by
    int nz, nx, ny, nB, nt;
    int64_t ldp, ps;  // column pitch, plane stride
    int ntz, ntx, ntiles;
    const E3Hooks<T>* hooks;
    const int* step_base;
    int step_offset;
    int nsrc;  // point sources: cell (iz, ix, iy), component src_c (0 x, 1 y, 2 z), wavelets[k * nt + t]
    const int* src_iz;
    const int* src_ix;
    const int* src_iy;
    const int* src_c;
    const T* wavelets;
};

template <typename T>
__device__ __forceinline__ void e3_band(const T* const* b, int64_t o, T& r, T& s, T& den) {
    r = __ldg(b[0] + o);
    s = __ldg(b[1] + o);
    den = __ldg(b[2] + o);
}

template <typename T, int N, int kMode>
__global__ void __launch_bounds__(kE3Threads) elastic3d_phase1_kernel(const __grid_constant__ E3Params<T> p) {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t ldp = p.ldp, ps = p.ps;
    T c[N], wz[N], wx[N], wy[N];
#pragma unroll
    for (int k = 0; k < N; ++k) {
        c[k] = p.c[k];
        wz[k] = p.wz[k];
        wx[k] = p.wx[k];
        wy[k] = p.wy[k];
    }
    const Divisor<T> dz = p.dz, dx = p.dx, dy = p.dy;
    const T dt = p.dt;
    const int nz = p.nz, nx = p.nx, ny = p.ny, nB = p.nB;
    for (int tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x) {
        const int tz = tile % p.ntz, rest = tile / p.ntz;
        const int i = tz * kE3Rows + lane, j = (rest % p.ntx) * kE3Cols + w, k = rest / p.ntx;
        if (i >= nz || j >= nx) continue;
        const int64_t q = i + (int64_t)j * ldp + (int64_t)k * ps;
        T rx = T(1), sx = dt, dnx = T(1), ry = T(1), sy = dt, dny = T(1), rz = T(1), sz = dt, dnz = T(1);
        if (j < nB || j >= nx - nB) e3_band(p.xb, i + (int64_t)(j < nB ? j : nB + j - (nx - nB)) * nz, rx, sx, dnx);
        if (k < nB || k >= ny - nB) e3_band(p.yb, j + (int64_t)(k < nB ? k : nB + k - (ny - nB)) * nx, ry, sy, dny);
        if (i >= nz - nB) e3_band(p.zb, (i - (nz - nB)) + (int64_t)j * nB, rz, sz, dnz);
        // damped along x / y / z (r = 1 elsewhere: el_rx)
        const bool bx = j < nB || j >= nx - nB, by = k < nB || k >= ny - nB, bz = i >= nz - nB;
        const T ax = el_raxpby<T, kMode>(bx, rx, p.f[kAx][q], sx, el_diff<T, N, kMode, false>(p.f[kVx], q, ldp, c, wx, dx));
        const T ay = el_raxpby<T, kMode>(by, ry, p.f[kAy][q], sy, el_diff<T, N, kMode, false>(p.f[kVy], q, ps, c, wy, dy));
        const T az = el_raxpby<T, kMode>(bz, rz, p.f[kAz][q], sz, el_diff<T, N, kMode, false>(p.f[kVz], q, 1, c, wz, dz));
        const T b1y =
            el_raxpby<T, kMode>(by, ry, p.f[kB1y][q], sy, el_diff<T, N, kMode, true>(p.f[kVz], q, ps, c, wy, dy));
        const T b1z = el_sub<T, kMode>(el_rx<T, kMode>(bz, rz, p.f[kB1z][q]),
                                       el_mul<T, kMode>(sz, el_diff<T, N, kMode, true>(p.f[kVy], q, 1, c, wz, dz)));
        const T b2z = el_raxpby<T, kMode>(bz, rz, p.f[kB2z][q], sz, el_diff<T, N, kMode, true>(p.f[kVx], q, 1, c, wz, dz));
        const T b2x = el_sub<T, kMode>(el_rx<T, kMode>(bx, rx, p.f[kB2x][q]),
                                       el_mul<T, kMode>(sx, el_diff<T, N, kMode, true>(p.f[kVz], q, ldp, c, wx, dx)));
        const T b3x =
            el_raxpby<T, kMode>(bx, rx, p.f[kB3x][q], sx, el_diff<T, N, kMode, true>(p.f[kVy], q, ldp, c, wx, dx));
        const T b3y = el_sub<T, kMode>(el_rx<T, kMode>(by, ry, p.f[kB3y][q]),
                                       el_mul<T, kMode>(sy, el_diff<T, N, kMode, true>(p.f[kVx], q, ps, c, wy, dy)));
        p.f[kAx][q] = ax;
        p.f[kAy][q] = ay;
        p.f[kAz][q] = az;
        p.f[kB1y][q] = b1y;
        p.f[kB1z][q] = b1z;
        p.f[kB2z][q] = b2z;
        p.f[kB2x][q] = b2x;
        p.f[kB3x][q] = b3x;
        p.f[kB3y][q] = b3y;
        p.f[kA][q] = el_add<T, kMode>(el_add<T, kMode>(ax, ay), az);
        p.f[kB1][q] = el_add<T, kMode>(b1y, b1z);
        p.f[kB2][q] = el_add<T, kMode>(b2z, b2x);
        p.f[kB3][q] = el_add<T, kMode>(b3x, b3y);
    }
}

// ((f(q) + f(q + o1)) + f(q + o2)) + f(q + o3): the file's 4-point sums
template <typename T, int kMode>
__device__ __forceinline__ T e3_sum4(const T* __restrict__ f, int64_t q, int64_t o1, int64_t o2, int64_t o3) {
    return el_add<T, kMode>(el_add<T, kMode>(el_add<T, kMode>(__ldg(f + q), __ldg(f + q + o1)), __ldg(f + q + o2)),
                            __ldg(f + q + o3));
}

// (0.25 S dt) / den, the division skipped where den == 1 (exact there)
template <typename T, int kMode>
__device__ __forceinline__ T e3_k(T num, T den) {
    return den != T(1) ? el_div<T, kMode>(num, den) : num;
}

template <typename T, int N, int kMode>
__global__ void __launch_bounds__(kE3Threads) elastic3d_phase2_kernel(const __grid_constant__ E3Params<T> p) {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const int t = *reinterpret_cast<volatile const int*>(p.step_base) + p.step_offset;
    const E3Hooks<T> h = *p.hooks;
    const int64_t n = (int64_t)p.nz * p.nx * p.ny;
    const T* src[3];
    T* snap[6];
#pragma unroll
    for (int s = 0; s < 3; ++s) src[s] = h.src[s] ? h.src[s] + (int64_t)(t - h.dense_t0) * n : nullptr;
#pragma unroll
    for (int s = 0; s < 6; ++s) snap[s] = h.snap[s] ? h.snap[s] + (int64_t)(t - h.snap_t0) * n : nullptr;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t ldp = p.ldp, ps = p.ps;
    T c[N], wz[N], wx[N], wy[N];
#pragma unroll
    for (int k = 0; k < N; ++k) {
        c[k] = p.c[k];
        wz[k] = p.wz[k];
        wx[k] = p.wx[k];
        wy[k] = p.wy[k];
    }
    const Divisor<T> dz = p.dz, dx = p.dx, dy = p.dy;
    const T dt = p.dt;
    const int nz = p.nz, nx = p.nx, ny = p.ny, nB = p.nB;
    for (int tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x) {
        const int tz = tile % p.ntz, rest = tile / p.ntz;
        const int i = tz * kE3Rows + lane, j = (rest % p.ntx) * kE3Cols + w, k = rest / p.ntx;
        if (i >= nz || j >= nx) continue;
        const int64_t q = i + (int64_t)j * ldp + (int64_t)k * ps;
        T rx = T(1), sx = dt, dnx = T(1), ry = T(1), sy = dt, dny = T(1), rz = T(1), sz = dt, dnz = T(1);
        if (j < nB || j >= nx - nB) e3_band(p.xb, i + (int64_t)(j < nB ? j : nB + j - (nx - nB)) * nz, rx, sx, dnx);
        if (k < nB || k >= ny - nB) e3_band(p.yb, j + (int64_t)(k < nB ? k : nB + k - (ny - nB)) * nx, ry, sy, dny);
        if (i >= nz - nB) e3_band(p.zb, (i - (nz - nB)) + (int64_t)j * nB, rz, sz, dnz);
        // 0.25 * S * dt of each pair of sums (the division by den follows per use):
        // formed once per run in FP64, where the step is bound by the FP64 pipe;
        // from the cached neighbours in FP32, where six more streams cost more
        T pzy, pzx, pxy, szy, szx, sxy;
        if constexpr (kMode == SSSI_MODE_FP32) {
            const T q4 = T(0.25);
            pzy = el_mul<T, kMode>(el_mul<T, kMode>(q4, e3_sum4<T, kMode>(p.vpSq, q, -1, -1 - ps, -ps)), dt);
            pzx = el_mul<T, kMode>(el_mul<T, kMode>(q4, e3_sum4<T, kMode>(p.vpSq, q, -ldp, -1 - ldp, -1)), dt);
            pxy = el_mul<T, kMode>(el_mul<T, kMode>(q4, e3_sum4<T, kMode>(p.vpSq, q, -ldp, -ldp - ps, -ps)), dt);
            szy = el_mul<T, kMode>(el_mul<T, kMode>(q4, e3_sum4<T, kMode>(p.vsSq, q, -1, -1 - ps, -ps)), dt);
            szx = el_mul<T, kMode>(el_mul<T, kMode>(q4, e3_sum4<T, kMode>(p.vsSq, q, -ldp, -1 - ldp, -1)), dt);
            sxy = el_mul<T, kMode>(el_mul<T, kMode>(q4, e3_sum4<T, kMode>(p.vsSq, q, -ldp, -ldp - ps, -ps)), dt);
        } else {
            pzy = __ldg(p.kc[0] + q);
            pzx = __ldg(p.kc[1] + q);
            pxy = __ldg(p.kc[2] + q);
            szy = __ldg(p.kc[3] + q);
            szx = __ldg(p.kc[4] + q);
            sxy = __ldg(p.kc[5] + q);
        }
        const bool bx = j < nB || j >= nx - nB, by = k < nB || k >= ny - nB, bz = i >= nz - nB;
        // injected values of the cell at step t
        T sv[3] = {T(0), T(0), T(0)};
        bool hs[3] = {false, false, false};
#pragma unroll
        for (int s = 0; s < 3; ++s)
            if (src[s]) {
                sv[s] = src[s][i + (int64_t)j * nz + (int64_t)k * nz * nx];
                hs[s] = true;
            }
        for (int m = 0; m < p.nsrc; ++m)
            if (p.src_iz[m] == i && p.src_ix[m] == j && p.src_iy[m] == k) {
                const int s = p.src_c[m];
                const T wv = p.wavelets[(int64_t)m * p.nt + t];
                for (int u = 0; u < 3; ++u)
                    if (u == s) {
                        sv[u] = hs[u] ? sv[u] + wv : wv;
                        hs[u] = true;
                    }
            }
        T vxp = el_raxpby<T, kMode>(bx, rx, p.f[kVxp][q], e3_k<T, kMode>(pzy, dnx),
                                    el_diff<T, N, kMode, true>(p.f[kA], q, ldp, c, wx, dx));
        T vyp = el_raxpby<T, kMode>(by, ry, p.f[kVyp][q], e3_k<T, kMode>(pzx, dny),
                                    el_diff<T, N, kMode, true>(p.f[kA], q, ps, c, wy, dy));
        T vzp = el_raxpby<T, kMode>(bz, rz, p.f[kVzp][q], e3_k<T, kMode>(pxy, dnz),
                                    el_diff<T, N, kMode, true>(p.f[kA], q, 1, c, wz, dz));
        if (hs[0]) vxp = el_add<T, kMode>(vxp, el_mul<T, kMode>(sx, sv[0]));
        if (hs[1]) vyp = el_add<T, kMode>(vyp, el_mul<T, kMode>(sy, sv[1]));
        if (hs[2]) vzp = el_add<T, kMode>(vzp, el_mul<T, kMode>(sz, sv[2]));
        const T vxsy = el_sub<T, kMode>(
            el_rx<T, kMode>(by, ry, p.f[kVxsy][q]),
            el_mul<T, kMode>(e3_k<T, kMode>(szy, dny), el_diff<T, N, kMode, false>(p.f[kB3], q, ps, c, wy, dy)));
        const T vxsz = el_raxpby<T, kMode>(bz, rz, p.f[kVxsz][q], e3_k<T, kMode>(szy, dnz),
                                          el_diff<T, N, kMode, false>(p.f[kB2], q, 1, c, wz, dz));
        const T vysx = el_raxpby<T, kMode>(bx, rx, p.f[kVysx][q], e3_k<T, kMode>(szx, dnx),
                                          el_diff<T, N, kMode, false>(p.f[kB3], q, ldp, c, wx, dx));
        const T vysz = el_sub<T, kMode>(
            el_rx<T, kMode>(bz, rz, p.f[kVysz][q]),
            el_mul<T, kMode>(e3_k<T, kMode>(szx, dnz), el_diff<T, N, kMode, false>(p.f[kB1], q, 1, c, wz, dz)));
        const T vzsx = el_sub<T, kMode>(
            el_rx<T, kMode>(bx, rx, p.f[kVzsx][q]),
            el_mul<T, kMode>(e3_k<T, kMode>(sxy, dnx), el_diff<T, N, kMode, false>(p.f[kB2], q, ldp, c, wx, dx)));
        const T vzsy = el_raxpby<T, kMode>(by, ry, p.f[kVzsy][q], e3_k<T, kMode>(sxy, dny),
                                          el_diff<T, N, kMode, false>(p.f[kB1], q, ps, c, wy, dy));
        const T vxs = el_add<T, kMode>(vxsy, vxsz), vys = el_add<T, kMode>(vysx, vysz);
        const T vzs = el_add<T, kMode>(vzsx, vzsy);
        p.f[kVxp][q] = vxp;
        p.f[kVyp][q] = vyp;
        p.f[kVzp][q] = vzp;
        p.f[kVxsy][q] = vxsy;
        p.f[kVxsz][q] = vxsz;
        p.f[kVysx][q] = vysx;
        p.f[kVysz][q] = vysz;
        p.f[kVzsx][q] = vzsx;
        p.f[kVzsy][q] = vzsy;
        p.f[kVx][q] = el_add<T, kMode>(vxp, vxs);
        p.f[kVy][q] = el_add<T, kMode>(vyp, vys);
        p.f[kVz][q] = el_add<T, kMode>(vzp, vzs);
        const int64_t qd = i + (int64_t)j * nz + (int64_t)k * nz * nx;
        const T outv[6] = {vzp, vxp, vyp, vzs, vxs, vys};
#pragma unroll
        for (int s = 0; s < 6; ++s)
            if (snap[s]) snap[s][qd] = outv[s];
    }
}

template <typename T>
void e3_launch(void (*kernel)(E3Params<T>), const E3Params<T>& p, int grid, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kE3Threads);
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
void e3_launch_step(const E3Params<T>& p, int mode, int grid, cudaStream_t s) {
    if constexpr (std::is_same<T, float>::value) {
        e3_launch<T>(elastic3d_phase1_kernel<T, N, SSSI_MODE_FP32>, p, grid, s);
        e3_launch<T>(elastic3d_phase2_kernel<T, N, SSSI_MODE_FP32>, p, grid, s);
    } else if (mode == SSSI_MODE_FP64_STRICT) {
        e3_launch<T>(elastic3d_phase1_kernel<T, N, SSSI_MODE_FP64_STRICT>, p, grid, s);
        e3_launch<T>(elastic3d_phase2_kernel<T, N, SSSI_MODE_FP64_STRICT>, p, grid, s);
    } else {
        e3_launch<T>(elastic3d_phase1_kernel<T, N, SSSI_MODE_FP64>, p, grid, s);
        e3_launch<T>(elastic3d_phase2_kernel<T, N, SSSI_MODE_FP64>, p, grid, s);
    }
}

template <typename T>
void e3_launch_step_n(int N, const E3Params<T>& p, int mode, int grid, cudaStream_t s) {
    switch (N) {
        case 1: e3_launch_step<T, 1>(p, mode, grid, s); break;
        case 2: e3_launch_step<T, 2>(p, mode, grid, s); break;
        case 3: e3_launch_step<T, 3>(p, mode, grid, s); break;
        case 4: e3_launch_step<T, 4>(p, mode, grid, s); break;
        case 5: e3_launch_step<T, 5>(p, mode, grid, s); break;
        case 6: e3_launch_step<T, 6>(p, mode, grid, s); break;
        case 7: e3_launch_step<T, 7>(p, mode, grid, s); break;
        default: e3_launch_step<T, 8>(p, mode, grid, s); break;
    }
}

// vp.^2, vs.^2 padded by nDiffOrder in all three dimensions by edge replication
template <typename T>
__global__ void e3_square_kernel(const double* vp, const double* vs, int nz, int nx, int ny, int N, int64_t ldp,
                                 int64_t ps, T* vp2, T* vs2) {
    const int64_t rows = nz + 2 * N, cols = nx + 2 * N, planes = ny + 2 * N, n = rows * cols * planes;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const int ip = (int)(q % rows) - N, jp = (int)((q / rows) % cols) - N, kp = (int)(q / (rows * cols)) - N;
        const int i = min(max(ip, 0), nz - 1), j = min(max(jp, 0), nx - 1), k = min(max(kp, 0), ny - 1);
        const int64_t src = i + (int64_t)j * nz + (int64_t)k * nz * nx;
        const double a = vp[src], b = vs[src];
        const int64_t o = ip + (int64_t)jp * ldp + (int64_t)kp * ps;
        vp2[o] = (T)__dmul_rn(a, a);
        vs2[o] = (T)__dmul_rn(b, b);
    }
}

// 0.25 S dt of the six 4-point sums the velocity updates use (constant in
// time), in the step's operation order: pzy, pzx, pxy from vp^2, szy, szx, sxy
// from vs^2, over the cell and its -z/-y, -x/-z and -x/-y neighbours.
template <typename T, int kMode>
__global__ void e3_coef_kernel(const E3Params<T> p, T* k0, T* k1, T* k2, T* k3, T* k4, T* k5) {
    const int64_t n = (int64_t)p.nz * p.nx * p.ny, ldp = p.ldp, ps = p.ps;
    const T dt = p.dt, q4 = T(0.25);
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(c % p.nz);
        const int64_t r = c / p.nz;
        const int j = (int)(r % p.nx), k = (int)(r / p.nx);
        const int64_t q = i + (int64_t)j * ldp + (int64_t)k * ps;
        k0[q] = el_mul<T, kMode>(el_mul<T, kMode>(q4, e3_sum4<T, kMode>(p.vpSq, q, -1, -1 - ps, -ps)), dt);
        k1[q] = el_mul<T, kMode>(el_mul<T, kMode>(q4, e3_sum4<T, kMode>(p.vpSq, q, -ldp, -1 - ldp, -1)), dt);
        k2[q] = el_mul<T, kMode>(el_mul<T, kMode>(q4, e3_sum4<T, kMode>(p.vpSq, q, -ldp, -ldp - ps, -ps)), dt);
        k3[q] = el_mul<T, kMode>(el_mul<T, kMode>(q4, e3_sum4<T, kMode>(p.vsSq, q, -1, -1 - ps, -ps)), dt);
        k4[q] = el_mul<T, kMode>(el_mul<T, kMode>(q4, e3_sum4<T, kMode>(p.vsSq, q, -ldp, -1 - ldp, -1)), dt);
        k5[q] = el_mul<T, kMode>(el_mul<T, kMode>(q4, e3_sum4<T, kMode>(p.vsSq, q, -ldp, -ldp - ps, -ps)), dt);
    }
}

template <typename T>
class Elastic3d {
  public:
    // vp: host copy (nz x nx x ny doubles); dvp, dvs: device copies
    Elastic3d(const double* vp, const double* dvp, const double* dvs, int64_t nz, int64_t nx, int64_t ny, int64_t nt,
              int N, int nB, double dz, double dx, double dy, double dt, int mode, cudaStream_t s)
        : N_(N), mode_(mode), s_(s) {
        ldp_ = (int64_t)kE3OrgRow + (nz + 31) / 32 * 32 + 32;
        ps_ = ldp_ * (nx + 2 * N);
        const size_t cells = (size_t)(ps_ * (ny + 2 * N));
        org_ = kE3OrgRow + (int64_t)N * ldp_ + (int64_t)N * ps_;
        for (auto& f : F_) {
            f.allocate(cells * sizeof(T));
            f.zero(s);
        }
        for (auto& f : V2_) {
            f.allocate(cells * sizeof(T));
            f.zero(s);
        }
        e3_square_kernel<T><<<152 * 4, 256, 0, s>>>(dvp, dvs, (int)nz, (int)nx, (int)ny, N, ldp_, ps_,
                                                    V2_[0].template as<T>() + org_, V2_[1].template as<T>() + org_);
        count_launch();
        SSSI_CHECK_CUDA(cudaGetLastError());
        // band coefficients (src/fwdTimeSpmlFor3dEw.m:57-80)
        const double L = (double)nB;
        const size_t nxb = (size_t)std::max<int64_t>(nz * 2 * nB, 1), nyb = (size_t)std::max<int64_t>(nx * 2 * nB, 1);
        const size_t nzb = (size_t)std::max<int64_t>((int64_t)nB * nx, 1);
        std::vector<T> hx[3], hy[3], hz[3];
        for (int m = 0; m < 3; ++m) {
            hx[m].assign(nxb, T(0));
            hy[m].assign(nyb, T(0));
            hz[m].assign(nzb, T(0));
        }
        auto put = [](std::vector<T>* h, size_t o, double v, double u, double L_, double dt_) {
            double r, sv, den;
            el_band(v, u, L_, dt_, r, sv, den);
            h[0][o] = (T)r;
            h[1][o] = (T)sv;
            h[2][o] = (T)den;
        };
        for (int b = 0; b < 2 * nB; ++b) {
            const int64_t j = b < nB ? b : nx - nB + (b - nB);
            const double u = b < nB ? (double)(nB - b) : (double)(b - nB + 1);
            for (int64_t i = 0; i < nz; ++i) put(hx, (size_t)(i + b * nz), vp[i + j * nz], u, L, dt);  // y = 0 slice
        }
        for (int b = 0; b < 2 * nB; ++b) {
            const int64_t k = b < nB ? b : ny - nB + (b - nB);
            const double u = b < nB ? (double)(nB - b) : (double)(b - nB + 1);
            for (int64_t j = 0; j < nx; ++j) put(hy, (size_t)(j + b * nx), vp[j * nz + k * nz * nx], u, L, dt);  // z = 0
        }
        for (int64_t j = 0; j < nx; ++j)
            for (int b = 0; b < nB; ++b) put(hz, (size_t)(b + j * nB), vp[(nz - nB + b) + j * nz], (double)(b + 1), L, dt);
        for (int m = 0; m < 3; ++m) {
            upload(bx_[m], hx[m]);
            upload(by_[m], hy[m]);
            upload(bz_[m], hz[m]);
        }
        hooks_dev_.allocate(sizeof(E3Hooks<T>));
        ctr_.allocate(sizeof(int));
        ctr_.zero(s);

        p_ = E3Params<T>{};
        for (int m = 0; m < kE3Fields; ++m) p_.f[m] = F_[m].template as<T>() + org_;
        p_.vpSq = V2_[0].template as<T>() + org_;
        p_.vsSq = V2_[1].template as<T>() + org_;
        for (int m = 0; m < 3; ++m) {
            p_.xb[m] = bx_[m].template as<T>();
            p_.yb[m] = by_[m].template as<T>();
            p_.zb[m] = bz_[m].template as<T>();
        }
        p_.dt = (T)dt;
        std::vector<double> cf(N);
        staggered_coefficients(N, cf.data());
        for (int k = 0; k < N; ++k) {
            p_.c[k] = (T)cf[k];
            p_.wz[k] = (T)(cf[k] / dz);
            p_.wx[k] = (T)(cf[k] / dx);
            p_.wy[k] = (T)(cf[k] / dy);
        }
        p_.dz = make_divisor<T>(dz);
        p_.dx = make_divisor<T>(dx);
        p_.dy = make_divisor<T>(dy);
        p_.nz = (int)nz;
        p_.nx = (int)nx;
        p_.ny = (int)ny;
        p_.nB = nB;
        p_.nt = (int)nt;
        p_.ldp = ldp_;
        p_.ps = ps_;
        p_.ntz = (int)((nz + kE3Rows - 1) / kE3Rows);
        p_.ntx = (int)((nx + kE3Cols - 1) / kE3Cols);
        const int64_t tiles = (int64_t)p_.ntz * p_.ntx * ny;
        SSSI_REQUIRE(tiles < (int64_t(1) << 31), SSSI_ERR_ARG, "grid too large");
        p_.ntiles = (int)tiles;
        p_.hooks = hooks_dev_.template as<E3Hooks<T>>();
        p_.step_base = ctr_.template as<int>();
        int dev = 0, sms = 0;
        SSSI_CHECK_CUDA(cudaGetDevice(&dev));
        SSSI_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        grid_ = std::max(1, std::min(p_.ntiles, sms * 4));
        // the velocity updates' coefficients, once (FP64; FP32 forms them per step)
        if constexpr (std::is_same<T, double>::value) {
            T* kc[6];
            for (int m = 0; m < 6; ++m) {
                K_[m].allocate(cells * sizeof(T));
                kc[m] = K_[m].template as<T>() + org_;
                p_.kc[m] = kc[m];
            }
            if (mode == SSSI_MODE_FP64_STRICT)
                e3_coef_kernel<T, SSSI_MODE_FP64_STRICT>
                    <<<sms * 4, 256, 0, s>>>(p_, kc[0], kc[1], kc[2], kc[3], kc[4], kc[5]);
            else
                e3_coef_kernel<T, SSSI_MODE_FP64><<<sms * 4, 256, 0, s>>>(p_, kc[0], kc[1], kc[2], kc[3], kc[4], kc[5]);
            count_launch();
            SSSI_CHECK_CUDA(cudaGetLastError());
        }
        set_hooks(E3Hooks<T>{});
    }
    ~Elastic3d() {
        if (graph_) cudaGraphExecDestroy(graph_);
    }
    E3Params<T>& params() { return p_; }
    void set_hooks(const E3Hooks<T>& h) {
        SSSI_CHECK_CUDA(cudaMemcpyAsync(hooks_dev_.get(), &h, sizeof(h), cudaMemcpyHostToDevice, s_));
        SSSI_CHECK_CUDA(cudaStreamSynchronize(s_));
    }
    void run(int nsteps) {
        int q = 0;
        int* base = ctr_.template as<int>();
        if (nsteps >= kE3GraphSteps) {
            if (!graph_) {
                std::lock_guard<std::mutex> lock(capture_mutex());
                cudaStream_t cs = capture_stream();
                cudaGraph_t g = nullptr;
                SSSI_CHECK_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
                try {
                    for (int k = 0; k < kE3GraphSteps; ++k) launch(k, cs);
                    launch_add_int(base, kE3GraphSteps, cs);
                } catch (...) {
                    cudaStreamEndCapture(cs, &g);
                    if (g) cudaGraphDestroy(g);
                    throw;
                }
                count_launch(-2 * kE3GraphSteps);  // recorded, not run
                cudaError_t e = cudaStreamEndCapture(cs, &g);
                if (e == cudaSuccess) e = cudaGraphInstantiate(&graph_, g, 0);
                if (g) cudaGraphDestroy(g);
                if (e != cudaSuccess) graph_ = nullptr;
                SSSI_CHECK_CUDA(e);
            }
            launch_store_int(base, step_, s_);
            count_launch();
            for (; q + kE3GraphSteps <= nsteps; q += kE3GraphSteps) {
                SSSI_CHECK_CUDA(cudaGraphLaunch(graph_, s_));
                count_launch(2 * kE3GraphSteps + 1);
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
    void upload(DeviceBuffer& d, const std::vector<T>& h) {
        d.allocate(h.size() * sizeof(T));
        SSSI_CHECK_CUDA(cudaMemcpyAsync(d.get(), h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s_));
    }
    void launch(int offset, cudaStream_t s) {
        E3Params<T> p = p_;
        p.step_offset = offset;
        e3_launch_step_n<T>(N_, p, mode_, grid_, s);
    }
    int N_, mode_;
    cudaStream_t s_;
    int64_t ldp_ = 0, ps_ = 0, org_ = 0;
    DeviceBuffer F_[kE3Fields], V2_[2], K_[6], bx_[3], by_[3], bz_[3], hooks_dev_, ctr_;
    E3Params<T> p_{};
    int grid_ = 1, step_ = 0;
    cudaGraphExec_t graph_ = nullptr;
};

void check_elastic3d(int64_t nz, int64_t nx, int64_t ny, int64_t nt, int N, int nB, double dz, double dx, double dy,
                     double dt, int mode) {
    SSSI_REQUIRE(nz > 0 && nx > 0 && ny > 0 && nt >= 0, SSSI_ERR_ARG, "bad sizes nz=%lld nx=%lld ny=%lld nt=%lld",
                 (long long)nz, (long long)nx, (long long)ny, (long long)nt);
    SSSI_REQUIRE(nz < (1 << 20) && nx < (1 << 20) && ny < (1 << 20) && nt < (1 << 30) &&
                     nz * nx * ny < (int64_t(1) << 36),
                 SSSI_ERR_ARG, "grid too large");
    SSSI_REQUIRE(N >= 1 && N <= kE3MaxOrder, SSSI_ERR_ARG, "nDiffOrder must be in 1..%d (got %d)", kE3MaxOrder, N);
    SSSI_REQUIRE(nB >= 0 && 2 * (int64_t)nB <= nx && 2 * (int64_t)nB <= ny && nB <= nz, SSSI_ERR_ARG,
                 "nBoundary must be in 0..min(nz, nx/2, ny/2) (got %d): the side bands may not overlap", nB);
    SSSI_REQUIRE(dz > 0 && dx > 0 && dy > 0 && dt > 0, SSSI_ERR_ARG, "dz, dx, dy, dt must be positive");
    SSSI_REQUIRE(mode == SSSI_MODE_FP64_STRICT || mode == SSSI_MODE_FP64 || mode == SSSI_MODE_FP32, SSSI_ERR_ARG,
                 "unknown mode %d", mode);
}

template <typename T>
void elastic3d_fwd(const double* vp, const double* vs, const double* const src_in[3], int64_t nz, int64_t nx,
                   int64_t ny, int64_t nt, int N, int nB, double dz, double dx, double dy, double dt, int mode,
                   int nsrc, const int64_t* siz, const int64_t* six, const int64_t* siy, const int* scomp,
                   const double* wavelets, double* snaps[6]) {
    cudaStream_t s = current_stream();
    const int64_t n = nz * nx * ny;
    std::vector<double> vph = host_copy(vp, (size_t)n, s);
    DeviceView dvp(vp, (size_t)n, true, s), dvs(vs, (size_t)n, true, s);
    Elastic3d<T> E(vph.data(), dvp.ptr, dvs.ptr, nz, nx, ny, nt, N, nB, dz, dx, dy, dt, mode, s);
    Staged<T> wav(wavelets, (size_t)(nsrc * nt), true, s);
    DeviceBuffer d_pos;
    if (nsrc > 0) {
        std::vector<int> hp((size_t)nsrc * 4);
        for (int k = 0; k < nsrc; ++k) {
            SSSI_REQUIRE(siz[k] >= 0 && siz[k] < nz && six[k] >= 0 && six[k] < nx && siy[k] >= 0 && siy[k] < ny &&
                             scomp[k] >= 0 && scomp[k] < 3,
                         SSSI_ERR_ARG, "point source %d at (%lld, %lld, %lld), component %d, is out of range", k,
                         (long long)siz[k], (long long)six[k], (long long)siy[k], scomp[k]);
            hp[(size_t)k] = (int)siz[k];
            hp[(size_t)(nsrc + k)] = (int)six[k];
            hp[(size_t)(2 * nsrc + k)] = (int)siy[k];
            hp[(size_t)(3 * nsrc + k)] = scomp[k];
        }
        d_pos.allocate(hp.size() * sizeof(int));
        SSSI_CHECK_CUDA(cudaMemcpyAsync(d_pos.get(), hp.data(), hp.size() * sizeof(int), cudaMemcpyHostToDevice, s));
        E3Params<T>& p = E.params();
        p.nsrc = nsrc;
        p.src_iz = d_pos.template as<int>();
        p.src_ix = d_pos.template as<int>() + nsrc;
        p.src_iy = d_pos.template as<int>() + 2 * nsrc;
        p.src_c = d_pos.template as<int>() + 3 * nsrc;
        p.wavelets = wav.ptr;
    }
    bool any = false;
    for (int k = 0; k < 3; ++k) any |= src_in[k] != nullptr;
    for (int k = 0; k < 6; ++k) any |= snaps[k] != nullptr;
    const int64_t K = any ? chunk_steps(nt, n) : std::max<int64_t>(nt, 1);
    std::vector<std::unique_ptr<SliceStream<T>>> srcs, outs;
    for (int k = 0; k < 3; ++k) srcs.emplace_back(new SliceStream<T>(const_cast<double*>(src_in[k]), n, K));
    for (int k = 0; k < 6; ++k) outs.emplace_back(new SliceStream<T>(snaps[k], n, K));
    timing_begin(s);
    for (int64_t t0 = 0; t0 < nt; t0 += K) {
        const int64_t kk = std::min(K, nt - t0);
        E3Hooks<T> h{};
        for (int k = 0; k < 3; ++k) {
            srcs[k]->load(t0, kk, s);
            h.src[k] = src_in[k] ? srcs[k]->slice(t0, t0) : nullptr;
        }
        h.dense_t0 = (int)t0;
        for (int k = 0; k < 6; ++k) h.snap[k] = snaps[k] ? outs[k]->slice(t0, t0) : nullptr;
        h.snap_t0 = (int)t0;
        E.set_hooks(h);
        E.run((int)kk);
        for (int k = 0; k < 6; ++k) outs[k]->store(t0, kk, s);
    }
    timing_end(s);
    SSSI_CHECK_CUDA(cudaStreamSynchronize(s));
}

}  // namespace
}  // namespace sssi

using namespace sssi;

extern "C" {

int sssi_fwdTimeSpmlFor3dEw(const double* vp, const double* vs, const double* source_x, const double* source_y,
                            const double* source_z, int64_t nz, int64_t nx, int64_t ny, int64_t nt, int nDiffOrder,
                            int nBoundary, double dz, double dx, double dy, double dt, double* snapshotVzp,
                            double* snapshotVxp, double* snapshotVyp, double* snapshotVzs, double* snapshotVxs,
                            double* snapshotVys, int mode) {
    return guarded([&] {
        check_elastic3d(nz, nx, ny, nt, nDiffOrder, nBoundary, dz, dx, dy, dt, mode);
        SSSI_REQUIRE(vp && vs, SSSI_ERR_ARG, "vp and vs are required");
        ensure_device();
        if (nt == 0) return;
        const double* src[3] = {source_x, source_y, source_z};
        double* snaps[6] = {snapshotVzp, snapshotVxp, snapshotVyp, snapshotVzs, snapshotVxs, snapshotVys};
        if (mode == SSSI_MODE_FP32)
            elastic3d_fwd<float>(vp, vs, src, nz, nx, ny, nt, nDiffOrder, nBoundary, dz, dx, dy, dt, mode, 0, nullptr,
                                 nullptr, nullptr, nullptr, nullptr, snaps);
        else
            elastic3d_fwd<double>(vp, vs, src, nz, nx, ny, nt, nDiffOrder, nBoundary, dz, dx, dy, dt, mode, 0,
                                  nullptr, nullptr, nullptr, nullptr, nullptr, snaps);
    });
}

int sssi_fwdTimeSpmlFor3dEwPoint(const double* vp, const double* vs, int64_t nz, int64_t nx, int64_t ny, int64_t nt,
                                 int nDiffOrder, int nBoundary, double dz, double dx, double dy, double dt, int nsrc,
                                 const int64_t* src_iz, const int64_t* src_ix, const int64_t* src_iy,
                                 const int* src_component, const double* wavelets, double* snapshotVzp,
                                 double* snapshotVxp, double* snapshotVyp, double* snapshotVzs, double* snapshotVxs,
                                 double* snapshotVys, int mode) {
    return guarded([&] {
        check_elastic3d(nz, nx, ny, nt, nDiffOrder, nBoundary, dz, dx, dy, dt, mode);
        SSSI_REQUIRE(vp && vs, SSSI_ERR_ARG, "vp and vs are required");
        SSSI_REQUIRE(nsrc >= 0 && nsrc <= 64, SSSI_ERR_ARG, "nsrc must be in 0..64 (got %d)", nsrc);
        SSSI_REQUIRE(nsrc == 0 || (src_iz && src_ix && src_iy && src_component && wavelets), SSSI_ERR_ARG,
                     "point sources need positions, components and wavelets");
        ensure_device();
        if (nt == 0) return;
        const double* src[3] = {nullptr, nullptr, nullptr};
        double* snaps[6] = {snapshotVzp, snapshotVxp, snapshotVyp, snapshotVzs, snapshotVxs, snapshotVys};
        if (mode == SSSI_MODE_FP32)
            elastic3d_fwd<float>(vp, vs, src, nz, nx, ny, nt, nDiffOrder, nBoundary, dz, dx, dy, dt, mode, nsrc,
                                 src_iz, src_ix, src_iy, src_component, wavelets, snaps);
        else
            elastic3d_fwd<double>(vp, vs, src, nz, nx, ny, nt, nDiffOrder, nBoundary, dz, dx, dy, dt, mode, nsrc,
                                  src_iz, src_ix, src_iy, src_component, wavelets, snaps);
    });
}

}  // extern "C"
