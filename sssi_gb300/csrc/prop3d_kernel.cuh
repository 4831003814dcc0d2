// Kernel body of the 3D CPML step (included by prop3d_f32.cu / prop3d_f64.cu).
// Numerics follow fwdTimeCpmlFor3dAw.m:74-147 (z, x, y first derivatives with
// phi, second derivatives with psi, then
// P_new = (v dt)^2 (zP + xP + yP + src) + 2 P - P_old); geometry in prop3d.cuh.
#pragma once

#include <type_traits>

#include "batch2d_kernel.cuh"
#include "prop3d.cuh"

namespace sssi {
namespace p3 {

using batch::ldg_t;
using batch::mem_add;
using batch::mem_new;
// FP32 memory variables (MemVar3): phi <- b phi + (b-1) d, as the FP64 form
__device__ __forceinline__ float mem_new(float b, float bm1, float m, float d) { return fmaf(b, m, bm1 * d); }
__device__ __forceinline__ float mem_add(float d, float m) { return d + m; }

// The RZ cells of one thread's column segment: one 16-byte access.
template <typename T>
struct Col;
template <>
struct Col<float> {
    static constexpr int R = 4;
    float v[4];
};
template <>
struct Col<double> {
    static constexpr int R = 2;
    double v[2];
};
__device__ __forceinline__ Col<float> ldc(const float* p) {
    const float4 q = *reinterpret_cast<const float4*>(p);
    return {{q.x, q.y, q.z, q.w}};
}
__device__ __forceinline__ Col<double> ldc(const double* p) {
    const double2 q = *reinterpret_cast<const double2*>(p);
    return {{q.x, q.y}};
}
__device__ __forceinline__ Col<float> ldc_nc(const float* p) {
    const float4 q = __ldg(reinterpret_cast<const float4*>(p));
    return {{q.x, q.y, q.z, q.w}};
}
__device__ __forceinline__ Col<double> ldc_nc(const double* p) {
    const double2 q = __ldg(reinterpret_cast<const double2*>(p));
    return {{q.x, q.y}};
}
__device__ __forceinline__ void stc(float* p, const float* v) {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void stc(double* p, const double* v) {
    *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
}

template <typename T, int N>
struct Layout3 {
    using S = Shape3D<T>;
    static constexpr int TZ = S::TZ, TX = S::TX, RZ = S::RZ;
    static constexpr int L = 2 * N - 1;
    static constexpr int HZ = tile_halo_rows(N);
    static constexpr int SP = TZ + 2 * HZ;  // rows of a plane box (column pitch)
    static constexpr int BW = TX + 2 * L;   // columns of a plane box
    static constexpr int kStages = 3;
    static constexpr unsigned kBoxBytes = sizeof(T) * SP * BW;
    static constexpr unsigned kTileBytes = sizeof(T) * TZ * TX;
    static constexpr unsigned kO = (kBoxBytes + 127) / 128 * 128;  // P_old tile within a stage
    static constexpr unsigned kV = kO + (kTileBytes + 127) / 128 * 128;
    static constexpr unsigned kQ = kV + (kTileBytes + 127) / 128 * 128;      // P tile of plane y+2N-1
    static constexpr unsigned kPlane = kQ + (kTileBytes + 127) / 128 * 128;  // one stage
    static constexpr unsigned kTx = kBoxBytes + 3 * kTileBytes;
    static constexpr unsigned kDesc = kStages * kPlane;
    static constexpr unsigned kBar = kDesc + (sizeof(Desc3<T>) + 127) / 128 * 128;
    static constexpr unsigned kScratch = kBar + 128;
    static constexpr int RZA = TZ + 2 * N - 1;     // zA rows
    static constexpr int ZP = (RZA + 3) / 4 * 4;   // zA column pitch
    static constexpr int CXA = TX + 2 * N - 1;     // xA columns (pitch TZ)
    static constexpr unsigned kXA = (sizeof(T) * ZP * TX + 127) / 128 * 128;
    static constexpr unsigned kAq = kScratch + kXA + (sizeof(T) * TZ * CXA + 127) / 128 * 128;
    static constexpr unsigned kSmem = kAq + 16u * (2 * N) * Shape3D<T>::kThreads;  // A_y queue: 2N slots per thread
};

// Band planes: the memory variables of the same cells one plane further on are
// brought into L1 while this plane is computed (each band plane would
// otherwise wait for its own round trips to L2).
__device__ __forceinline__ void prefetch_l1(const void* p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }
constexpr unsigned kWaitLimit3 = 1u << 24;

// Stage one of a band tile for plane y (every thread of the block): zA rows
// z0-N .. z0+TZ+N-2 and xA columns x0-N .. x0+TX+N-2 of the plane, with phi
// applied inside the bands; phi is stored for the tile's own cells.
template <typename T, int N>
__device__ __noinline__ void band_plane_stage1(const Const3<T>& cc, const Desc3<T>& d, int ph, const T* Pb, int z0,
                                               int x0, int y, bool bz, bool bx, T* scratch) {
    using G = Layout3<T, N>;
    using M = typename MemVar3<T>::type;
    constexpr int TZ = G::TZ, TX = G::TX, NT = Shape3D<T>::kThreads;
    constexpr int L = G::L, HZ = G::HZ, SP = G::SP;
    const int tid = threadIdx.x;
    const int nz = d.nz, nx = d.nx, nB = d.nB;
    if (bz) {
        constexpr int CELLS = G::RZA * TX;
        constexpr int MU = (CELLS + NT - 1) / NT;
        const int zb0 = nz - nB;
        const int64_t plane = (int64_t)y * nB * nx;
        const M* phi_in = d.zphi[ph] + plane;
        M* phi_out = d.zphi[ph ^ 1] + plane;
        bool in[MU];
        T b[MU], bm[MU];
        M m[MU];
#pragma unroll
        for (int u = 0; u < MU; ++u) {
            const int idx = tid + u * NT;
            const int r = idx % G::RZA, c = idx / G::RZA;
            const int ip = z0 - N + r, j = x0 + c;
            in[u] = idx < CELLS && j < nx && ip >= zb0 && ip < nz;
            b[u] = T(0);
            bm[u] = T(0);
            m[u] = M{};
            if (in[u]) {
                const int q = (ip - zb0) + j * nB;
                b[u] = ldg_t(d.zb + q);
                bm[u] = ldg_t(d.zbm1 + q);
                m[u] = ldg_t(phi_in + q);
                if (y + 1 < d.ny) prefetch_l1(phi_in + (int64_t)nB * nx + q);
            }
        }
        T* zA = scratch;
#pragma unroll
        for (int u = 0; u < MU; ++u) {
            const int idx = tid + u * NT;
            if (idx < CELLS) {
                const int r = idx % G::RZA, c = idx / G::RZA;
                const T* col = Pb + (c + L) * SP + (r - N + HZ);
                T dd = cc.wz[0] * (col[1] - col[0]);
#pragma unroll
                for (int n = 1; n < N; ++n) dd = fma(cc.wz[n], col[1 + n] - col[-n], dd);
                if (in[u]) {
                    m[u] = mem_new(b[u], bm[u], m[u], dd);
                    dd = mem_add(dd, m[u]);
                }
                zA[c * G::ZP + r] = dd;
            }
        }
#pragma unroll
        for (int u = 0; u < MU; ++u) {
            const int idx = tid + u * NT;
            const int r = idx % G::RZA, c = idx / G::RZA;
            if (in[u] && r >= N && r < N + TZ) phi_out[(z0 - N + r - zb0) + (x0 + c) * nB] = m[u];
        }
    }
    if (bx) {
        constexpr int CELLS = TZ * G::CXA;
        constexpr int MU = (CELLS + NT - 1) / NT;
        const int64_t plane = (int64_t)y * nz * 2 * nB;
        const M* phi_in = d.xphi[ph] + plane;
        M* phi_out = d.xphi[ph ^ 1] + plane;
        int qc[MU];
        T b[MU], bm[MU];
        M m[MU];
#pragma unroll
        for (int u = 0; u < MU; ++u) {
            const int idx = tid + u * NT;
            const int r = idx % TZ, cx = idx / TZ;
            const int i = z0 + r, jc = x0 - N + cx;
            const bool band = i >= 0 && jc >= 0 && jc < nx && (jc < nB || jc >= nx - nB);
            qc[u] = (idx < CELLS && i < nz && band) ? i + (jc < nB ? jc : nB + jc - (nx - nB)) * nz : -1;
            b[u] = T(0);
            bm[u] = T(0);
            m[u] = M{};
            if (qc[u] >= 0) {
                b[u] = ldg_t(d.xb + qc[u]);
                bm[u] = ldg_t(d.xbm1 + qc[u]);
                m[u] = ldg_t(phi_in + qc[u]);
                if (y + 1 < d.ny) prefetch_l1(phi_in + (int64_t)nz * 2 * nB + qc[u]);
            }
        }
        T* xA = scratch + G::kXA / sizeof(T);
#pragma unroll
        for (int u = 0; u < MU; ++u) {
            const int idx = tid + u * NT;
            if (idx < CELLS) {
                const int r = idx % TZ, cx = idx / TZ;
                const T* row = Pb + (r + HZ) + (cx - N + L) * SP;
                T dd = cc.wx[0] * (row[SP] - row[0]);
#pragma unroll
                for (int n = 1; n < N; ++n) dd = fma(cc.wx[n], row[(1 + n) * SP] - row[-n * SP], dd);
                if (qc[u] >= 0) {
                    m[u] = mem_new(b[u], bm[u], m[u], dd);
                    dd = mem_add(dd, m[u]);
                }
                xA[cx * TZ + r] = dd;
            }
        }
#pragma unroll
        for (int u = 0; u < MU; ++u) {
            const int cx = (tid + u * NT) / TZ;
            if (qc[u] >= 0 && cx >= N && cx < N + TX) phi_out[qc[u]] = m[u];
        }
    }
}

// Band paths, out of line so the interior path keeps its registers.
// D- zA (+ psi_z) of one thread's RZ cells at plane y: zA row r0+t of the
// scratch is global row i0-N+t.
template <typename T, int N>
__device__ __forceinline__ Col<T> z_band_second(const Const3<T>& cc, const Desc3<T>& d, const T* scratch, int i0, int j,
                                             int y, int r0, int c0) {
    using G = Layout3<T, N>;
    using M = typename MemVar3<T>::type;
    constexpr int RZ = G::RZ;
    constexpr int ZW = (2 * N + RZ - 1 + RZ - 1) / RZ;
    const int nz = d.nz, nx = d.nx, nB = d.nB;
    const int zb0 = nz - nB;
    M* zpsi = d.zpsi + (int64_t)y * nB * nx;
    bool in[RZ];
    T pb[RZ], pbm[RZ];
    M ps[RZ];
#pragma unroll
    for (int o = 0; o < RZ; ++o) {
        const int i = i0 + o;
        in[o] = i >= zb0 && i < nz;
        pb[o] = T(0);
        pbm[o] = T(0);
        ps[o] = M{};
        if (in[o]) {
            const int q = (i - zb0) + j * nB;
            pb[o] = ldg_t(d.zb + q);
            pbm[o] = ldg_t(d.zbm1 + q);
            ps[o] = zpsi[q];
        }
    }
    if (y + 1 < d.ny && in[0] | in[RZ - 1]) prefetch_l1(zpsi + (int64_t)nB * nx + (max(i0, zb0) - zb0) + j * nB);
    const T* za = scratch + c0 * G::ZP + r0;
    T w[RZ * ZW];
#pragma unroll
    for (int q = 0; q < ZW; ++q) {
        const Col<T> v = ldc(za + RZ * q);
#pragma unroll
        for (int e = 0; e < RZ; ++e) w[RZ * q + e] = v.v[e];
    }
    Col<T> out;
#pragma unroll
    for (int o = 0; o < RZ; ++o) {
        T dd = cc.wz[0] * (w[o + N] - w[o + N - 1]);
#pragma unroll
        for (int k = 1; k < N; ++k) dd = fma(cc.wz[k], w[o + N + k] - w[o + N - 1 - k], dd);
        if (in[o]) {
            ps[o] = mem_new(pb[o], pbm[o], ps[o], dd);
            dd = mem_add(dd, ps[o]);
            zpsi[(i0 + o - zb0) + j * nB] = ps[o];
        }
        out.v[o] = dd;
    }
    return out;
}

// D- xA (+ psi_x): xA column c0+t of the scratch is global column j-N+t.
template <typename T, int N>
__device__ __forceinline__ Col<T> x_band_second(const Const3<T>& cc, const Desc3<T>& d, const T* scratch, int i0, int j,
                                             int y, int r0, int c0) {
    using G = Layout3<T, N>;
    using M = typename MemVar3<T>::type;
    constexpr int RZ = G::RZ, TZ = G::TZ;
    const int nz = d.nz, nx = d.nx, nB = d.nB;
    M* xpsi = d.xpsi + (int64_t)y * nz * 2 * nB;
    const int qo = (j < nB || j >= nx - nB) ? (j < nB ? j : nB + j - (nx - nB)) * nz : -1;
    T pb[RZ], pbm[RZ];
    M ps[RZ];
#pragma unroll
    for (int o = 0; o < RZ; ++o) {
        pb[o] = T(0);
        pbm[o] = T(0);
        ps[o] = M{};
        if (qo >= 0 && i0 + o < nz) {
            const int q = qo + i0 + o;
            pb[o] = ldg_t(d.xb + q);
            pbm[o] = ldg_t(d.xbm1 + q);
            ps[o] = xpsi[q];
        }
    }
    if (y + 1 < d.ny && qo >= 0 && i0 < nz) prefetch_l1(xpsi + (int64_t)nz * 2 * nB + qo + i0);
    const T* xa = scratch + G::kXA / sizeof(T) + r0;
    Col<T> a[2 * N];
#pragma unroll
    for (int t = 0; t < 2 * N; ++t) a[t] = ldc(xa + (c0 + t) * TZ);
    Col<T> out;
#pragma unroll
    for (int o = 0; o < RZ; ++o) {
        T dd = cc.wx[0] * (a[N].v[o] - a[N - 1].v[o]);
#pragma unroll
        for (int k = 1; k < N; ++k) dd = fma(cc.wx[k], a[N + k].v[o] - a[N - 1 - k].v[o], dd);
        if (qo >= 0 && i0 + o < nz) {
            ps[o] = mem_new(pb[o], pbm[o], ps[o], dd);
            dd = mem_add(dd, ps[o]);
            xpsi[qo + i0 + o] = ps[o];
        }
        out.v[o] = dd;
    }
    return out;
}

// phi_y at plane pa (a y band plane): A_y = D+ P + phi, phi stored when the
// plane belongs to this work item.
template <typename T>
__device__ __forceinline__ Col<T> y_band_first(const Desc3<T>& d, int cur, int i0, int j, int pa, bool store, Col<T> a) {
    using M = typename MemVar3<T>::type;
    constexpr int RZ = Col<T>::R;
    const int nz = d.nz, nx = d.nx, ny = d.ny, nB = d.nB;
    const int cb = pa < nB ? pa : nB + pa - (ny - nB);
    const T b = ldg_t(d.yb + j + cb * nx), bm = ldg_t(d.ybm1 + j + cb * nx);
    const int64_t q = (int64_t)i0 + (int64_t)j * nz + (int64_t)cb * nz * nx;
    const M* phi_in = d.yphi[cur] + q;
    M* phi_out = d.yphi[cur ^ 1] + q;
    M m[RZ];
#pragma unroll
    for (int o = 0; o < RZ; ++o) m[o] = i0 + o < nz ? ldg_t(phi_in + o) : M{};
    if (pa + 1 < nB || (pa + 1 >= ny - nB && pa + 1 < ny)) {
        const int cn = pa + 1 < nB ? pa + 1 : nB + pa + 1 - (ny - nB);
        prefetch_l1(d.yphi[cur] + (int64_t)i0 + (int64_t)j * nz + (int64_t)cn * nz * nx);
    }
#pragma unroll
    for (int o = 0; o < RZ; ++o) {
        if (i0 + o < nz) {
            m[o] = mem_new(b, bm, m[o], a.v[o]);
            a.v[o] = mem_add(a.v[o], m[o]);
            if (store) phi_out[o] = m[o];
        }
    }
    return a;
}

// psi_y at plane y (a y band plane): D- A_y + psi.
template <typename T>
__device__ __forceinline__ Col<T> y_band_second(const Desc3<T>& d, int i0, int j, int y, Col<T> l) {
    using M = typename MemVar3<T>::type;
    constexpr int RZ = Col<T>::R;
    const int nz = d.nz, nx = d.nx, ny = d.ny, nB = d.nB;
    const int cb = y < nB ? y : nB + y - (ny - nB);
    const T b = ldg_t(d.yb + j + cb * nx), bm = ldg_t(d.ybm1 + j + cb * nx);
    M* psi = d.ypsi + (int64_t)i0 + (int64_t)j * nz + (int64_t)cb * nz * nx;
    M p[RZ];
#pragma unroll
    for (int o = 0; o < RZ; ++o) p[o] = i0 + o < nz ? psi[o] : M{};
    if (y + 1 < nB || (y + 1 >= ny - nB && y + 1 < ny)) {
        const int cn = y + 1 < nB ? y + 1 : nB + y + 1 - (ny - nB);
        prefetch_l1(d.ypsi + (int64_t)i0 + (int64_t)j * nz + (int64_t)cn * nz * nx);
    }
#pragma unroll
    for (int o = 0; o < RZ; ++o) {
        if (i0 + o < nz) {
            p[o] = mem_new(b, bm, p[o], l.v[o]);
            psi[o] = p[o];
            l.v[o] = mem_add(l.v[o], p[o]);
        }
    }
    return l;
}

// z and x second derivatives of one thread's RZ cells at plane y (rows
// i0.., column j; r0 / c0 within the tile).
template <typename T, int N>
__device__ __forceinline__ void zx_second(const Const3<T>& cc, const Desc3<T>& d, const T* Pb, const T* scratch,
                                          bool bz, bool bx, int i0, int j, int y, int r0, int c0, T* lz, T* lx) {
    using G = Layout3<T, N>;
    constexpr int RZ = G::RZ, L = G::L, HZ = G::HZ, SP = G::SP;
    constexpr int WIN = RZ + 2 * HZ;
    if (!bz) {
        const T* col = Pb + (c0 + L) * SP + r0;
        T w[WIN];
#pragma unroll
        for (int q = 0; q < WIN / RZ; ++q) {
            const Col<T> v = ldc(col + RZ * q);
#pragma unroll
            for (int e = 0; e < RZ; ++e) w[RZ * q + e] = v.v[e];
        }
        if constexpr (batch::kPacked<T>) {
            // rows o, o+1 as one pair; offsets of even parity keep both operands in
            // aligned register pairs, odd ones stay scalar (same operations per row)
#pragma unroll
            for (int o = 0; o < RZ; o += 2) {
                float2 acc = __fmul2_rn(cc.az2[0], make_float2(w[HZ + o], w[HZ + o + 1]));
#pragma unroll
                for (int m = 1; m <= L; ++m) {
                    if (m % 2 == 0) {
                        const float2 sum = __fadd2_rn(make_float2(w[HZ + o + m], w[HZ + o + 1 + m]),
                                                      make_float2(w[HZ + o - m], w[HZ + o + 1 - m]));
                        acc = __ffma2_rn(cc.az2[m], sum, acc);
                    } else {
                        acc.x = fmaf(cc.az[m], w[HZ + o + m] + w[HZ + o - m], acc.x);
                        acc.y = fmaf(cc.az[m], w[HZ + o + 1 + m] + w[HZ + o + 1 - m], acc.y);
                    }
                }
                lz[o] = acc.x;
                lz[o + 1] = acc.y;
            }
        } else {
#pragma unroll
            for (int o = 0; o < RZ; ++o) {
                T acc = cc.az[0] * w[HZ + o];
#pragma unroll
                for (int m = 1; m <= L; ++m) acc = fma(cc.az[m], w[HZ + o + m] + w[HZ + o - m], acc);
                lz[o] = acc;
            }
        }
    } else {
        const Col<T> z = z_band_second<T, N>(cc, d, scratch, i0, j, y, r0, c0);
#pragma unroll
        for (int o = 0; o < RZ; ++o) lz[o] = z.v[o];
    }
    if (!bx) {
        const T* rowp = Pb + r0 + HZ + c0 * SP;
        if constexpr (batch::kPacked<T>) {
            float2 acc[RZ / 2];
#pragma unroll
            for (int h = 0; h < RZ / 2; ++h) acc[h] = make_float2(0.0f, 0.0f);
#pragma unroll
            for (int q = 0; q <= 2 * L; ++q) {
                const Col<T> v = ldc(rowp + q * SP);
                const float2 a = cc.ax2[q < L ? L - q : q - L];
#pragma unroll
                for (int h = 0; h < RZ / 2; ++h) acc[h] = __ffma2_rn(a, make_float2(v.v[2 * h], v.v[2 * h + 1]), acc[h]);
            }
#pragma unroll
            for (int h = 0; h < RZ / 2; ++h) {
                lx[2 * h] = acc[h].x;
                lx[2 * h + 1] = acc[h].y;
            }
        } else {
#pragma unroll
            for (int o = 0; o < RZ; ++o) lx[o] = T(0);
#pragma unroll
            for (int q = 0; q <= 2 * L; ++q) {
                const Col<T> v = ldc(rowp + q * SP);
                const T a = cc.ax[q < L ? L - q : q - L];
#pragma unroll
                for (int o = 0; o < RZ; ++o) lx[o] = fma(a, v.v[o], lx[o]);
            }
        }
    } else {
        const Col<T> x = x_band_second<T, N>(cc, d, scratch, i0, j, y, r0, c0);
#pragma unroll
        for (int o = 0; o < RZ; ++o) lx[o] = x.v[o];
    }
}

template <typename T, int N>
__global__ void __launch_bounds__(Shape3D<T>::kThreads, Shape3D<T>::kMinBlocks)
    prop3d_kernel(const Desc3<T>* __restrict__ dp, const __grid_constant__ Const3<T> cc) {
    using G = Layout3<T, N>;
    using M = typename MemVar3<T>::type;
    constexpr int TZ = G::TZ, TX = G::TX, RZ = G::RZ;
    constexpr int NS = G::kStages;
    constexpr int NQ = 2 * N;  // queue length
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + G::kBar);
    T* scratch = reinterpret_cast<T*>(smem + G::kScratch);
    const Desc3<T>& d = *reinterpret_cast<const Desc3<T>*>(smem + G::kDesc);
    const int tid = threadIdx.x;

    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    if (tid == 0) {
#pragma unroll
        for (int q = 0; q < NS; ++q) mbar_init(&bar[q], 1);
        fence_barrier_init();
    }
    {  // the descriptor is written by the host only
        constexpr int kVec = (int)(sizeof(Desc3<T>) / 16);
        const uint4* src = reinterpret_cast<const uint4*>(dp);
        uint4* dst = reinterpret_cast<uint4*>(smem + G::kDesc);
        for (int q = tid; q < kVec; q += blockDim.x) dst[q] = src[q];
    }
    __syncthreads();
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const int step = *reinterpret_cast<volatile const int*>(cc.step_base) + cc.step_offset;
    const int cur = step & 1;  // forward modelling: time index = step
    const int tau = step;
    const T* P = d.field[cur];
    T* Pnew = d.field[cur ^ 1];  // holds P_old until each thread overwrites its own cells
    const int nz = d.nz, nx = d.nx, ny = d.ny, nB = d.nB;
    const int64_t ldz = d.ldz, ldxy = d.ldxy;
    const int r0 = RZ * (tid % (TZ / RZ)), c0 = tid / (TZ / RZ);
    const int ntile = d.ntz * d.ntx;
    unsigned phase_bits = 0, inflight = 0;
    bool failed = false;

    // dynamic schedule: the first item of a block is its index, later ones come
    // from the step's counter; this step clears the counter of the next one
    // (the next step reads it only after this grid has completed)
    int* next = d.next + (step & 1);
    if (blockIdx.x == 0 && tid == 0) d.next[(step + 1) & 1] = 0;
    __shared__ int s_item;
    for (int k = blockIdx.x; k < cc.nitems && !failed;) {
        const int2 item = d.order[cc.sched][k];
        const int tile = item.x;
        const int z0 = (tile % d.ntz) * TZ - d.zs, x0 = (tile / d.ntz) * TX;
        const int y0 = item.y & 0xffff, y1 = (unsigned)item.y >> 16;
        const bool bz = nB > 0 && z0 + TZ + N - 1 > nz - nB;
        const bool bx = nB > 0 && (x0 - N < nB || x0 + TX + N - 2 >= nx - nB);
        const int i0 = z0 + r0, j = x0 + c0;
        const bool act = i0 < nz && (j | i0) >= 0 && j < nx;  // j >= 0: tests i0 >= 0 (rows above the grid)
        // per-item facts (uniform over the block): what the planes of this item
        // need beyond the stencil
        bool item_src = d.src_dense != nullptr;
        for (int q = 0; q < d.nsrc; ++q)
            item_src |= d.src_iz[q] >= z0 && d.src_iz[q] < z0 + TZ && d.src_ix[q] >= x0 && d.src_ix[q] < x0 + TX &&
                        d.src_iy[q] >= y0 && d.src_iy[q] < y1;
        const bool rec_here = d.rec != nullptr && i0 == 0;
        const bool item_snap = d.snap != nullptr;
        const bool item_yband = nB > 0 && (y0 - 2 * N < nB || y1 + 2 * N > ny - nB);
        // plane y of a field: base + y * ldxy; own column segment at i0 + j * ldz
        const int64_t own = (int64_t)i0 + (int64_t)j * ldz;

        // TMA: planes y0 .. y0+NS-2 now, plane y+NS-1 at output step y
        auto issue = [&](int y) {
            if (tid == 0 && y < y1) {
                const int s = (y - y0) % NS;
                inflight |= 1u << s;
                fence_proxy_async_shared();
                mbar_arrive_expect_tx(&bar[s], G::kTx);
                unsigned char* st = smem + s * G::kPlane;
                tma_load_3d(st, &dp->tm_plane[cur], &bar[s], z0, x0, y + G::L);
                tma_load_3d(st + G::kO, &dp->tm_tile[cur ^ 1], &bar[s], z0 + G::HZ, x0 + G::L, y + G::L);
                tma_load_3d(st + G::kV, &dp->tm_v, &bar[s], z0 + G::HZ, x0 + G::L, y + G::L);
                tma_load_3d(st + G::kQ, &dp->tm_tile[cur], &bar[s], z0 + G::HZ, x0 + G::L, y + 2 * N - 1 + G::L);
            }
        };
        __syncthreads();  // the previous item's last planes are no longer read
        for (int q = 0; q < NS - 1; ++q) issue(y0 + q);

        // Items with no band, source or snapshot work and whole tile rows and
        // columns inside the grid run a copy of the plane loop without the
        // per-plane tests for those (kLean).
        const bool lean = !bz && !bx && !item_yband && !item_src && !item_snap && z0 + TZ <= nz && x0 + TX <= nx;
        auto plane_loop = [&](auto leanc) {
            constexpr bool kLean = decltype(leanc)::value;
            // y queues.  Registers: before the shift of step s, Pq[k] = P(s-1+k)
            // (k = 0 .. 2N-1); after it Pq[k] = P(s+k).  Shared memory: A_y(p) in
            // slot (p - ys - N + 1) mod NQ of this thread, at Aq[slot * NT].
            const int ys = y0 - 2 * N + 1;
            constexpr int NT = Shape3D<T>::kThreads;
            T Pq[NQ][RZ];
            Col<T>* Aq = reinterpret_cast<Col<T>*>(smem + G::kAq) + tid;
#pragma unroll
            for (int k = 0; k < NQ; ++k)
#pragma unroll
                for (int o = 0; o < RZ; ++o) Pq[k][o] = T(0);
            // P(ys .. ys+2N-2) (planes below 0 are the zero padding); threads
            // outside the grid load nothing.  The warm-up steps (s < y0) take
            // P(s+2N-1) from global memory, loaded kAhead steps ahead (all of them
            // at once up to order 4) so that the short steps do not each wait for
            // a load: pw[k] = P(s+2N-1+k).
            constexpr int kAhead = 2 * N - 1 < 7 ? 2 * N - 1 : 7;
            Col<T> pw[kAhead] = {};
            if (act) {
#pragma unroll
                for (int k = 1; k < NQ; ++k) {
                    const Col<T> v = ldc_nc(P + own + (int64_t)(ys - 1 + k) * ldxy);
#pragma unroll
                    for (int o = 0; o < RZ; ++o) Pq[k][o] = v.v[o];
                }
#pragma unroll
                for (int k = 0; k < kAhead; ++k)
                    if (ys + k < y0) pw[k] = ldc_nc(P + own + (int64_t)(ys + NQ - 1 + k) * ldxy);
            }

            int u = 0;        // (s - ys) mod NQ
            int st_next = 0;  // ring stage of the next output plane
            // queue in P(s+2N-1), then A_y at plane s+N-1 into slot u
            auto queue_in = [&](const Col<T>& pin, int s, int u) {
                // queue in: P(s+2N-1)
#pragma unroll
                for (int k = 0; k < NQ - 1; ++k)
#pragma unroll
                    for (int o = 0; o < RZ; ++o) Pq[k][o] = Pq[k + 1][o];
#pragma unroll
                for (int o = 0; o < RZ; ++o) Pq[NQ - 1][o] = pin.v[o];
                // A_y at plane pa = s+N-1: D+ from P(s .. s+2N-1), phi_y in the y bands
                {
                    const int pa = s + N - 1;
                    T a[RZ];
                    if constexpr (batch::kPacked<T>) {
                        // x - y as fma(-1, y, x): the same rounding as the subtraction
                        const float2 m1 = make_float2(-1.0f, -1.0f);
#pragma unroll
                        for (int o = 0; o < RZ; o += 2) {
                            auto pr = [&](int k) { return make_float2(Pq[k][o], Pq[k][o + 1]); };
                            float2 dd = __fmul2_rn(cc.wy2[0], __ffma2_rn(m1, pr(N - 1), pr(N)));
#pragma unroll
                            for (int k = 1; k < N; ++k)
                                dd = __ffma2_rn(cc.wy2[k], __ffma2_rn(m1, pr(N - 1 - k), pr(N + k)), dd);
                            a[o] = dd.x;
                            a[o + 1] = dd.y;
                        }
                    } else {
#pragma unroll
                        for (int o = 0; o < RZ; ++o) {
                            T dd = cc.wy[0] * (Pq[N][o] - Pq[N - 1][o]);
#pragma unroll
                            for (int k = 1; k < N; ++k) dd = fma(cc.wy[k], Pq[N + k][o] - Pq[N - 1 - k][o], dd);
                            a[o] = dd;
                        }
                    }
                    if (!kLean && item_yband && pa >= 0 && pa < ny && (pa < nB || pa >= ny - nB) && act) {
                        Col<T> av;
#pragma unroll
                        for (int o = 0; o < RZ; ++o) av.v[o] = a[o];
                        av = y_band_first<T>(d, cur, i0, j, pa, pa >= y0 && pa < y1, av);
#pragma unroll
                        for (int o = 0; o < RZ; ++o) a[o] = av.v[o];
                    }
                    {
                        Col<T> w;
#pragma unroll
                        for (int o = 0; o < RZ; ++o) w.v[o] = a[o];
                        Aq[u * NT] = w;
                    }
                }
            };
            // warm-up: the first 2N-1 planes only fill the queues
            for (int s = ys; s < y0; ++s, u = (u + 1 == NQ) ? 0 : u + 1) {
                const Col<T> pin = pw[0];  // P(s+2N-1)
#pragma unroll
                for (int k = 0; k + 1 < kAhead; ++k) pw[k] = pw[k + 1];
                if (act && s + kAhead < y0)  // the plane of warm-up step s + kAhead
                    pw[kAhead - 1] = ldc_nc(P + own + (int64_t)(s + NQ - 1 + kAhead) * ldxy);
                queue_in(pin, s, u);
            }
            for (int s = y0; s < y1 && !failed; ++s, u = (u + 1 == NQ) ? 0 : u + 1) {
                {
                    const int st = st_next;
                    st_next = st_next + 1 == NS ? 0 : st_next + 1;
                    Col<T> pin{};  // P(s+2N-1)
                    {
                        // output plane y = s: its copies (plane box, P_old, (v dt)^2, and the
                        // own tile of P at y+2N-1) have arrived once the barrier passes
                        bool ok = true;
                        if ((inflight >> st) & 1u) ok = mbar_wait_bounded(&bar[st], (phase_bits >> st) & 1u, kWaitLimit3);
                        if (__syncthreads_or(!ok)) {
                            failed = true;
                            break;
                        }
                        phase_bits ^= 1u << st;
                        inflight &= ~(1u << st);
                        // every thread is past plane s-1: its stage takes plane s+NS-1
                        issue(s + NS - 1);
                        if (act) pin = ldc(reinterpret_cast<const T*>(smem + st * G::kPlane + G::kQ) + c0 * TZ + r0);
                    }
                    queue_in(pin, s, u);
                    const int y = s;
                    const T* Pb = reinterpret_cast<const T*>(smem + st * G::kPlane);
                    if (!kLean && (bz || bx)) {
                        band_plane_stage1<T, N>(cc, d, cur, Pb, z0, x0, y, bz, bx, scratch);
                        __syncthreads();
                    }
                    if (act) {
                        T lz[RZ], lx[RZ], ly[RZ];
                        zx_second<T, N>(cc, d, Pb, scratch, !kLean && bz, !kLean && bx, i0, j, y, r0, c0, lz, lx);
                        // D- A_y at plane y from A_y(y-N .. y+N-1) (all 2N slots, weights of
                        // queue position u), psi_y in the y bands
                        {
                            Col<T> a[NQ];
#pragma unroll
                            for (int q = 0; q < NQ; ++q) a[q] = Aq[q * NT];
                            if constexpr (batch::kPacked<T>) {
                                const float2* wq = cc.wyq2 + u * 16;
#pragma unroll
                                for (int o = 0; o < RZ; o += 2) {
                                    float2 dd = __fmul2_rn(wq[0], make_float2(a[0].v[o], a[0].v[o + 1]));
#pragma unroll
                                    for (int q = 1; q < NQ; ++q)
                                        dd = __ffma2_rn(wq[q], make_float2(a[q].v[o], a[q].v[o + 1]), dd);
                                    ly[o] = dd.x;
                                    ly[o + 1] = dd.y;
                                }
                            } else {
                                const T* wq = cc.wyq + u * 16;
#pragma unroll
                                for (int o = 0; o < RZ; ++o) {
                                    T dd = wq[0] * a[0].v[o];
#pragma unroll
                                    for (int q = 1; q < NQ; ++q) dd = fma(wq[q], a[q].v[o], dd);
                                    ly[o] = dd;
                                }
                            }
                        }
                        if (!kLean && item_yband && (y < nB || y >= ny - nB)) {
                            Col<T> lv;
#pragma unroll
                            for (int o = 0; o < RZ; ++o) lv.v[o] = ly[o];
                            lv = y_band_second<T>(d, i0, j, y, lv);
#pragma unroll
                            for (int o = 0; o < RZ; ++o) ly[o] = lv.v[o];
                        }
                        // update
                        const int64_t qi = (int64_t)i0 + (int64_t)j * nz + (int64_t)y * nz * nx;  // interior index
                        T lap[RZ], pn[RZ];
                        if constexpr (batch::kPacked<T>) {
#pragma unroll
                            for (int o = 0; o < RZ; o += 2) {
                                const float2 l = __fadd2_rn(__fadd2_rn(make_float2(lz[o], lz[o + 1]), make_float2(lx[o], lx[o + 1])),
                                                            make_float2(ly[o], ly[o + 1]));
                                lap[o] = l.x;
                                lap[o + 1] = l.y;
                            }
                        } else {
#pragma unroll
                            for (int o = 0; o < RZ; ++o) lap[o] = (lz[o] + lx[o]) + ly[o];
                        }
                        if (!kLean && item_src) {
                            if (d.src_dense) {
                                const T* sd = d.src_dense + (int64_t)(tau - d.dense_t0) * ((int64_t)nz * nx * ny) + qi;
#pragma unroll
                                for (int o = 0; o < RZ; ++o)
                                    if (i0 + o < nz) lap[o] += sd[o];
                            }
                            for (int q = 0; q < d.nsrc; ++q)
                                if (d.src_iy[q] == y && d.src_ix[q] == j && d.src_iz[q] >= i0 && d.src_iz[q] < i0 + RZ) {
#pragma unroll
                                    for (int o = 0; o < RZ; ++o)
                                        if (d.src_iz[q] == i0 + o) lap[o] += d.src_wavelet[(int64_t)q * d.nt + tau];
                                }
                        }
                        const T* pc = Pq[0];
                        const Col<T> po = ldc(reinterpret_cast<const T*>(smem + st * G::kPlane + G::kO) + c0 * TZ + r0);
                        const Col<T> vv = ldc(reinterpret_cast<const T*>(smem + st * G::kPlane + G::kV) + c0 * TZ + r0);
                        if constexpr (batch::kPacked<T>) {
#pragma unroll
                            for (int o = 0; o < RZ; o += 2) {
                                const float2 t = __ffma2_rn(make_float2(2.0f, 2.0f), make_float2(pc[o], pc[o + 1]),
                                                            make_float2(-po.v[o], -po.v[o + 1]));
                                const float2 r = __ffma2_rn(make_float2(vv.v[o], vv.v[o + 1]), make_float2(lap[o], lap[o + 1]), t);
                                pn[o] = r.x;
                                pn[o + 1] = r.y;
                            }
                        } else {
#pragma unroll
                            for (int o = 0; o < RZ; ++o) pn[o] = fma(vv.v[o], lap[o], fma(T(2), pc[o], -po.v[o]));
                        }
                        T* dst = Pnew + own + (int64_t)y * ldxy;
                        if (kLean || i0 + RZ <= nz) {
                            stc(dst, pn);
                        } else {
#pragma unroll
                            for (int o = 0; o < RZ; ++o)
                                if (i0 + o < nz) dst[o] = pn[o];
                        }
                        if (rec_here) d.rec[j + (int64_t)y * nx + (int64_t)tau * nx * ny] = pn[0];
                        if (!kLean && item_snap) {
                            T* sn = d.snap + (int64_t)(tau - d.snap_t0) * ((int64_t)nz * nx * ny) + qi;
#pragma unroll
                            for (int o = 0; o < RZ; ++o)
                                if (i0 + o < nz) sn[o] = pn[o];
                        }
                    }
                }
            }
        };
        if (lean)
            plane_loop(std::true_type{});
        else
            plane_loop(std::false_type{});
        __syncthreads();  // every thread has read s_item
        if (tid == 0) s_item = (int)gridDim.x + atomicAdd(next, 1);
        __syncthreads();
        k = s_item;
    }
    if (failed) {
        if (tid == 0) {
            atomicExch(cc.err, 1);
            for (int q = 0; q < NS; ++q)
                if ((inflight >> q) & 1u) mbar_wait_bounded(&bar[q], (phase_bits >> q) & 1u, kWaitLimit3);
        }
        __syncthreads();
    }
}

}  // namespace p3

template <typename T, int N>
void launch_prop3d_n(const Desc3<T>* d, const Const3<T>& c, int grid, cudaStream_t stream) {
    using G = p3::Layout3<T, N>;
    static bool configured = false;
    if (!configured) {
        SSSI_CHECK_CUDA(
            cudaFuncSetAttribute(p3::prop3d_kernel<T, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::kSmem));
        configured = true;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(Shape3D<T>::kThreads);
    cfg.dynamicSmemBytes = G::kSmem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    SSSI_CHECK_CUDA(cudaLaunchKernelEx(&cfg, p3::prop3d_kernel<T, N>, d, c));
    count_launch();
}

template <typename T, int N>
int prop3d_occupancy_n() {
    const size_t smem = p3::Layout3<T, N>::kSmem;
    int n = 0;
    cudaError_t e =
        cudaFuncSetAttribute(p3::prop3d_kernel<T, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, p3::prop3d_kernel<T, N>, Shape3D<T>::kThreads, smem);
    if (e != cudaSuccess || n < 1) {
        cudaGetLastError();
        n = 1;
    }
    return n;
}

#define SSSI_PROP3D_INSTANCE(T, N)                                                          \
    template void launch_prop3d_n<T, N>(const Desc3<T>*, const Const3<T>&, int, cudaStream_t); \
    template int prop3d_occupancy_n<T, N>();

}  // namespace sssi
