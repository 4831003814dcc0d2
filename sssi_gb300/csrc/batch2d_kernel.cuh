// Kernel body of the batched 2D CPML step (included by the per-type,
// per-order translation units batch2d_{f32,f64}_{a,b}.cu).
//
// Tile loop of one persistent CTA (see tile2d.cuh for the numerics):
//   iteration k computes the CTA's k-th work item from pipeline stage k&1
//   while the TMA copies of item k+1 land in the other stage.  Warp 0 prepares
//   an item: it stores the shot's ShotTail (prefetched into registers one
//   iteration earlier) in the stage's shared slot, works out the shot's local
//   step and time index, and (lane 0) issues the three box copies.  Items of
//   shots that are not active at this batch step are skipped without copies.
#pragma once

#include <cstddef>
#include <limits>

#include "batch2d.cuh"

namespace sssi {
namespace batch {

template <typename T>
struct V4 {
    T v[4];
};

__device__ __forceinline__ V4<float> ld4(const float* p) {
    const float4 q = *reinterpret_cast<const float4*>(p);
    return {{q.x, q.y, q.z, q.w}};
}
__device__ __forceinline__ V4<double> ld4(const double* p) {
    const double2 a = reinterpret_cast<const double2*>(p)[0];
    const double2 b = reinterpret_cast<const double2*>(p)[1];
    return {{a.x, a.y, b.x, b.y}};
}
__device__ __forceinline__ void st4(float* p, const float* v) {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void st4(double* p, const double* v) {
    reinterpret_cast<double2*>(p)[0] = make_double2(v[0], v[1]);
    reinterpret_cast<double2*>(p)[1] = make_double2(v[2], v[3]);
}

// ---- CPML memory variables ----
// FP64: phi <- b phi + (b-1) d.
__device__ __forceinline__ double mem_new(double b, double bm1, double m, double d) { return fma(b, m, bm1 * d); }
__device__ __forceinline__ double mem_add(double d, double m) { return d + m; }
// FP32, compensated: phi = hi + lo carried through the update with error-free
// products (fma residuals) and a two-sum; rounded operations use intrinsics so
// the compiler cannot fuse them.
__device__ __forceinline__ float2 mem_new(float b, float bm1, float2 m, float d) {
    const float p1 = __fmul_rn(b, m.x);
    const float e1 = fmaf(b, m.x, -p1);
    const float p2 = __fmul_rn(bm1, d);
    const float e2 = fmaf(bm1, d, -p2);
    const float s = __fadd_rn(p1, p2);
    const float bb = __fsub_rn(s, p1);
    const float e3 = __fadd_rn(__fsub_rn(p1, __fsub_rn(s, bb)), __fsub_rn(p2, bb));
    float lo = fmaf(b, m.y, __fadd_rn(__fadd_rn(e1, e2), e3));
    const float hi = __fadd_rn(s, lo);
    lo = __fsub_rn(lo, __fsub_rn(hi, s));
    return make_float2(hi, lo);
}
__device__ __forceinline__ float mem_add(float d, float2 m) { return (d + m.x) + m.y; }

// Compensated running sum (hi, lo) += x: two-sum of hi and x, error kept in lo.
__device__ __forceinline__ float2 comp_add(float2 acc, float x) {
    const float s = __fadd_rn(acc.x, x);
    const float bb = __fsub_rn(s, acc.x);
    const float e = __fadd_rn(__fsub_rn(acc.x, __fsub_rn(s, bb)), __fsub_rn(x, bb));
    return make_float2(s, __fadd_rn(acc.y, e));
}

__device__ __forceinline__ float f32(float x) { return x; }
__device__ __forceinline__ float f32(double x) { return static_cast<float>(x); }

constexpr int kNoTile = 0x7fffffff;
constexpr unsigned kHalf = 32u;  // TileInfo flag: half of a tile (its TX/2 columns at x0)

// Per-tile facts shared by the block (written by warp 0 with the ShotTail).
struct TileInfo {
    int tile;        // position in the work list (kNoTile: the CTA has no more tiles)
    int shot;        // -1: nothing to do (no tile, or the shot is inactive)
    int tloc;        // local step of the shot
    int tau;         // time index of the step
    int z0, x0;      // tile origin within the shot
    unsigned flags;  // kBandZ | kBandX | kSource | kRare | kAmax
};

// FP32 cells go through the packed two-lane instructions (fma.rn.f32x2 and
// friends) where both operands sit in aligned register pairs: each lane rounds
// exactly as the scalar instruction does, so results are unchanged and the
// instruction count of the stencil sums is about halved.
template <typename T>
constexpr bool kPacked = std::is_same<T, float>::value;

template <typename T, int RX>
struct Blk {
    T v[RX][4];
};

template <typename T>
__device__ __forceinline__ T ldg_t(const T* p) { return __ldg(p); }
__device__ __forceinline__ float2 ldg_t(const float2* p) { return __ldg(p); }

// ---- band tiles (two-stage form with the CPML memory variables) ----
// A tile whose stencil reaches a damped band in z (bz) or in x (bx) first
// computes that direction's first derivative A = D+ P (+ phi inside the band)
// once per cell, cooperatively, into shared memory: zA at rows z0-N ..
// z0+TZ+N-2 of the tile's columns, xA at columns x0-N .. x0+TX+N-2 of its
// rows.  The second derivative D- A (+ psi) then reads them back.  All global
// operands of a batch are loaded before any memory variable is stored, so a
// batch costs one round trip to L2.
template <typename T, int N, class Sh>
struct BandScratch {
    static constexpr int TZ = Sh::TZ, TX = Sh::TX;
    static constexpr int RZ = TZ + 2 * N - 1;    // zA rows
    static constexpr int ZP = (RZ + 3) / 4 * 4;  // pitch of a zA column
    static constexpr int CX = TX + 2 * N - 1;    // xA columns (pitch TZ)
    static constexpr unsigned kX = (sizeof(T) * ZP * TX + 127) / 128 * 128;  // byte offset of xA
    static constexpr unsigned kBytes = kX + (sizeof(T) * TZ * CX + 127) / 128 * 128;
};

// Stage one of a half tile, one cell per item (a half tile has too few
// four-row units to share them evenly between the threads).
template <typename T, int N, class Sh, int TX>
__device__ __noinline__ void band_stage1_cells(const BatchConst<T>& bc, const ShotTail<T>& sh, int ph, const T* Pb, int z0,
                                         int x0, bool bz, bool bx, T* scratch) {
    using S = Sh;
    using B = BandScratch<T, N, Sh>;
    using M = typename MemVar<T>::type;
    constexpr int TZ = S::TZ, NT = S::kThreads;
    constexpr int CXW = TX + 2 * N - 1;  // xA columns used (pitch TZ)
    constexpr int L = 2 * N - 1;
    constexpr int HZ = tile_halo_rows(N);
    constexpr int SP = TZ + 2 * HZ;
    const int tid = threadIdx.x;
    const int nz = sh.nz, nx = sh.nx, nB = sh.nB;
    if (bz) {
        constexpr int CELLS = B::RZ * TX;
        constexpr int MU = (CELLS + NT - 1) / NT;
        const int zb0 = nz - nB;
        const T* zb = sh.zb;
        const T* zbm1 = sh.zbm1;
        const M* phi_in = sh.zphi[ph];
        M* phi_out = sh.zphi[ph ^ 1];
        bool in[MU];
        T b[MU], bm[MU];
        M m[MU];
#pragma unroll
        for (int u = 0; u < MU; ++u) {
            const int idx = tid + u * NT;
            const int r = idx % B::RZ, c = idx / B::RZ;
            const int ip = z0 - N + r, j = x0 + c;
            in[u] = idx < CELLS && (unsigned)j < (unsigned)nx && ip >= zb0 && ip < nz;
            b[u] = T(0);
            bm[u] = T(0);
            m[u] = M{};
            if (in[u]) {
                const int64_t q = (ip - zb0) + (int64_t)j * nB;
                b[u] = ldg_t(zb + q);
                bm[u] = ldg_t(zbm1 + q);
                m[u] = ldg_t(phi_in + q);
            }
        }
        T* zA = scratch;
#pragma unroll
        for (int u = 0; u < MU; ++u) {
            const int idx = tid + u * NT;
            if (idx < CELLS) {
                const int r = idx % B::RZ, c = idx / B::RZ;
                const T* col = Pb + (c + L) * SP + (r - N + HZ);  // P at row z0-N+r
                T d = bc.wz[0] * (col[1] - col[0]);
#pragma unroll
                for (int n = 1; n < N; ++n) d = fma(bc.wz[n], col[1 + n] - col[-n], d);
                if (in[u]) {
                    m[u] = mem_new(b[u], bm[u], m[u], d);
                    d = mem_add(d, m[u]);
                }
                zA[c * B::ZP + r] = d;
            }
        }
#pragma unroll
        for (int u = 0; u < MU; ++u) {
            const int idx = tid + u * NT;
            const int r = idx % B::RZ, c = idx / B::RZ;
            if (in[u] && r >= N && r < N + TZ) phi_out[(z0 - N + r - zb0) + (int64_t)(x0 + c) * nB] = m[u];
        }
    }
    if (bx) {
        constexpr int CELLS = TZ * CXW;
        constexpr int MU = (CELLS + NT - 1) / NT;
        const T* xb = sh.xb;
        const T* xbm1 = sh.xbm1;
        const M* phi_in = sh.xphi[ph];
        M* phi_out = sh.xphi[ph ^ 1];
        int64_t qc[MU];
        T b[MU], bm[MU];
        M m[MU];
#pragma unroll
        for (int u = 0; u < MU; ++u) {
            const int idx = tid + u * NT;
            const int r = idx % TZ, cx = idx / TZ;
            const int i = z0 + r, jc = x0 - N + cx;
            const bool band = i >= 0 && jc >= 0 && jc < nx && (jc < nB || jc >= nx - nB);
            qc[u] = (idx < CELLS && i < nz && band) ? i + (int64_t)(jc < nB ? jc : nB + jc - (nx - nB)) * nz : -1;
            b[u] = T(0);
            bm[u] = T(0);
            m[u] = M{};
            if (qc[u] >= 0) {
                b[u] = ldg_t(xb + qc[u]);
                bm[u] = ldg_t(xbm1 + qc[u]);
                m[u] = ldg_t(phi_in + qc[u]);
            }
        }
        T* xA = scratch + B::kX / sizeof(T);
#pragma unroll
        for (int u = 0; u < MU; ++u) {
            const int idx = tid + u * NT;
            if (idx < CELLS) {
                const int r = idx % TZ, cx = idx / TZ;
                const T* row = Pb + (r + HZ) + (cx - N + L) * SP;  // P at column x0-N+cx
                T d = bc.wx[0] * (row[SP] - row[0]);
#pragma unroll
                for (int n = 1; n < N; ++n) d = fma(bc.wx[n], row[(1 + n) * SP] - row[-n * SP], d);
                if (qc[u] >= 0) {
                    m[u] = mem_new(b[u], bm[u], m[u], d);
                    d = mem_add(d, m[u]);
                }
                xA[cx * TZ + r] = d;
            }
        }
#pragma unroll
        for (int u = 0; u < MU; ++u) {
            const int cx = (tid + u * NT) / TZ;
            if (qc[u] >= 0 && cx >= N && cx < N + TX) phi_out[qc[u]] = m[u];
        }
    }
}

// Stage one of a band tile, run by every thread of the block; the caller
// synchronises the block before the scratch is read.  A thread's unit is four
// consecutive rows of one scratch column, read from the P box with 16-byte
// loads; the memory-variable operands of all its units are loaded first, so a
// tile costs one round trip to L2 per direction.  Per cell the arithmetic is
// that of the cell-by-cell form: D+ = sum_k w_k (P[+k+1] - P[-k]) in order of
// k, then phi and A = D+ + phi inside the band.
template <typename T, int N, class Sh, int TX>
__device__ __noinline__ void band_stage1(const BatchConst<T>& bc, const ShotTail<T>& sh, int ph, const T* Pb, int z0,
                                         int x0, bool bz, bool bx, T* scratch) {
    using S = Sh;
    using B = BandScratch<T, N, Sh>;
    using M = typename MemVar<T>::type;
    constexpr int TZ = S::TZ, NT = S::kThreads;
    constexpr int CXW = TX + 2 * N - 1;  // xA columns used (pitch TZ)
    constexpr int L = 2 * N - 1;
    constexpr int HZ = tile_halo_rows(N);
    constexpr int SP = TZ + 2 * HZ;
    const int tid = threadIdx.x;
    const int nz = sh.nz, nx = sh.nx, nB = sh.nB;
    if (bz) {
        // zA row r is global row z0-N+r, box row HZ-N+r; a unit's window is box
        // rows 4g .. 4g+HZ+3 (within the box for every g)
        constexpr int G4 = (B::RZ + 3) / 4;
        constexpr int UNITS = G4 * TX;
        constexpr int MU = (UNITS + NT - 1) / NT;
        const int zb0 = nz - nB;
        // the two phi buffers are distinct: loads of later units may move ahead of
        // the stores of earlier ones
        const T* __restrict__ zb = sh.zb;
        const T* __restrict__ zbm1 = sh.zbm1;
        const M* __restrict__ phi_in = sh.zphi[ph];
        M* __restrict__ phi_out = sh.zphi[ph ^ 1];
        T* zA = scratch;
#pragma unroll
        for (int u = 0; u < MU; ++u) {
            const int unit = tid + u * NT;
            if (unit < UNITS) {
                const int g = unit % G4, c = unit / G4, j = x0 + c;
                T b[4], bm[4];
                M m[4];
#pragma unroll
                for (int o = 0; o < 4; ++o) {
                    const int p = z0 - N + 4 * g + o;
                    b[o] = T(0);
                    bm[o] = T(0);
                    m[o] = M{};
                    if ((unsigned)j < (unsigned)nx && p >= zb0 && p < nz) {
                        const int64_t q = (p - zb0) + (int64_t)j * nB;
                        b[o] = ldg_t(zb + q);
                        bm[o] = ldg_t(zbm1 + q);
                        m[o] = ldg_t(phi_in + q);
                    }
                }
                const T* colp = Pb + (c + L) * SP + 4 * g;
                T w[HZ + 4];
#pragma unroll
                for (int q = 0; q < (HZ + 4) / 4; ++q) {
                    const V4<T> v = ld4(colp + 4 * q);
#pragma unroll
                    for (int e = 0; e < 4; ++e) w[4 * q + e] = v.v[e];
                }
                T out[4];
#pragma unroll
                for (int o = 0; o < 4; ++o) {
                    constexpr int C0 = HZ - N;  // window index of the row's own P
                    T d = bc.wz[0] * (w[C0 + o + 1] - w[C0 + o]);
#pragma unroll
                    for (int n = 1; n < N; ++n) d = fma(bc.wz[n], w[C0 + o + 1 + n] - w[C0 + o - n], d);
                    const int r = 4 * g + o, p = z0 - N + r;
                    if ((unsigned)j < (unsigned)nx && p >= zb0 && p < nz) {
                        m[o] = mem_new(b[o], bm[o], m[o], d);
                        d = mem_add(d, m[o]);
                        if (r >= N && r < N + TZ) phi_out[(p - zb0) + (int64_t)j * nB] = m[o];
                    }
                    out[o] = d;
                }
                st4(zA + c * B::ZP + 4 * g, out);
            }
        }
    }
    if (bx) {
        // xA column cx is global column x0-N+cx; its D+ reads box columns cx .. cx+2N-1
        constexpr int G4 = TZ / 4;
        constexpr int UNITS = G4 * CXW;
        constexpr int MU = (UNITS + NT - 1) / NT;
        const T* __restrict__ xb = sh.xb;
        const T* __restrict__ xbm1 = sh.xbm1;
        const M* __restrict__ phi_in = sh.xphi[ph];
        M* __restrict__ phi_out = sh.xphi[ph ^ 1];
        T* xA = scratch + B::kX / sizeof(T);
#pragma unroll
        for (int u = 0; u < MU; ++u) {
            const int unit = tid + u * NT;
            if (unit < UNITS) {
                const int g = unit % G4, cx = unit / G4;
                const int i = z0 + 4 * g, jc = x0 - N + cx;
                const bool band = i >= 0 && jc >= 0 && jc < nx && (jc < nB || jc >= nx - nB);
                const int64_t qc = band ? i + (int64_t)(jc < nB ? jc : nB + jc - (nx - nB)) * nz : -1;
                T b[4], bm[4];
                M m[4];
#pragma unroll
                for (int o = 0; o < 4; ++o) {
                    b[o] = T(0);
                    bm[o] = T(0);
                    m[o] = M{};
                    if (qc >= 0 && i + o < nz) {
                        b[o] = ldg_t(xb + qc + o);
                        bm[o] = ldg_t(xbm1 + qc + o);
                        m[o] = ldg_t(phi_in + qc + o);
                    }
                }
                V4<T> a[2 * N];
#pragma unroll
                for (int t = 0; t < 2 * N; ++t) a[t] = ld4(Pb + (cx + t) * SP + HZ + 4 * g);
                T out[4];
#pragma unroll
                for (int o = 0; o < 4; ++o) {
                    T d = bc.wx[0] * (a[N].v[o] - a[N - 1].v[o]);
#pragma unroll
                    for (int n = 1; n < N; ++n) d = fma(bc.wx[n], a[N + n].v[o] - a[N - 1 - n].v[o], d);
                    if (qc >= 0 && i + o < nz) {
                        m[o] = mem_new(b[o], bm[o], m[o], d);
                        d = mem_add(d, m[o]);
                        if (cx >= N && cx < N + TX) phi_out[qc + o] = m[o];
                    }
                    out[o] = d;
                }
                st4(xA + cx * TZ + 4 * g, out);
            }
        }
    }
}

// Stage one of a residual pair's band tile (FP32, whole tiles): the same
// units as band_stage1, for both fields of the pair at once.  P (box Pb) uses
// the shot's band coefficients and memory variables; D = Q - P (box Pd) uses
// the same coefficients b_P, b_P - 1, its own memory variables (zoff / xoff
// entries on) and the difference db = b_Q - b_P (zoff / xoff entries after
// b_P):
//     phi_D <- b_P phi_D + (b_P - 1) D+D + db (phi_Q + D+Q),
//     phi_Q = phi_P + phi_D,  D+Q = D+P + D+D  (phi before the update),
// which is phi_Q - phi_P of the two fields' own recursions written out.  The
// second model's factor is thus b_P + db exactly, wherever it multiplies, so
// Q = P + D sees no rounding of its own model that P does not share.  A_P and
// A_D go to scratch and scratch_d.
template <typename T, int N, class Sh, int TX>
__device__ __noinline__ void band_stage1_pair(const BatchConst<T>& bc, const ShotTail<T>& sh, int ph, const T* Pb,
                                              const T* Pd, int z0, int x0, bool bz, bool bx, T* scratch,
                                              T* scratch_d) {
    using S = Sh;
    using B = BandScratch<T, N, Sh>;
    using M = typename MemVar<T>::type;
    constexpr int TZ = S::TZ, NT = S::kThreads;
    constexpr int CXW = TX + 2 * N - 1;
    constexpr int L = 2 * N - 1;
    constexpr int HZ = tile_halo_rows(N);
    constexpr int SP = TZ + 2 * HZ;
    const int tid = threadIdx.x;
    const int nz = sh.nz, nx = sh.nx, nB = sh.nB;
    if (bz) {
        constexpr int G4 = (B::RZ + 3) / 4;
        constexpr int UNITS = G4 * TX;
        constexpr int MU = (UNITS + NT - 1) / NT;
        const int zb0 = nz - nB;
        const int64_t zoff = (int64_t)nB * nx;
        const T* __restrict__ zb = sh.zb;
        const T* __restrict__ zbm1 = sh.zbm1;
        const M* __restrict__ phi_in = sh.zphi[ph];
        M* __restrict__ phi_out = sh.zphi[ph ^ 1];
#pragma unroll
        for (int u = 0; u < MU; ++u) {
            const int unit = tid + u * NT;
            if (unit < UNITS) {
                const int g = unit % G4, c = unit / G4, j = x0 + c;
                T out[4], outd[4];
                const T* colp = Pb + (c + L) * SP + 4 * g;
                const T* cold = Pd + (c + L) * SP + 4 * g;
#pragma unroll
                for (int o = 0; o < 4; ++o) {
                    constexpr int C0 = HZ - N;
                    T d = bc.wz[0] * (colp[C0 + o + 1] - colp[C0 + o]);
                    T e = bc.wz[0] * (cold[C0 + o + 1] - cold[C0 + o]);
#pragma unroll
                    for (int n = 1; n < N; ++n) {
                        d = fma(bc.wz[n], colp[C0 + o + 1 + n] - colp[C0 + o - n], d);
                        e = fma(bc.wz[n], cold[C0 + o + 1 + n] - cold[C0 + o - n], e);
                    }
                    const int r = 4 * g + o, p = z0 - N + r;
                    if ((unsigned)j < (unsigned)nx && p >= zb0 && p < nz) {
                        const int64_t q = (p - zb0) + (int64_t)j * nB;
                        M m = ldg_t(phi_in + q);
                        M md = ldg_t(phi_in + zoff + q);
                        const T b = ldg_t(zb + q), bm = ldg_t(zbm1 + q);
                        const T cpl = ldg_t(zb + zoff + q) * (((m.x + m.y) + d) + ((md.x + md.y) + e));
                        m = mem_new(b, bm, m, d);
                        md = comp_add(mem_new(b, bm, md, e), cpl);
                        d = mem_add(d, m);
                        e = mem_add(e, md);
                        if (r >= N && r < N + TZ) {
                            phi_out[q] = m;
                            phi_out[zoff + q] = md;
                        }
                    }
                    out[o] = d;
                    outd[o] = e;
                }
                st4(scratch + c * B::ZP + 4 * g, out);
                st4(scratch_d + c * B::ZP + 4 * g, outd);
            }
        }
    }
    if (bx) {
        constexpr int G4 = TZ / 4;
        constexpr int UNITS = G4 * CXW;
        constexpr int MU = (UNITS + NT - 1) / NT;
        const int64_t xoff = (int64_t)nz * 2 * nB;
        const T* __restrict__ xb = sh.xb;
        const T* __restrict__ xbm1 = sh.xbm1;
        const M* __restrict__ phi_in = sh.xphi[ph];
        M* __restrict__ phi_out = sh.xphi[ph ^ 1];
        T* xA = scratch + B::kX / sizeof(T);
        T* xAd = scratch_d + B::kX / sizeof(T);
#pragma unroll
        for (int u = 0; u < MU; ++u) {
            const int unit = tid + u * NT;
            if (unit < UNITS) {
                const int g = unit % G4, cx = unit / G4;
                const int i = z0 + 4 * g, jc = x0 - N + cx;
                const bool band = i >= 0 && jc >= 0 && jc < nx && (jc < nB || jc >= nx - nB);
                const int64_t qc = band ? i + (int64_t)(jc < nB ? jc : nB + jc - (nx - nB)) * nz : -1;
                V4<T> a[2 * N], ad[2 * N];
#pragma unroll
                for (int t = 0; t < 2 * N; ++t) {
                    a[t] = ld4(Pb + (cx + t) * SP + HZ + 4 * g);
                    ad[t] = ld4(Pd + (cx + t) * SP + HZ + 4 * g);
                }
                T out[4], outd[4];
#pragma unroll
                for (int o = 0; o < 4; ++o) {
                    T d = bc.wx[0] * (a[N].v[o] - a[N - 1].v[o]);
                    T e = bc.wx[0] * (ad[N].v[o] - ad[N - 1].v[o]);
#pragma unroll
                    for (int n = 1; n < N; ++n) {
                        d = fma(bc.wx[n], a[N + n].v[o] - a[N - 1 - n].v[o], d);
                        e = fma(bc.wx[n], ad[N + n].v[o] - ad[N - 1 - n].v[o], e);
                    }
                    if (qc >= 0 && i + o < nz) {
                        const int64_t q = qc + o;
                        M m = ldg_t(phi_in + q);
                        M md = ldg_t(phi_in + xoff + q);
                        const T b = ldg_t(xb + q), bm = ldg_t(xbm1 + q);
                        const T cpl = ldg_t(xb + xoff + q) * (((m.x + m.y) + d) + ((md.x + md.y) + e));
                        m = mem_new(b, bm, m, d);
                        md = comp_add(mem_new(b, bm, md, e), cpl);
                        d = mem_add(d, m);
                        e = mem_add(e, md);
                        if (cx >= N && cx < N + TX) {
                            phi_out[q] = m;
                            phi_out[xoff + q] = md;
                        }
                    }
                    out[o] = d;
                    outd[o] = e;
                }
                st4(xA + cx * TZ + 4 * g, out);
                st4(xAd + cx * TZ + 4 * g, outd);
            }
        }
    }
}

// Optional per-step outputs other than the receiver row (dense snapshots, the
// RTM FP16 pack and max, the imaging sums).  Out of line for the same reason.
template <typename T, int RX>
__device__ __noinline__ unsigned rare_outputs(const ShotTail<T>& sh, const TileInfo& ti, int i0, int j0,
                                              Blk<T, RX> pn, Blk<T, RX> pc) {
    const int nz = sh.nz, nx = sh.nx, tau = ti.tau;
    const int64_t ncell = (int64_t)nz * nx;
    const int nrow = min(4, nz - i0);
    const int ncol = min(RX, nx - j0);
    unsigned amax_bits = 0u;
    if (sh.snap) {
        T* snap = sh.snap + (int64_t)(tau - sh.snap_t0) * ncell;
        for (int c = 0; c < ncol; ++c)
            for (int o = 0; o < nrow; ++o) snap[(i0 + o) + (int64_t)(j0 + c) * nz] = pn.v[c][o];
    }
    const int stride = sh.stride > 0 ? sh.stride : 1;
    // the thread's cells lie in one 32 x 32 scale block: i0 is a multiple of 4
    // and j0 of 2, so neither straddles a multiple of 32
    const int64_t blk = (i0 >> 5) + (int64_t)(j0 >> 5) * ((nz + 31) >> 5);
    const int64_t nblk = (int64_t)((nz + 31) >> 5) * ((nx + 31) >> 5);
    if (sh.pack && tau >= 1 && (tau - 1) % stride == 0) {
        // FP16 with error feedback: the cell's rounding error of the previous
        // stored step is added before rounding and the new one kept (FP32), so
        // the rounding errors of consecutive snapshots cancel in the imaging sum
        const int k = (tau - 1) / stride;
        const float scale = fp16_scale_from_amax(sh.amax[k * nblk + blk]);
        const float inv = 1.0f / scale;  // a power of two: exact
        __half* pack = sh.pack + (int64_t)k * ncell;
        float* perr = sh.perr;
        for (int c = 0; c < ncol; ++c) {
            const int64_t q0 = i0 + (int64_t)(j0 + c) * nz;
            if (nrow == 4 && (q0 & 3) == 0 && (ncell & 3) == 0) {  // four cells: 8- and 16-byte accesses
                float4 e = *reinterpret_cast<const float4*>(perr + q0);
                const float x[4] = {__fadd_rn(f32(pc.v[c][0]), e.x), __fadd_rn(f32(pc.v[c][1]), e.y),
                                    __fadd_rn(f32(pc.v[c][2]), e.z), __fadd_rn(f32(pc.v[c][3]), e.w)};
                __half h[4];
#pragma unroll
                for (int o = 0; o < 4; ++o) h[o] = __float2half_rn(__fmul_rn(x[o], scale));
                e = make_float4(__fsub_rn(x[0], __fmul_rn(__half2float(h[0]), inv)),
                                __fsub_rn(x[1], __fmul_rn(__half2float(h[1]), inv)),
                                __fsub_rn(x[2], __fmul_rn(__half2float(h[2]), inv)),
                                __fsub_rn(x[3], __fmul_rn(__half2float(h[3]), inv)));
                *reinterpret_cast<float4*>(perr + q0) = e;
                const __half2 lo = __halves2half2(h[0], h[1]);
                const __half2 hi = __halves2half2(h[2], h[3]);
                uint2 w;
                w.x = *reinterpret_cast<const unsigned*>(&lo);
                w.y = *reinterpret_cast<const unsigned*>(&hi);
                *reinterpret_cast<uint2*>(pack + q0) = w;
            } else {
                for (int o = 0; o < nrow; ++o) {
                    const float x = __fadd_rn(f32(pc.v[c][o]), perr[q0 + o]);
                    const __half h = __float2half_rn(__fmul_rn(x, scale));
                    perr[q0 + o] = __fsub_rn(x, __fmul_rn(__half2float(h), inv));
                    pack[q0 + o] = h;
                }
            }
        }
    }
    if (sh.amax && tau % stride == 0) {
        for (int c = 0; c < ncol; ++c)
            for (int o = 0; o < nrow; ++o) amax_bits = max(amax_bits, __float_as_uint(fabsf(f32(pn.v[c][o]))));
    }
    // illumination sum of the forward field, from the FP32 field itself
    if (sh.s2acc && tau % stride == 0) {
        float2* s2 = sh.s2acc;
        for (int c = 0; c < ncol; ++c) {
            const int64_t q0 = i0 + (int64_t)(j0 + c) * nz;
            float2 a[4];
#pragma unroll
            for (int o = 0; o < 4; ++o)
                if (o < nrow) a[o] = s2[q0 + o];
#pragma unroll
            for (int o = 0; o < 4; ++o)
                if (o < nrow) {
                    const float f = f32(pn.v[c][o]);
                    s2[q0 + o] = comp_add(a[o], __fmul_rn(f, f));
                }
        }
    }
    // Imaging: the operands of a column's cells are loaded before any of its
    // sums is stored, so those cells share one round trip to memory.
    if constexpr (std::is_same<T, double>::value) {
        if (sh.img_f64) {
            const double* f64 = sh.img_f64 + (int64_t)tau * ncell;
            double* im = sh.img_m;
            double* is2 = sh.img_s2;
#pragma unroll
            for (int c = 0; c < RX; ++c) {
                if (c >= ncol) break;
                const int64_t q0 = i0 + (int64_t)(j0 + c) * nz;
                double f[4], m[4], s2[4];
#pragma unroll
                for (int o = 0; o < 4; ++o)
                    if (o < nrow) {
                        f[o] = f64[q0 + o];
                        m[o] = im[q0 + o];
                        s2[o] = is2[q0 + o];
                    }
#pragma unroll
                for (int o = 0; o < 4; ++o)
                    if (o < nrow) {
                        im[q0 + o] = fma(f[o], pn.v[c][o], m[o]);
                        is2[q0 + o] = fma(f[o], f[o], s2[o]);
                    }
            }
        }
    }
    if (sh.img_f16 && tau % stride == 0) {
        const int k = tau / stride;
        const __half* f16 = sh.img_f16 + (int64_t)k * ncell;
        const float inv = 1.0f / fp16_scale_from_amax(sh.img_amax[k * nblk + blk]);  // a power of two
        float2* im = sh.img_m2;
        float2* is2 = sh.img_s22;
#pragma unroll
        for (int c = 0; c < RX; ++c) {
            if (c >= ncol) break;
            const int64_t q0 = i0 + (int64_t)(j0 + c) * nz;
            __half h[4];
            float2 m[4], s2[4];
            if (nrow == 4 && (q0 & 3) == 0 && (ncell & 3) == 0) {
                // a whole aligned column of four cells: 8- and 16-byte accesses
                const uint2 hv = *reinterpret_cast<const uint2*>(f16 + q0);
                const __half2 h01 = *reinterpret_cast<const __half2*>(&hv.x);
                const __half2 h23 = *reinterpret_cast<const __half2*>(&hv.y);
                h[0] = __low2half(h01);
                h[1] = __high2half(h01);
                h[2] = __low2half(h23);
                h[3] = __high2half(h23);
                const float4 ma = *reinterpret_cast<const float4*>(im + q0);
                const float4 mb = *reinterpret_cast<const float4*>(im + q0 + 2);
                const float4 sa = is2 ? *reinterpret_cast<const float4*>(is2 + q0) : make_float4(0, 0, 0, 0);
                const float4 sb = is2 ? *reinterpret_cast<const float4*>(is2 + q0 + 2) : make_float4(0, 0, 0, 0);
                m[0] = make_float2(ma.x, ma.y);
                m[1] = make_float2(ma.z, ma.w);
                m[2] = make_float2(mb.x, mb.y);
                m[3] = make_float2(mb.z, mb.w);
                s2[0] = make_float2(sa.x, sa.y);
                s2[1] = make_float2(sa.z, sa.w);
                s2[2] = make_float2(sb.x, sb.y);
                s2[3] = make_float2(sb.z, sb.w);
                float2 mn[4], sn[4];
#pragma unroll
                for (int o = 0; o < 4; ++o) {
                    const float f = __half2float(h[o]) * inv;
                    const float r = f32(pn.v[c][o]);
                    mn[o] = comp_add(m[o], __fmul_rn(f, r));
                    sn[o] = comp_add(s2[o], __fmul_rn(f, f));
                }
                *reinterpret_cast<float4*>(im + q0) = make_float4(mn[0].x, mn[0].y, mn[1].x, mn[1].y);
                *reinterpret_cast<float4*>(im + q0 + 2) = make_float4(mn[2].x, mn[2].y, mn[3].x, mn[3].y);
                if (is2) {
                    *reinterpret_cast<float4*>(is2 + q0) = make_float4(sn[0].x, sn[0].y, sn[1].x, sn[1].y);
                    *reinterpret_cast<float4*>(is2 + q0 + 2) = make_float4(sn[2].x, sn[2].y, sn[3].x, sn[3].y);
                }
                continue;
            }
#pragma unroll
            for (int o = 0; o < 4; ++o)
                if (o < nrow) {
                    h[o] = f16[q0 + o];
                    m[o] = im[q0 + o];
                    if (is2) s2[o] = is2[q0 + o];
                }
#pragma unroll
            for (int o = 0; o < 4; ++o)
                if (o < nrow) {
                    const float f = __half2float(h[o]) * inv;
                    const float r = f32(pn.v[c][o]);
                    im[q0 + o] = comp_add(m[o], __fmul_rn(f, r));
                    if (is2) is2[q0 + o] = comp_add(s2[o], __fmul_rn(f, f));
                }
        }
    }
    return amax_bits;
}

// Injected terms of column j, rows i0..i0+3, added to lap: a dense source
// slice, the surface row (row 0), point sources.  Only tiles flagged kSource.
template <typename T>
__device__ __forceinline__ void add_sources(const ShotTail<T>& sh, int tau, int i0, int j, T* lap) {
    const int nz = sh.nz, nx = sh.nx;
    const T* src_dense = sh.src_dense ? sh.src_dense + (int64_t)(tau - sh.dense_t0) * ((int64_t)nz * nx) : nullptr;
    const T* src_row = (sh.src_row && i0 == 0) ? sh.src_row + (int64_t)tau * nx : nullptr;
#pragma unroll
    for (int o = 0; o < 4; ++o) {
        const int i = i0 + o;
        T sv = T(0);
        if (src_dense && i < nz) sv = src_dense[i + (int64_t)j * nz];
        if (src_row && o == 0) sv = src_row[j];
        for (int s = 0; s < sh.nsrc; ++s)
            if (i == sh.src_iz[s] && j == sh.src_ix[s]) sv += sh.src_wavelet[(int64_t)s * sh.nt + tau];
        lap[o] += sv;
    }
}

// What the P pass of a residual pair hands to its D pass, per cell of the
// thread: P's lap with the injected terms, and psi_P + D- A_P in the z and x
// bands (psi_P before its update).
template <typename T, int RX>
struct PairIO {
    T lap[RX][4];
    T cz[RX][4];
    T cx[RX][4];
    const T* lo;      // P's low parts, current and previous field (tiles in shared memory)
    const T* lo_old;
};

// P of a residual pair is carried as hi + lo (two FP32 words): its rounding
// noise would otherwise scatter off the model difference into D.  The
// stencil reads hi only (the lo terms change lap by about an FP32 rounding);
// the update 2P - P_old + w lap is done with error-free transformations.
// Returns the new (hi, lo).
__device__ __forceinline__ float2 pair_update_hi_lo(float hi, float lo, float hi_old, float lo_old, float w,
                                                    float lap) {
    // 2 hi - hi_old exactly as s + e (2 hi is exact)
    const float a = __fmul_rn(2.0f, hi);
    const float s = __fsub_rn(a, hi_old);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(-hi_old, bb));
    // w lap exactly as p + pe
    const float p = __fmul_rn(w, lap);
    const float pe = fmaf(w, lap, -p);
    // s + p as h + e2
    const float h = __fadd_rn(s, p);
    const float b2 = __fsub_rn(h, s);
    const float e2 = __fadd_rn(__fsub_rn(s, __fsub_rn(h, b2)), __fsub_rn(p, b2));
    // the low-order terms, then renormalise
    const float l = __fadd_rn(__fadd_rn(__fadd_rn(e, pe), e2), __fsub_rn(__fmul_rn(2.0f, lo), lo_old));
    const float hn = __fadd_rn(h, l);
    return make_float2(hn, __fsub_rn(l, __fsub_rn(hn, h)));
}

// Roles of tile_cells: a single field, or the P / D pass of a residual pair.
constexpr int kRoleSingle = 0, kRolePairP = 1, kRolePairD = 2;

// All cells of one thread: rows i0..i0+3, columns j0..j0+RX-1.  kBandZ / kBandX:
// the tile is a band tile in z / x, its first derivatives are in `scratch`;
// otherwise the composed stencil is used in that direction.
//
// Residual pairs run it twice per tile: kRolePairP advances P as a single
// field (its outputs are the shot's) but carries it as hi + lo (the low part
// 2 dcol columns on) and fills `io`; kRolePairD advances D = Q - P from the D
// box (Pb), D's previous tile (Ob), P's (v dt)^2 (Vb) and the difference of
// the two models' (v dt)^2 (Vd):
//     D_new = wP lap_D + (wQ - wP) (lap_D + lap_P) + 2 D - D_old,
// with P's band coefficients, D's memory variables and the coupling terms
// db (psi_Q + D- A_Q) in the band tiles (db = b_Q - b_P, psi_Q = psi_P +
// psi_D before the update), and writes D's row 0 to rec_d.  Every factor of
// the second model is P's FP32 factor plus the exact difference, so the
// rounding of the models is shared by P and Q and cancels in D.
// kRareOut: the call to rare_outputs is compiled in (a batch without snapshots,
// FP16 packs or imaging runs a variant without it: the call's register
// saves cost the whole-tile loop about 10 %).
template <typename T, int N, class Sh, int RX, int kRole = kRoleSingle, bool kRareOut = true>
__device__ __forceinline__ void tile_cells(const BatchConst<T>& bc, const ShotTail<T>& sh, const TileInfo& ti,
                                           const T* Pb, const T* Ob, const T* Vb, int z0, int x0, int r0, int c0,
                                           unsigned flags, const T* scratch, unsigned& amax_bits,
                                           PairIO<T, RX>* io = nullptr, const T* Vd = nullptr) {
    using S = Sh;
    using B = BandScratch<T, N, Sh>;
    using M = typename MemVar<T>::type;
    constexpr int TZ = S::TZ;
    constexpr int L = 2 * N - 1;
    constexpr int HZ = tile_halo_rows(N);
    constexpr int SP = TZ + 2 * HZ;  // pitch of a P-box column
    constexpr int WIN = 4 + 2 * HZ;  // z window of one column
    const int nz = sh.nz, nx = sh.nx, nB = sh.nB;
    const int i0 = z0 + r0, j0 = x0 + c0;
    const int ph = ti.tloc & 1;
    const bool bz = flags & kBandZ, bx = flags & kBandX;

    Blk<T, RX> lz, lx, pc;

    // ---------------- z ----------------
    if (!bz) {
#pragma unroll
        for (int c = 0; c < RX; ++c) {
            const T* col = Pb + (c0 + c + L) * SP + r0;
            T w[WIN];
#pragma unroll
            for (int q = 0; q < WIN / 4; ++q) {
                const V4<T> v = ld4(col + 4 * q);
                w[4 * q] = v.v[0];
                w[4 * q + 1] = v.v[1];
                w[4 * q + 2] = v.v[2];
                w[4 * q + 3] = v.v[3];
            }
            if constexpr (kPacked<T>) {
                // rows 2h, 2h+1 as one pair: offsets m of even parity keep both operands
                // in aligned register pairs (packed instructions); odd offsets stay scalar.
                // Per row the operations and their order are those of the scalar form.
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    constexpr int b0 = HZ;
                    const int o = 2 * h;
                    pc.v[c][o] = w[b0 + o];
                    pc.v[c][o + 1] = w[b0 + o + 1];
                    float2 acc = __fmul2_rn(bc.az2[0], make_float2(w[b0 + o], w[b0 + o + 1]));
#pragma unroll
                    for (int m = 1; m <= L; ++m) {
                        if (m % 2 == 0) {
                            const float2 sum = __fadd2_rn(make_float2(w[b0 + o + m], w[b0 + o + 1 + m]),
                                                          make_float2(w[b0 + o - m], w[b0 + o + 1 - m]));
                            acc = __ffma2_rn(bc.az2[m], sum, acc);
                        } else {
                            acc.x = fmaf(bc.az[m], w[b0 + o + m] + w[b0 + o - m], acc.x);
                            acc.y = fmaf(bc.az[m], w[b0 + o + 1 + m] + w[b0 + o + 1 - m], acc.y);
                        }
                    }
                    lz.v[c][o] = acc.x;
                    lz.v[c][o + 1] = acc.y;
                }
            } else {
#pragma unroll
                for (int o = 0; o < 4; ++o) {
                    pc.v[c][o] = w[HZ + o];
                    T acc = bc.az[0] * w[HZ + o];
#pragma unroll
                    for (int m = 1; m <= L; ++m) acc = fma(bc.az[m], w[HZ + o + m] + w[HZ + o - m], acc);
                    lz.v[c][o] = acc;
                }
            }
        }
    } else {
        // D- zA (+ psi): zA row r0+t of the scratch is global row i0-N+t
        constexpr int ZW = (2 * N + 3 + 3) / 4;  // 4-vectors covering the 2N+3 rows used
        const int zb0 = nz - nB;
        // a pair's D pass uses the second model's coefficients and D's own psi,
        // zoff entries after P's; both passes read b_Q - b_P 2 zoff entries on
        const int64_t zoff = (int64_t)nB * nx;
        const T* zb = sh.zb;
        const T* zbm1 = sh.zbm1;
        M* zpsi = sh.zpsi + (kRole == kRolePairD ? zoff : 0);
        bool in[RX][4];
        T pb[RX][4], pbm[RX][4];
        T pdb[kRole == kRolePairD ? RX : 1][4];  // D pass: b_Q - b_P
        M ps[RX][4];
#pragma unroll
        for (int c = 0; c < RX; ++c)
#pragma unroll
            for (int o = 0; o < 4; ++o) {
                const int i = i0 + o, j = j0 + c;
                in[c][o] = j < nx && i >= zb0 && i < nz;
                pb[c][o] = T(0);
                pbm[c][o] = T(0);
                ps[c][o] = M{};
                if constexpr (kRole == kRolePairD) pdb[c][o] = T(0);
                if (in[c][o]) {
                    const int64_t q = (i - zb0) + (int64_t)j * nB;
                    pb[c][o] = ldg_t(zb + q);
                    pbm[c][o] = ldg_t(zbm1 + q);
                    ps[c][o] = zpsi[q];
                    if constexpr (kRole == kRolePairD) pdb[c][o] = ldg_t(zb + zoff + q);
                }
            }
#pragma unroll
        for (int c = 0; c < RX; ++c) {
            const V4<T> cen = ld4(Pb + (c0 + c + L) * SP + r0 + HZ);
            const T* za = scratch + (c0 + c) * B::ZP + r0;
            T w[4 * ZW];
#pragma unroll
            for (int q = 0; q < ZW; ++q) {
                const V4<T> v = ld4(za + 4 * q);
                w[4 * q] = v.v[0];
                w[4 * q + 1] = v.v[1];
                w[4 * q + 2] = v.v[2];
                w[4 * q + 3] = v.v[3];
            }
#pragma unroll
            for (int o = 0; o < 4; ++o) {
                pc.v[c][o] = cen.v[o];
                T d = bc.wz[0] * (w[o + N] - w[o + N - 1]);
#pragma unroll
                for (int k = 1; k < N; ++k) d = fma(bc.wz[k], w[o + N + k] - w[o + N - 1 - k], d);
                if (in[c][o]) {
                    // a pair's P pass hands over psi_P + D- A_P (psi before the update);
                    // the D pass adds db (psi_Q + D- A_Q) to D's recursion
                    if constexpr (kRole == kRolePairP) io->cz[c][o] = mem_add(d, ps[c][o]);
                    T cpl = T(0);
                    if constexpr (kRole == kRolePairD) cpl = pdb[c][o] * (io->cz[c][o] + mem_add(d, ps[c][o]));
                    ps[c][o] = mem_new(pb[c][o], pbm[c][o], ps[c][o], d);
                    if constexpr (kRole == kRolePairD) ps[c][o] = comp_add(ps[c][o], cpl);
                    d = mem_add(d, ps[c][o]);
                }
                lz.v[c][o] = d;
            }
        }
#pragma unroll
        for (int c = 0; c < RX; ++c)
#pragma unroll
            for (int o = 0; o < 4; ++o)
                if (in[c][o]) zpsi[(i0 + o - zb0) + (int64_t)(j0 + c) * nB] = ps[c][o];
    }

    // ---------------- x ----------------
    if (!bx) {
        const T* rowp = Pb + r0 + HZ;  // the thread's 4 rows; column offset added below
        if constexpr (kPacked<T>) {
            float2 acc[RX][2];
#pragma unroll
            for (int c = 0; c < RX; ++c) acc[c][0] = acc[c][1] = make_float2(0.0f, 0.0f);
#pragma unroll
            for (int q = 0; q < RX + 2 * L; ++q) {
                const V4<T> v = ld4(rowp + (c0 + q) * SP);
#pragma unroll
                for (int c = 0; c < RX; ++c) {
                    const int m = q - L - c;
                    if (m >= -L && m <= L) {
                        const float2 a = bc.ax2[m < 0 ? -m : m];
                        acc[c][0] = __ffma2_rn(a, make_float2(v.v[0], v.v[1]), acc[c][0]);
                        acc[c][1] = __ffma2_rn(a, make_float2(v.v[2], v.v[3]), acc[c][1]);
                    }
                }
            }
#pragma unroll
            for (int c = 0; c < RX; ++c) {
                lx.v[c][0] = acc[c][0].x;
                lx.v[c][1] = acc[c][0].y;
                lx.v[c][2] = acc[c][1].x;
                lx.v[c][3] = acc[c][1].y;
            }
        } else {
#pragma unroll
            for (int c = 0; c < RX; ++c)
#pragma unroll
                for (int o = 0; o < 4; ++o) lx.v[c][o] = T(0);
#pragma unroll
            for (int q = 0; q < RX + 2 * L; ++q) {
                const V4<T> v = ld4(rowp + (c0 + q) * SP);
#pragma unroll
                for (int c = 0; c < RX; ++c) {
                    const int m = q - L - c;  // offset of column q from output column c
                    if (m >= -L && m <= L) {
                        const T a = bc.ax[m < 0 ? -m : m];
#pragma unroll
                        for (int o = 0; o < 4; ++o) lx.v[c][o] = fma(a, v.v[o], lx.v[c][o]);
                    }
                }
            }
        }
    } else {
        // D- xA (+ psi): xA column c0+t of the scratch is global column j0-N+t
        const int64_t xoff = (int64_t)nz * 2 * nB;
        const T* xb = sh.xb;
        const T* xbm1 = sh.xbm1;
        M* xpsi = sh.xpsi + (kRole == kRolePairD ? xoff : 0);
        int64_t qo[RX];
        T pb[RX][4], pbm[RX][4];
        T pdb[kRole == kRolePairD ? RX : 1][4];  // D pass: b_Q - b_P
        M ps[RX][4];
#pragma unroll
        for (int c = 0; c < RX; ++c) {
            const int j = j0 + c;
            qo[c] = (j < nx && (j < nB || j >= nx - nB)) ? (int64_t)(j < nB ? j : nB + j - (nx - nB)) * nz : -1;
#pragma unroll
            for (int o = 0; o < 4; ++o) {
                pb[c][o] = T(0);
                pbm[c][o] = T(0);
                ps[c][o] = M{};
                if constexpr (kRole == kRolePairD) pdb[c][o] = T(0);
                if (qo[c] >= 0 && i0 + o < nz) {
                    const int64_t q = qo[c] + i0 + o;
                    pb[c][o] = ldg_t(xb + q);
                    pbm[c][o] = ldg_t(xbm1 + q);
                    ps[c][o] = xpsi[q];
                    if constexpr (kRole == kRolePairD) pdb[c][o] = ldg_t(xb + xoff + q);
                }
            }
        }
        const T* xa = scratch + B::kX / sizeof(T) + r0;
        V4<T> a[RX + 2 * N - 1];
#pragma unroll
        for (int t = 0; t < RX + 2 * N - 1; ++t) a[t] = ld4(xa + (c0 + t) * TZ);
#pragma unroll
        for (int c = 0; c < RX; ++c)
#pragma unroll
            for (int o = 0; o < 4; ++o) {
                T d = bc.wx[0] * (a[c + N].v[o] - a[c + N - 1].v[o]);
#pragma unroll
                for (int k = 1; k < N; ++k) d = fma(bc.wx[k], a[c + N + k].v[o] - a[c + N - 1 - k].v[o], d);
                if (qo[c] >= 0 && i0 + o < nz) {
                    if constexpr (kRole == kRolePairP) io->cx[c][o] = mem_add(d, ps[c][o]);
                    T cpl = T(0);
                    if constexpr (kRole == kRolePairD) cpl = pdb[c][o] * (io->cx[c][o] + mem_add(d, ps[c][o]));
                    ps[c][o] = mem_new(pb[c][o], pbm[c][o], ps[c][o], d);
                    if constexpr (kRole == kRolePairD) ps[c][o] = comp_add(ps[c][o], cpl);
                    d = mem_add(d, ps[c][o]);
                }
                lx.v[c][o] = d;
            }
#pragma unroll
        for (int c = 0; c < RX; ++c)
#pragma unroll
            for (int o = 0; o < 4; ++o)
                if (qo[c] >= 0 && i0 + o < nz) xpsi[qo[c] + i0 + o] = ps[c][o];
    }

    // ---------------- update ----------------
    const int tau = ti.tau;
    const bool full_rows = i0 + 3 < nz;
    T* const Pnew = sh.field[ph ^ 1] + (kRole == kRolePairD ? (int64_t)sh.dcol * sh.ldp : 0);
    Blk<T, RX> pn;
#pragma unroll
    for (int c = 0; c < RX; ++c) {
        const int j = j0 + c;
        if (j >= nx) continue;
        const V4<T> po = ld4(Ob + (c0 + c) * TZ + r0);
        const V4<T> vv = ld4(Vb + (c0 + c) * TZ + r0);
        T lap[4];
        if constexpr (kPacked<T>) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const float2 l2 = __fadd2_rn(make_float2(lz.v[c][2 * h], lz.v[c][2 * h + 1]),
                                             make_float2(lx.v[c][2 * h], lx.v[c][2 * h + 1]));
                lap[2 * h] = l2.x;
                lap[2 * h + 1] = l2.y;
            }
        } else {
#pragma unroll
            for (int o = 0; o < 4; ++o) lap[o] = lz.v[c][o] + lx.v[c][o];
        }
        if constexpr (kRole == kRolePairD) {
            // D_new = wP lap_D + (wQ - wP) (lap_D + lap_P) + 2 D - D_old, lap_P with
            // the injected terms: Q's factor is wP + (wQ - wP) exactly
            const V4<T> vd = ld4(Vd + (c0 + c) * TZ + r0);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const float2 t = __ffma2_rn(make_float2(2.0f, 2.0f), make_float2(pc.v[c][2 * h], pc.v[c][2 * h + 1]),
                                            make_float2(-po.v[2 * h], -po.v[2 * h + 1]));
                const float2 dw = make_float2(vd.v[2 * h], vd.v[2 * h + 1]);
                const float2 lq = __fadd2_rn(make_float2(lap[2 * h], lap[2 * h + 1]),
                                             make_float2(io->lap[c][2 * h], io->lap[c][2 * h + 1]));
                const float2 u = __ffma2_rn(dw, lq, t);
                const float2 r = __ffma2_rn(make_float2(vv.v[2 * h], vv.v[2 * h + 1]),
                                            make_float2(lap[2 * h], lap[2 * h + 1]), u);
                pn.v[c][2 * h] = r.x;
                pn.v[c][2 * h + 1] = r.y;
            }
        } else {
            if (flags & kSource) add_sources<T>(sh, tau, i0, j, lap);
            if constexpr (kRole == kRolePairP) {
#pragma unroll
                for (int o = 0; o < 4; ++o) io->lap[c][o] = lap[o];
                const V4<T> lc = ld4(io->lo + (c0 + c) * TZ + r0);
                const V4<T> lold = ld4(io->lo_old + (c0 + c) * TZ + r0);
                T lnew[4];
#pragma unroll
                for (int o = 0; o < 4; ++o) {
                    const float2 r = pair_update_hi_lo(pc.v[c][o], lc.v[o], po.v[o], lold.v[o], vv.v[o], lap[o]);
                    pn.v[c][o] = r.x;
                    lnew[o] = r.y;
                }
                T* dlo = Pnew + 2 * (int64_t)sh.dcol * sh.ldp + i0 + (int64_t)j * sh.ldp;
                if (full_rows) {
                    st4(dlo, lnew);
                } else {
#pragma unroll
                    for (int o = 0; o < 4; ++o)
                        if (i0 + o < nz) dlo[o] = lnew[o];
                }
            } else if constexpr (kPacked<T>) {
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const float2 t = __ffma2_rn(make_float2(2.0f, 2.0f), make_float2(pc.v[c][2 * h], pc.v[c][2 * h + 1]),
                                                make_float2(-po.v[2 * h], -po.v[2 * h + 1]));
                    const float2 u = __ffma2_rn(make_float2(vv.v[2 * h], vv.v[2 * h + 1]),
                                                make_float2(lap[2 * h], lap[2 * h + 1]), t);
                    pn.v[c][2 * h] = u.x;
                    pn.v[c][2 * h + 1] = u.y;
                }
            } else {
#pragma unroll
                for (int o = 0; o < 4; ++o) pn.v[c][o] = fma(vv.v[o], lap[o], fma(T(2), pc.v[c][o], -po.v[o]));
            }
        }
        T* dst = Pnew + i0 + (int64_t)j * sh.ldp;
        if (full_rows) {
            st4(dst, pn.v[c]);
        } else {
#pragma unroll
            for (int o = 0; o < 4; ++o)
                if (i0 + o < nz) dst[o] = pn.v[c][o];
        }
    }
    T* const rec = kRole == kRolePairD ? sh.rec_d : sh.rec;
    if (rec && i0 == 0) {
        T* r = rec + (int64_t)tau * nx;
        const int ncol = min(RX, nx - j0);
        for (int c = 0; c < ncol; ++c) r[j0 + c] = pn.v[c][0];
    }
    if constexpr (kRole != kRolePairD) {
        // blow-up check on the receiver row: a non-finite value there (a time
        // step beyond the stability limit grows without bound) fails the shot
        if (i0 == 0 && sh.status) {
            const int ncol = min(RX, nx - j0);
            bool bad = false;
            for (int c = 0; c < ncol; ++c) bad |= !(fabs(pn.v[c][0]) <= std::numeric_limits<T>::max());
            if (bad) atomicExch(sh.status, SSSI_ERR_UNSTABLE);
        }
    }
    if constexpr (kRole != kRolePairD && kRareOut)
        if (flags & kRare) amax_bits = max(amax_bits, rare_outputs<T, RX>(sh, ti, i0, j0, pn, pc));
}

// Per-tile work flags at step tau, worked out by the preparing thread from
// the work item's step-independent flags (bands, point sources) and the
// shot's sched word.
__device__ __forceinline__ unsigned tile_flags(unsigned sched, int z0, unsigned f, int tau) {
    if ((sched & kSchedDense) || ((sched & kSchedRow) && z0 <= 0)) f |= kSource;  // z0 <= 0: the tile holds row 0
    bool rare = (sched & (kSchedSnap | kSchedImg64)) != 0u;
    if (sched & (kSchedAmax | kSchedPack | kSchedImg16)) {  // outputs every stride steps
        const int stride = (int)(sched >> kSchedStrideShift);
        const bool on_stride = tau % stride == 0;
        if ((sched & kSchedAmax) && on_stride) f |= kAmax;
        rare |= ((sched & kSchedPack) && ((tau >= 1 && (tau - 1) % stride == 0) || on_stride)) ||
                ((sched & (kSchedAmax | kSchedImg16)) && on_stride);
    }
    if (rare) f |= kRare;
    return f;
}

// Shared-memory layout of one pipeline stage (byte offsets, 128-aligned).
// kPair: the stage also holds a residual pair's D box (kP2), D's previous
// tile (kO2), the (v dt)^2 difference (kV2) and the low parts of P's current
// and previous tiles (kL, kL2), and the band scratch is doubled (P's, then
// D's).
template <typename T, int N, class Sh, bool kPair = false>
struct StageLayout {
    using S = Sh;
    static constexpr int L = 2 * N - 1;
    static constexpr int HZ = tile_halo_rows(N);
    static constexpr int SP = S::TZ + 2 * HZ;
    static constexpr unsigned kPBoxBytes = sizeof(T) * SP * (S::TX + 2 * L);
    static constexpr unsigned kTileBytes = sizeof(T) * S::TZ * S::TX;
    static constexpr unsigned kBoxA = (kPBoxBytes + 127) / 128 * 128;
    static constexpr unsigned kTileA = (kTileBytes + 127) / 128 * 128;
    static constexpr unsigned kP = 0;
    static constexpr unsigned kP2 = kPair ? kBoxA : 0;
    static constexpr unsigned kO = kBoxA * (kPair ? 2 : 1);
    static constexpr unsigned kO2 = kO + (kPair ? kTileA : 0);
    static constexpr unsigned kV = kO2 + kTileA;
    static constexpr unsigned kV2 = kV + (kPair ? kTileA : 0);
    static constexpr unsigned kL = kV2 + kTileA;               // pairs: P's low part, current field
    static constexpr unsigned kL2 = kL + (kPair ? kTileA : 0);  // pairs: P's low part, previous field
    static constexpr unsigned kTail = kPair ? kL2 + kTileA : kL;
    static constexpr unsigned kInfo = kTail + (sizeof(ShotTail<T>) + 127) / 128 * 128;
    static constexpr unsigned kStage = kInfo + 128;  // TileInfo (32 bytes) rounded up
    static constexpr unsigned kTx = kPBoxBytes + 2 * kTileBytes;          // bytes the TMA copies deliver
    static constexpr unsigned kTxPair = 2 * kPBoxBytes + 6 * kTileBytes;  // the same for a residual pair
    static constexpr int kStages = 2;                                     // tiles in the copy pipeline
    static constexpr unsigned kBar = kStages * kStage;                    // one mbarrier per stage
    static constexpr unsigned kScratch = kBar + 128;                      // band scratch
    static constexpr unsigned kScratchD = kScratch + BandScratch<T, N, Sh>::kBytes;  // pairs: D's
    static constexpr unsigned kSmem = kScratch + (kPair ? 2 : 1) * BandScratch<T, N, Sh>::kBytes;
};


// kSplit: the work lists may hold half tiles (schedules of small grids); the
// variant without them keeps the whole-tile path free of their handling.
// kPair: the batch holds residual pairs (FP32, whole tiles only).
// kRareOut: some shot of the batch writes snapshots, FP16 packs, maxima or
// imaging sums (without: whole tiles only, no call to rare_outputs).
template <typename T, int N, bool kSplit, class Sh, bool kPair, bool kRareOut>
__global__ void __launch_bounds__(Sh::kThreads, kPair ? Sh::kMinBlocks / 2 : Sh::kMinBlocks)
    batch2d_kernel(const ShotDesc<T>* __restrict__ shots, const __grid_constant__ BatchConst<T> bc) {
    using S = Sh;
    using G = StageLayout<T, N, Sh, kPair>;
    static_assert(!kPair || (std::is_same<T, float>::value && !kSplit), "residual pairs: FP32 whole tiles");
    static_assert(kRareOut || (!kSplit && !kPair), "the variant without rare outputs takes whole single tiles");
    constexpr int V = Sh::kIndex;  // tensor maps of this shape
    constexpr int TZ = S::TZ, TX = S::TX, RX = S::RX;
    constexpr int HZ = G::HZ, L = G::L;
    extern __shared__ __align__(128) unsigned char smem[];
    constexpr int NS = G::kStages;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + G::kBar);

    const int tid = threadIdx.x;
    const int lane = tid & 31;
    // The next step's grid may be scheduled once every block of this one runs;
    // its blocks then wait (griddepcontrol.wait) for this grid to complete.
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    if (tid == 0) {
#pragma unroll
        for (int q = 0; q < NS; ++q) mbar_init(&bar[q], 1);
        fence_barrier_init();
    }
    __syncthreads();
    int step = 0;

    // Each CTA walks its own list of work items.  Warp 0 keeps the next item
    // and its shot's ShotTail in registers (loaded one iteration ahead), so
    // preparing a stage costs shared-memory stores and three TMA issues.
    const int wbeg = bc.cta_begin[blockIdx.x], wend = bc.cta_begin[blockIdx.x + 1];
    constexpr int kTailVec = (int)(sizeof(ShotTail<T>) / 16);
    static_assert(kTailVec <= 32, "ShotTail must fit one 16-byte load per lane");
    int2 item = make_int2(-1, 0);  // prefetched work item (pack_work_item; x = -1: none)
    unsigned inflight = 0;          // lane 0 of warp 0: stages with copies not yet consumed
    uint4 tail_reg = make_uint4(0, 0, 0, 0);
    auto fetch = [&](int w) {  // warp 0: load item w and its shot's tail into registers
        item = w < wend ? bc.work[w] : make_int2(-1, 0);
        if (item.x >= 0 && lane < kTailVec)
            tail_reg = reinterpret_cast<const uint4*>(&shots[item.x & 0xffffff].s)[lane];
    };
    // lane 0 of warp 0: the three copies of a stage prepared earlier (first
    // stages).  Every stage's barrier completes one phase per use: a stage with
    // nothing to copy (no tile, or an inactive shot) gets a plain arrival.
    auto issue = [&](int s) {
        unsigned char* st = smem + s * G::kStage;
        const TileInfo* info = reinterpret_cast<const TileInfo*>(st + G::kInfo);
        // test knob: at bc.debug_step block 0 issues nothing for its first tile, so
        // that tile's barrier wait runs out and the failure path is exercised
        const bool withheld = bc.debug_step >= 0 && step == bc.debug_step && blockIdx.x == 0 && s == 0;
        if (lane == 0 && info->shot >= 0 && !withheld) {
            const ShotTail<T>& g = *reinterpret_cast<const ShotTail<T>*>(st + G::kTail);
            const int k = info->shot, z0 = info->z0, x0 = info->x0, cur = info->tloc & 1;
            const bool pair = kPair && (g.sched & kSchedPair);
            inflight |= 1u << s;
            fence_proxy_async_shared();
            mbar_arrive_expect_tx(&bar[s], pair ? G::kTxPair : G::kTx);
            tma_load_2d(st + G::kP, &shots[k].tm_box[V][cur], &bar[s], g.oz + z0 - HZ, x0);
            tma_load_2d(st + G::kO, &shots[k].tm_tile[V][cur ^ 1], &bar[s], g.oz + z0, x0 + L);
            tma_load_2d(st + G::kV, &shots[k].tm_v[V], &bar[s], g.oz + z0, x0 + L);
            if (pair) {
                tma_load_2d(st + G::kP2, &shots[k].tm_box[V][cur], &bar[s], g.oz + z0 - HZ, x0 + g.dcol);
                tma_load_2d(st + G::kO2, &shots[k].tm_tile[V][cur ^ 1], &bar[s], g.oz + z0, x0 + L + g.dcol);
                tma_load_2d(st + G::kV2, &shots[k].tm_v[V], &bar[s], g.oz + z0, x0 + L + g.dcol);
                tma_load_2d(st + G::kL, &shots[k].tm_tile[V][cur], &bar[s], g.oz + z0, x0 + L + 2 * g.dcol);
                tma_load_2d(st + G::kL2, &shots[k].tm_tile[V][cur ^ 1], &bar[s], g.oz + z0, x0 + L + 2 * g.dcol);
            }
        }
    };
    // warp 0: put the prefetched item into stage s (tile = its position in the
    // list); with `copy`, lane 0 also issues the stage's three copies (or the
    // plain arrival).  Lane 0 works from registers: the item and the head of the
    // shot's tail.
    // a residual pair's column offset of D, from the lane that holds it
    constexpr int kDcolOff = (int)offsetof(ShotTail<T>, dcol);
    static_assert(kDcolOff % 4 == 0, "dcol is a 32-bit word");
    auto prepare = [&](int w, int s, bool copy) {
        unsigned char* st = smem + s * G::kStage;
        TileInfo* info = reinterpret_cast<TileInfo*>(st + G::kInfo);
        const int k = item.x >= 0 ? (item.x & 0xffffff) : -1;
        if (k >= 0 && lane < kTailVec) reinterpret_cast<uint4*>(st + G::kTail)[lane] = tail_reg;
        int dcol = 0;
        if constexpr (kPair) {
            constexpr int word = (kDcolOff % 16) / 4;
            const unsigned x = word == 0 ? tail_reg.x : word == 1 ? tail_reg.y : word == 2 ? tail_reg.z : tail_reg.w;
            dcol = (int)__shfl_sync(0xffffffffu, x, kDcolOff / 16);
        }
        if (lane == 0) {
            const int t_start = (int)tail_reg.x, nt = (int)tail_reg.y, oz = (int)tail_reg.w;
            const unsigned sched = tail_reg.z;
            int shot = -1, tloc = 0, tau = 0;
            if (k >= 0) {
                tloc = step - t_start;
                if (tloc >= 0 && tloc < nt) {
                    shot = k;
                    tau = (sched & kSchedReverse) ? nt - 1 - tloc : tloc;
                }
            }
            const unsigned top = (unsigned)item.x >> 24;  // static flags | half << 3
            const unsigned half = kSplit ? (top >> 3) & 3u : 0u;  // 0 whole tile, 1 / 2 left / right half
            const int z0 = work_item_z0(item), x0 = work_item_x0(item) + (half == 2u ? TX / 2 : 0);
            info->tile = w < wend ? w : kNoTile;
            info->shot = shot;
            info->tloc = tloc;
            info->tau = tau;
            info->z0 = z0;
            info->x0 = x0;
            info->flags = shot >= 0 ? tile_flags(sched, z0, top & 7u, tau) | (half ? kHalf : 0u) : 0u;
            if (copy && shot >= 0) {
                const int cur = tloc & 1;
                const bool pair = kPair && (sched & kSchedPair);
                inflight |= 1u << s;
                fence_proxy_async_shared();
                mbar_arrive_expect_tx(&bar[s], pair ? G::kTxPair : G::kTx);
                tma_load_2d(st + G::kP, &shots[k].tm_box[V][cur], &bar[s], oz + z0 - HZ, x0);
                tma_load_2d(st + G::kO, &shots[k].tm_tile[V][cur ^ 1], &bar[s], oz + z0, x0 + L);
                tma_load_2d(st + G::kV, &shots[k].tm_v[V], &bar[s], oz + z0, x0 + L);
                if (pair) {
                    tma_load_2d(st + G::kP2, &shots[k].tm_box[V][cur], &bar[s], oz + z0 - HZ, x0 + dcol);
                    tma_load_2d(st + G::kO2, &shots[k].tm_tile[V][cur ^ 1], &bar[s], oz + z0, x0 + L + dcol);
                    tma_load_2d(st + G::kV2, &shots[k].tm_v[V], &bar[s], oz + z0, x0 + L + dcol);
                    tma_load_2d(st + G::kL, &shots[k].tm_tile[V][cur], &bar[s], oz + z0, x0 + L + 2 * dcol);
                    tma_load_2d(st + G::kL2, &shots[k].tm_tile[V][cur ^ 1], &bar[s], oz + z0, x0 + L + 2 * dcol);
                }
            }
        }
        __syncwarp();
    };

    const int r0 = 4 * (tid % (TZ / 4));
    const int c0 = RX * (tid / (TZ / 4));
    unsigned phase_bits = 0;  // completed uses of each stage's barrier (bit s = parity)

    // Work lists and descriptors are written by the host only.  The step base is
    // written only by the one-thread kernels that run between graph replays and
    // at the start of a run; those do not trigger their dependents early, so a
    // step launched after one of them starts only once it has completed, and the
    // base can be read before the wait.  Fields and memory variables are written
    // by the previous step: the copies are issued after the wait.
    step = *reinterpret_cast<volatile const int*>(bc.step_base) + bc.step_offset;
    if (tid < 32) {
        fetch(wbeg);
        for (int q = 0; q < NS - 1; ++q) {  // the first NS-1 items go into stages 0 .. NS-2
            prepare(wbeg + q, q, false);
            fetch(wbeg + q + 1);
        }
    }
    asm volatile("griddepcontrol.wait;" ::: "memory");
    if (tid < 32)
        for (int q = 0; q < NS - 1; ++q) issue(q);
    __syncthreads();
    bool failed = false;
    for (int k = 0;; ++k) {
        const int s = k % NS;
        const unsigned char* st = smem + s * G::kStage;
        // One block barrier per tile: past it every thread has finished tile k-1
        // (its stage and the band scratch are free to reuse) and sees the
        // TileInfo of tile k, which warp 0 wrote before that barrier.
        const TileInfo ti = *reinterpret_cast<const TileInfo*>(st + G::kInfo);
        if (ti.tile == kNoTile) break;
        if (tid < 32) {
            prepare(wbeg + k + NS - 1, (k + NS - 1) % NS, true);
            fetch(wbeg + k + NS);
        }
        if (ti.shot >= 0) {
            const bool ok = mbar_wait_bounded(&bar[s], (phase_bits >> s) & 1u, bc.wait_limit);
            if (__syncthreads_or(!ok)) {
                failed = true;
                break;
            }
            phase_bits ^= 1u << s;
            inflight &= ~(1u << s);
            const ShotTail<T>& sh = *reinterpret_cast<const ShotTail<T>*>(st + G::kTail);
            const T* Pb = reinterpret_cast<const T*>(st + G::kP);
            const T* Ob = reinterpret_cast<const T*>(st + G::kO);
            const T* Vb = reinterpret_cast<const T*>(st + G::kV);
            const int z0 = ti.z0, x0 = ti.x0;
            unsigned amax_bits = 0u;
            // rows above and columns left of the grid (first tiles of a shifted
            // shot) are skipped; x0 and c0 are even, so a thread's columns are
            // all on one side of column 0
            const int i0 = z0 + r0, j0 = x0 + c0;
            T* scratch = reinterpret_cast<T*>(smem + G::kScratch);
            if constexpr (kSplit) {
                // a half tile (band tiles of small grids, split so that they do not set
                // the length of the step) has TX/2 columns: the first half of the threads
                const bool half = ti.flags & kHalf;
                if (ti.flags & (kBandZ | kBandX)) {
                    if (half)
                        band_stage1_cells<T, N, Sh, TX / 2>(bc, sh, ti.tloc & 1, Pb, z0, x0, ti.flags & kBandZ,
                                                        ti.flags & kBandX, scratch);
                    else
                        band_stage1<T, N, Sh, TX>(bc, sh, ti.tloc & 1, Pb, z0, x0, ti.flags & kBandZ, ti.flags & kBandX,
                                              scratch);
                    __syncthreads();
                }
                if (i0 < sh.nz && (j0 | i0) >= 0 && j0 < sh.nx && (!half || c0 < TX / 2))
                    tile_cells<T, N, Sh, RX>(bc, sh, ti, Pb, Ob, Vb, z0, x0, r0, c0, ti.flags, scratch, amax_bits);
            } else {
                bool done = false;
                if constexpr (kPair) {
                    if (sh.sched & kSchedPair) {
                        // a residual pair: P's and D's cells in one tile, P first
                        const T* Pd = reinterpret_cast<const T*>(st + G::kP2);
                        const T* Od = reinterpret_cast<const T*>(st + G::kO2);
                        const T* Vd = reinterpret_cast<const T*>(st + G::kV2);
                        T* scratch_d = reinterpret_cast<T*>(smem + G::kScratchD);
                        if (ti.flags & (kBandZ | kBandX)) {
                            band_stage1_pair<T, N, Sh, TX>(bc, sh, ti.tloc & 1, Pb, Pd, z0, x0, ti.flags & kBandZ,
                                                           ti.flags & kBandX, scratch, scratch_d);
                            __syncthreads();
                        }
                        if (i0 < sh.nz && (j0 | i0) >= 0 && j0 < sh.nx) {
                            PairIO<T, RX> io;
                            io.lo = reinterpret_cast<const T*>(st + G::kL);
                            io.lo_old = reinterpret_cast<const T*>(st + G::kL2);
                            tile_cells<T, N, Sh, RX, kRolePairP>(bc, sh, ti, Pb, Ob, Vb, z0, x0, r0, c0, ti.flags,
                                                                 scratch, amax_bits, &io);
                            tile_cells<T, N, Sh, RX, kRolePairD>(bc, sh, ti, Pd, Od, Vb, z0, x0, r0, c0, ti.flags,
                                                                 scratch_d, amax_bits, &io, Vd);
                        }
                        done = true;
                    }
                }
                if (!done) {
                    if (ti.flags & (kBandZ | kBandX)) {
                        band_stage1<T, N, Sh, TX>(bc, sh, ti.tloc & 1, Pb, z0, x0, ti.flags & kBandZ,
                                                  ti.flags & kBandX, scratch);
                        __syncthreads();
                    }
                    if (i0 < sh.nz && (j0 | i0) >= 0 && j0 < sh.nx)
                        tile_cells<T, N, Sh, RX, kRoleSingle, kRareOut>(bc, sh, ti, Pb, Ob, Vb, z0, x0, r0, c0,
                                                                        ti.flags, scratch, amax_bits);
                }
            }
            if (kRareOut && (ti.flags & kAmax)) {
                // block maxima: one atomic per group of lanes whose cells share a
                // 32 x 32 scale block (lanes that computed nothing skip)
                const int nbz = (sh.nz + 31) >> 5;
                const int key = amax_bits ? (i0 >> 5) + (j0 >> 5) * nbz : -1;
                const unsigned peers = __match_any_sync(0xffffffffu, key);
                const unsigned w = __reduce_max_sync(peers, amax_bits);
                if (key >= 0 && w && lane == __ffs(peers) - 1) {
                    const int64_t nblk = (int64_t)nbz * ((sh.nx + 31) >> 5);
                    atomicMax(sh.amax + (int64_t)(ti.tau / (sh.stride > 0 ? sh.stride : 1)) * nblk + key, w);
                }
            }
        }
        __syncthreads();
    }
    if (failed) {
        if (tid == 0) {
            atomicExch(bc.err, 1);
            // copies issued for stages not yet consumed may still be in flight: wait for
            // them, bounded by the default limit (a copy that was issued lands); if one
            // never does, the block leaves with it outstanding and the reported failure
            // is the only guarantee left
            for (int q = 0; q < NS; ++q)
                if ((inflight >> q) & 1u) mbar_wait_bounded(&bar[q], (phase_bits >> q) & 1u, kDefaultWaitLimit);
        }
        __syncthreads();
    }
}

}  // namespace batch

template <typename T, int N, bool kSplit, class Sh, bool kPair, bool kRareOut = true>
void launch_batch2d_variant(const ShotDesc<T>* shots, const BatchConst<T>& bc, int grid, cudaStream_t stream) {
    using G = batch::StageLayout<T, N, Sh, kPair>;
    static bool configured = false;
    if (!configured) {
        SSSI_CHECK_CUDA(cudaFuncSetAttribute(batch::batch2d_kernel<T, N, kSplit, Sh, kPair, kRareOut>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::kSmem));
        configured = true;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(Sh::kThreads);
    cfg.dynamicSmemBytes = G::kSmem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    SSSI_CHECK_CUDA(cudaLaunchKernelEx(&cfg, batch::batch2d_kernel<T, N, kSplit, Sh, kPair, kRareOut>, shots, bc));
    count_launch();
}

template <typename T, int N, class Sh>
void launch_batch2d_shape(const ShotDesc<T>* shots, const BatchConst<T>& bc, int grid, bool split, bool lean,
                          cudaStream_t stream) {
    if (split)
        launch_batch2d_variant<T, N, true, Sh, false>(shots, bc, grid, stream);
    else if (lean)
        launch_batch2d_variant<T, N, false, Sh, false, false>(shots, bc, grid, stream);
    else
        launch_batch2d_variant<T, N, false, Sh, false>(shots, bc, grid, stream);
}

template <typename T, int N>
void launch_batch2d_n(const ShotDesc<T>* shots, const BatchConst<T>& bc, int grid, bool split, int shape, bool pair,
                      bool lean, cudaStream_t stream) {
    if constexpr (kBatchShapes<T> > 1) {
        if (pair) {
            SSSI_REQUIRE(shape == 1 && !split, SSSI_ERR_INTERNAL, "residual pairs run with 32 x 32 whole tiles");
            launch_batch2d_variant<T, N, false, BatchShape<T, 1>, true>(shots, bc, grid, stream);
            return;
        }
        if (shape == 1) {
            launch_batch2d_shape<T, N, BatchShape<T, 1>>(shots, bc, grid, split, lean, stream);
            return;
        }
        if constexpr (kBatchShapes<T> > 2)
            if (shape == 2) {
                launch_batch2d_shape<T, N, BatchShape<T, 2>>(shots, bc, grid, split, lean, stream);
                return;
            }
    }
    SSSI_REQUIRE(!pair, SSSI_ERR_INTERNAL, "residual pairs are FP32 only");
    SSSI_REQUIRE(shape == 0, SSSI_ERR_INTERNAL, "tile shape %d not built for this type", shape);
    launch_batch2d_shape<T, N, BatchShape<T, 0>>(shots, bc, grid, split, lean, stream);
}

template <typename T, int N, class Sh, bool kPair>
int batch2d_occupancy_shape() {
    const size_t smem = batch::StageLayout<T, N, Sh, kPair>::kSmem;
    int n = 0;
    cudaError_t e = cudaFuncSetAttribute(batch::batch2d_kernel<T, N, false, Sh, kPair, true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch::batch2d_kernel<T, N, false, Sh, kPair, true>,
                                                          Sh::kThreads, smem);
    if (e != cudaSuccess || n < 1) {
        cudaGetLastError();
        n = 1;
    }
    return n;
}

template <typename T, int N>
int batch2d_occupancy_n(int shape, bool pair) {
    if constexpr (kBatchShapes<T> > 1) {
        if (pair) return batch2d_occupancy_shape<T, N, BatchShape<T, 1>, true>();
        if (shape == 1) return batch2d_occupancy_shape<T, N, BatchShape<T, 1>, false>();
        if constexpr (kBatchShapes<T> > 2)
            if (shape == 2) return batch2d_occupancy_shape<T, N, BatchShape<T, 2>, false>();
    }
    return batch2d_occupancy_shape<T, N, BatchShape<T, 0>, false>();
}

#define SSSI_BATCH2D_INSTANCE(T, N)                                                                      \
    template void launch_batch2d_n<T, N>(const ShotDesc<T>*, const BatchConst<T>&, int, bool, int, bool, \
                                         bool, cudaStream_t);                                            \
    template int batch2d_occupancy_n<T, N>(int, bool);

}  // namespace sssi
