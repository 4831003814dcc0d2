// Kernel body of the tiled 2D CPML step (included by one translation unit per
// element type; see tile2d.cuh for the design).
#pragma once

#include "tile2d.cuh"

namespace sssi {
namespace tile {

// ---- 4-element vectors in shared memory (16 bytes for float, 32 for double) ----
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
// FP32, compensated: phi = hi + lo carried exactly through the update with
// error-free products (fma residuals) and a two-sum; the rounded operations
// use intrinsics so the compiler cannot fuse them.
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

// All cells of one thread: rows i0..i0+3, columns j0..j0+RX-1.
template <typename T, int N, bool ZC, bool XC>
__device__ __forceinline__ void tile_cells(const TileStep<T>& p, const T* Pb, const T* Ob, const T* Vb, int z0,
                                           int x0, int r0, int c0, float pack_scale, float img_inv,
                                           unsigned& amax_bits) {
    using S = TileShape<T>;
    using M = typename MemVar<T>::type;
    constexpr int TZ = S::TZ, RX = S::RX;
    constexpr int L = 2 * N - 1;
    constexpr int HZ = tile_halo_rows(N);
    constexpr int SP = TZ + 2 * HZ;  // pitch of a P-box column
    constexpr int WIN = 4 + 2 * HZ;  // z window of one column
    const int nz = p.nz, nx = p.nx, nB = p.nB;
    const int zb0 = nz - nB;
    const int i0 = z0 + r0, j0 = x0 + c0;

    T lz[RX][4], lx[RX][4], pc[RX][4];

    // ---------------- z ----------------
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
#pragma unroll
        for (int o = 0; o < 4; ++o) pc[c][o] = w[HZ + o];
        if constexpr (ZC) {
#pragma unroll
            for (int o = 0; o < 4; ++o) {
                T acc = p.az[0] * w[HZ + o];
#pragma unroll
                for (int m = 1; m <= L; ++m) acc = fma(p.az[m], w[HZ + o + m] + w[HZ + o - m], acc);
                lz[c][o] = acc;
            }
        } else {
            const int j = j0 + c;
            const bool jok = j < nx;
            // zA at rows i0-N .. i0+3+N-1 (index e = o' + N)
            T za[4 + L];
#pragma unroll
            for (int e = 0; e < 4 + L; ++e) {
                const int op = e - N;
                T d = p.wz[0] * (w[HZ + op + 1] - w[HZ + op]);
#pragma unroll
                for (int n = 1; n < N; ++n) d = fma(p.wz[n], w[HZ + op + 1 + n] - w[HZ + op - n], d);
                const int ip = i0 + op;
                T a = d;
                if (jok && ip >= zb0 && ip < nz && ip >= 0) {
                    const int64_t q = (ip - zb0) + (int64_t)j * nB;
                    const M phi = mem_new(p.zb[q], p.zbm1[q], p.zphi_in[q], d);
                    if (op >= 0 && op < 4) p.zphi_out[q] = phi;
                    a = mem_add(d, phi);
                }
                za[e] = a;
            }
#pragma unroll
            for (int o = 0; o < 4; ++o) {
                T d = p.wz[0] * (za[o + N] - za[o + N - 1]);
#pragma unroll
                for (int k = 1; k < N; ++k) d = fma(p.wz[k], za[o + N + k] - za[o + N - 1 - k], d);
                const int i = i0 + o;
                if (jok && i >= zb0 && i < nz) {
                    const int64_t q = (i - zb0) + (int64_t)j * nB;
                    const M psi = mem_new(p.zb[q], p.zbm1[q], p.zpsi[q], d);
                    p.zpsi[q] = psi;
                    d = mem_add(d, psi);
                }
                lz[c][o] = d;
            }
        }
    }

    // ---------------- x ----------------
    const T* rowp = Pb + r0 + HZ;  // the thread's 4 rows, column index added below
    if constexpr (XC) {
#pragma unroll
        for (int c = 0; c < RX; ++c)
#pragma unroll
            for (int o = 0; o < 4; ++o) lx[c][o] = T(0);
#pragma unroll
        for (int q = 0; q < RX + 2 * L; ++q) {
            const V4<T> v = ld4(rowp + (c0 + q) * SP);
#pragma unroll
            for (int c = 0; c < RX; ++c) {
                const int m = q - L - c;  // offset of column q from output column c
                if (m >= -L && m <= L) {
                    const T a = p.ax[m < 0 ? -m : m];
#pragma unroll
                    for (int o = 0; o < 4; ++o) lx[c][o] = fma(a, v.v[o], lx[c][o]);
                }
            }
        }
    } else {
#pragma unroll
        for (int c = 0; c < RX; ++c)
#pragma unroll
            for (int o = 0; o < 4; ++o) lx[c][o] = T(0);
        V4<T> win[2 * N];  // P columns jq-2N+1 .. jq
#pragma unroll
        for (int q = 0; q < RX + 2 * L; ++q) {
#pragma unroll
            for (int k = 0; k < 2 * N - 1; ++k) win[k] = win[k + 1];
            win[2 * N - 1] = ld4(rowp + (c0 + q) * SP);
            if (q < L) continue;
            // xA at column e relative to j0: e = q - L - N + ... : interior column j0 - L + q - N
            const int e = q - L - N + 0;  // xA column offset from j0 (ranges -N .. RX+N-2)
            const int jc = j0 + e;
            T xa[4];
#pragma unroll
            for (int o = 0; o < 4; ++o) {
                T d = p.wx[0] * (win[N].v[o] - win[N - 1].v[o]);
#pragma unroll
                for (int n = 1; n < N; ++n) d = fma(p.wx[n], win[N + n].v[o] - win[N - 1 - n].v[o], d);
                xa[o] = d;
            }
            if (jc >= 0 && jc < nx && (jc < nB || jc >= nx - nB)) {
                const int cb = jc < nB ? jc : nB + jc - (nx - nB);
                const bool own = e >= 0 && e < RX;
#pragma unroll
                for (int o = 0; o < 4; ++o) {
                    const int i = i0 + o;
                    if (i < nz) {
                        const int64_t qq = i + (int64_t)cb * nz;
                        const M phi = mem_new(p.xb[qq], p.xbm1[qq], p.xphi_in[qq], xa[o]);
                        if (own) p.xphi_out[qq] = phi;
                        xa[o] = mem_add(xa[o], phi);
                    }
                }
            }
            // D- at output c: sum_k w_k (xA(c+k) - xA(c-1-k)); xA column e feeds
            // c = e - k with +w_k and c = e + 1 + k with -w_k
#pragma unroll
            for (int k = 0; k < N; ++k) {
                const int cp = e - k, cm = e + 1 + k;
                if (cp >= 0 && cp < RX) {
#pragma unroll
                    for (int o = 0; o < 4; ++o) lx[cp][o] = fma(p.wx[k], xa[o], lx[cp][o]);
                }
                if (cm >= 0 && cm < RX) {
#pragma unroll
                    for (int o = 0; o < 4; ++o) lx[cm][o] = fma(-p.wx[k], xa[o], lx[cm][o]);
                }
            }
        }
#pragma unroll
        for (int c = 0; c < RX; ++c) {
            const int j = j0 + c;
            if (j < nx && (j < nB || j >= nx - nB)) {
                const int cb = j < nB ? j : nB + j - (nx - nB);
#pragma unroll
                for (int o = 0; o < 4; ++o) {
                    const int i = i0 + o;
                    if (i < nz) {
                        const int64_t qq = i + (int64_t)cb * nz;
                        const M psi = mem_new(p.xb[qq], p.xbm1[qq], p.xpsi[qq], lx[c][o]);
                        p.xpsi[qq] = psi;
                        lx[c][o] = mem_add(lx[c][o], psi);
                    }
                }
            }
        }
    }

    // ---------------- update and epilogue ----------------
    // Sources are accumulated in T: a double here would put work on the FP64
    // pipe for every cell (it is a small fraction of the FP32 rate on GB300).
    // Point sources are tested only when one falls inside this thread's block.
    bool has_point = false;
    for (int s = 0; s < p.nsrc; ++s)
        has_point |= p.src_iz[s] >= i0 && p.src_iz[s] < i0 + 4 && p.src_ix[s] >= j0 && p.src_ix[s] < j0 + RX;
    const bool full_rows = i0 + 3 < nz;
    T pn[RX][4];
#pragma unroll
    for (int c = 0; c < RX; ++c) {
        const int j = j0 + c;
        if (j >= nx) continue;
        const V4<T> po = ld4(Ob + (c0 + c) * TZ + r0);
        const V4<T> vv = ld4(Vb + (c0 + c) * TZ + r0);
#pragma unroll
        for (int o = 0; o < 4; ++o) {
            const int i = i0 + o;
            T sv = T(0);
            if (p.src_dense && i < nz) sv = p.src_dense[i + (int64_t)j * nz];
            if (p.src_row && i == 0) sv = p.src_row[j];
            if (has_point) {
                for (int s = 0; s < p.nsrc; ++s)
                    if (i == p.src_iz[s] && j == p.src_ix[s]) sv += p.src_wavelet[(int64_t)s * p.nt + p.t];
            }
            const T lap = lz[c][o] + lx[c][o] + sv;
            pn[c][o] = fma(vv.v[o], lap, fma(T(2), pc[c][o], -po.v[o]));
        }
        T* dst = p.Pnew + i0 + (int64_t)j * p.ldp;
        if (full_rows) {
            st4(dst, pn[c]);
        } else {
#pragma unroll
            for (int o = 0; o < 4; ++o)
                if (i0 + o < nz) dst[o] = pn[c][o];
        }
    }
    // Optional outputs.  Each is a separate branch on a launch-wide pointer so
    // that no conversion to double runs unless that output was asked for.
    const int nrow = min(4, nz - i0);
    const int ncol = min(RX, nx - j0);
    if (p.rec && i0 == 0) {
        for (int c = 0; c < ncol; ++c) p.rec[j0 + c] = pn[c][0];
    }
    if (p.snap) {
        for (int c = 0; c < ncol; ++c)
            for (int o = 0; o < nrow; ++o) p.snap[(i0 + o) + (int64_t)(j0 + c) * nz] = pn[c][o];
    }
    if (p.pack) {
        for (int c = 0; c < ncol; ++c)
            for (int o = 0; o < nrow; ++o)
                p.pack[(i0 + o) + (int64_t)(j0 + c) * nz] = __float2half_rn(f32(pc[c][o]) * pack_scale);
    }
    if (p.amax) {
        for (int c = 0; c < ncol; ++c)
            for (int o = 0; o < nrow; ++o) amax_bits = max(amax_bits, __float_as_uint(fabsf(f32(pn[c][o]))));
    }
    if constexpr (std::is_same<T, double>::value) {
        if (p.img_f64) {
            for (int c = 0; c < ncol; ++c)
                for (int o = 0; o < nrow; ++o) {
                    const int64_t q = (i0 + o) + (int64_t)(j0 + c) * nz;
                    const double f = p.img_f64[q];
                    p.img_m[q] = fma(f, pn[c][o], p.img_m[q]);
                    p.img_s2[q] = fma(f, f, p.img_s2[q]);
                }
        }
    }
    if (p.img_f16) {
        for (int c = 0; c < ncol; ++c)
            for (int o = 0; o < nrow; ++o) {
                const int64_t q = (i0 + o) + (int64_t)(j0 + c) * nz;
                const float f = __half2float(p.img_f16[q]) * img_inv;
                const float r = f32(pn[c][o]);
                p.img_m2[q] = comp_add(p.img_m2[q], __fmul_rn(f, r));
                p.img_s22[q] = comp_add(p.img_s22[q], __fmul_rn(f, f));
            }
    }
}

// Shared-memory layout of one pipeline stage (byte offsets, 128-aligned).
template <typename T, int N>
struct StageLayout {
    using S = TileShape<T>;
    static constexpr int L = 2 * N - 1;
    static constexpr int HZ = tile_halo_rows(N);
    static constexpr int SP = S::TZ + 2 * HZ;
    static constexpr unsigned kPBoxBytes = sizeof(T) * SP * (S::TX + 2 * L);
    static constexpr unsigned kTileBytes = sizeof(T) * S::TZ * S::TX;
    static constexpr unsigned kP = 0;
    static constexpr unsigned kO = (kPBoxBytes + 127) / 128 * 128;
    static constexpr unsigned kV = kO + (kTileBytes + 127) / 128 * 128;
    static constexpr unsigned kStage = kV + (kTileBytes + 127) / 128 * 128;
    static constexpr unsigned kTx = kPBoxBytes + 2 * kTileBytes;  // bytes the TMA copies deliver
    static constexpr unsigned kSmem = 2 * kStage + 64;            // two stages + barriers
};

constexpr unsigned kWaitLimit = 1u << 24;

template <typename T, int N>
__global__ void __launch_bounds__(TileShape<T>::kThreads, TileShape<T>::kMinBlocks) tile2d_kernel(const __grid_constant__ CUtensorMap tm_cur,
                                                              const __grid_constant__ CUtensorMap tm_old,
                                                              const __grid_constant__ CUtensorMap tm_v,
                                                              const TileStep<T> p) {
    using S = TileShape<T>;
    using G = StageLayout<T, N>;
    constexpr int TZ = S::TZ, TX = S::TX, RX = S::RX;
    constexpr int HZ = G::HZ, L = G::L;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + 2 * G::kStage);

    const int tid = threadIdx.x;
    const int ntiles = p.ntz * p.ntx;
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_barrier_init();
    }
    __syncthreads();

    auto issue = [&](int tile, int s) {
        const int z0 = (tile % p.ntz) * TZ, x0 = (tile / p.ntz) * TX;
        unsigned char* st = smem + s * G::kStage;
        fence_proxy_async_shared();
        mbar_arrive_expect_tx(&bar[s], G::kTx);
        tma_load_2d(st + G::kP, &tm_cur, &bar[s], p.oz + z0 - HZ, x0);
        tma_load_2d(st + G::kO, &tm_old, &bar[s], p.oz + z0, x0 + L);
        tma_load_2d(st + G::kV, &tm_v, &bar[s], p.oz + z0, x0 + L);
    };

    float pack_scale = 1.0f;
    if (p.pack) {
        pack_scale = fp16_scale_from_amax(*p.pack_amax);
        if (blockIdx.x == 0 && tid == 0 && p.pack_inv_scale_out) *p.pack_inv_scale_out = 1.0f / pack_scale;
    }
    const float img_inv = p.img_f16 ? *p.img_inv_scale : 1.0f;
    unsigned amax_bits = 0u;

    const int r0 = 4 * (tid % (TZ / 4));
    const int c0 = RX * (tid / (TZ / 4));
    const bool zc_all = p.nB == 0;

    int tile = blockIdx.x;
    if (tid == 0 && tile < ntiles) issue(tile, 0);
    for (int k = 0; tile < ntiles; ++k, tile += gridDim.x) {
        const int s = k & 1;
        const int next = tile + gridDim.x;
        if (tid == 0 && next < ntiles) issue(next, s ^ 1);
        const bool ok = mbar_wait_bounded(&bar[s], (k >> 1) & 1, kWaitLimit);
        if (__syncthreads_or(!ok)) {
            if (tid == 0) {
                atomicExch(p.err, 1);
                if (next < ntiles) mbar_wait_bounded(&bar[s ^ 1], ((k + 1) >> 1) & 1, kWaitLimit);
            }
            return;
        }
        const unsigned char* st = smem + s * G::kStage;
        const T* Pb = reinterpret_cast<const T*>(st + G::kP);
        const T* Ob = reinterpret_cast<const T*>(st + G::kO);
        const T* Vb = reinterpret_cast<const T*>(st + G::kV);
        const int z0 = (tile % p.ntz) * TZ, x0 = (tile / p.ntz) * TX;
        if (z0 + r0 < p.nz && x0 + c0 < p.nx) {
            const bool zc = zc_all || z0 + TZ + N - 1 <= p.nz - p.nB;
            const bool xc = zc_all || (x0 - N >= p.nB && x0 + TX + N - 1 <= p.nx - p.nB);
            if (zc && xc)
                tile_cells<T, N, true, true>(p, Pb, Ob, Vb, z0, x0, r0, c0, pack_scale, img_inv, amax_bits);
            else if (zc)
                tile_cells<T, N, true, false>(p, Pb, Ob, Vb, z0, x0, r0, c0, pack_scale, img_inv, amax_bits);
            else if (xc)
                tile_cells<T, N, false, true>(p, Pb, Ob, Vb, z0, x0, r0, c0, pack_scale, img_inv, amax_bits);
            else
                tile_cells<T, N, false, false>(p, Pb, Ob, Vb, z0, x0, r0, c0, pack_scale, img_inv, amax_bits);
        }
        __syncthreads();  // stage s is refilled by the next iteration's issue
    }
    if (p.amax) {
        const unsigned w = __reduce_max_sync(0xffffffffu, amax_bits);
        if ((tid & 31) == 0 && w) atomicMax(p.amax, w);
    }
}

}  // namespace tile

template <typename T, int N>
void launch_tile2d_n(const CUtensorMap& tm_cur, const CUtensorMap& tm_old, const CUtensorMap& tm_v,
                     const TileStep<T>& p, int grid, cudaStream_t stream) {
    using G = tile::StageLayout<T, N>;
    static bool configured = false;
    if (!configured) {
        SSSI_CHECK_CUDA(cudaFuncSetAttribute(tile::tile2d_kernel<T, N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)G::kSmem));
        configured = true;
    }
    tile::tile2d_kernel<T, N><<<grid, TileShape<T>::kThreads, G::kSmem, stream>>>(tm_cur, tm_old, tm_v, p);
    count_launch();
    SSSI_CHECK_CUDA(cudaGetLastError());
}

template <typename T, int N>
size_t tile2d_smem_n() {
    return tile::StageLayout<T, N>::kSmem;
}

template <typename T, int N>
int tile2d_occupancy_n() {
    const size_t smem = tile::StageLayout<T, N>::kSmem;
    int n = 0;
    cudaError_t e = cudaFuncSetAttribute(tile::tile2d_kernel<T, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, tile::tile2d_kernel<T, N>, TileShape<T>::kThreads, smem);
    if (e != cudaSuccess || n < 1) {
        cudaGetLastError();
        n = 1;
    }
    return n;
}

#define SSSI_TILE2D_INSTANCE(T, N)                                                                           \
    template void launch_tile2d_n<T, N>(const CUtensorMap&, const CUtensorMap&, const CUtensorMap&,        \
                                        const TileStep<T>&, int, cudaStream_t);                            \
    template size_t tile2d_smem_n<T, N>();                                                                 \
    template int tile2d_occupancy_n<T, N>();

}  // namespace sssi
