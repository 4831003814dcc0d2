// Fused 2D acoustic CPML time step for sm_103a.
//
// One launch advances the whole grid by one time step
// (src/fd_cmex/fwdTimeCpmlFor2dAw_mex.c:183-290): both first-derivative
// stages of both axes, the CPML memory-variable updates, the leapfrog update,
// source injection, receiver gather and snapshot output, in one pass over the
// wavefield.  It serves the strict FP64 mode (the reference's rounding
// sequence) and the no-allocation entry point; the fused FP64 and FP32 modes
// run on the batched tiled kernel.
//
// Work decomposition: a block owns BZ consecutive rows (one row per thread,
// so a warp reads 32 consecutive z samples of one column: coalesced) and
// marches along x over W columns.  Each thread keeps the last 2N samples of
// its row of P and the last 2N values of xA in registers, so every x
// derivative is computed exactly once per cell; the column being updated is
// staged in shared memory with l = 2N-1 halo rows above and below for the z
// derivatives.  Halo columns at the ends of the march and halo rows of the z
// stencil are recomputed (not exchanged), so blocks never wait on each other.
// The CPML memory variables phi are double-buffered because halo recomputation
// reads them in neighbouring blocks during the step; psi is touched only by the
// owner of a cell and is updated in place.
#include "cpml2d.cuh"

namespace sssi {

namespace {

// ---- arithmetic policies ----------------------------------------------------
// Strict: every operation rounded separately, in the reference's order:
//   D = sum_k (c_k * (a_k - b_k)) / d        (finiteDifference.c:116-117)
// Fast: D = sum_k w_k * (a_k - b_k) with w_k = c_k/d, fused multiply-adds.
template <typename T, bool STRICT>
struct Arith;

template <>
struct Arith<double, true> {
    template <int N>
    __device__ __forceinline__ static double dsum(const double* c, const Divisor<double>& d, const double* a,
                                                  const double* b) {
        double s = div_rn(__dmul_rn(c[0], __dsub_rn(a[0], b[0])), d);
#pragma unroll
        for (int k = 1; k < N; ++k) s = __dadd_rn(s, div_rn(__dmul_rn(c[k], __dsub_rn(a[k], b[k])), d));
        return s;
    }
    // b*m + bm1*d
    __device__ __forceinline__ static double mem(double b, double m, double bm1, double d) {
        return __dadd_rn(__dmul_rn(b, m), __dmul_rn(bm1, d));
    }
    __device__ __forceinline__ static double add(double a, double b) { return __dadd_rn(a, b); }
    // vdt2*((zp + xp) + s) + 2*p - po
    __device__ __forceinline__ static double update(double vdt2, double zp, double xp, double s, double p,
                                                    double po) {
        return __dsub_rn(__dadd_rn(__dmul_rn(vdt2, __dadd_rn(__dadd_rn(zp, xp), s)), __dmul_rn(2.0, p)), po);
    }
};

template <typename T>
struct ArithFast {
    template <int N>
    __device__ __forceinline__ static T dsum(const T* w, const Divisor<T>&, const T* a, const T* b) {
        T s = w[0] * (a[0] - b[0]);
#pragma unroll
        for (int k = 1; k < N; ++k) s = fma(w[k], a[k] - b[k], s);
        return s;
    }
    template <typename TA>
    __device__ __forceinline__ static TA mem(TA b, TA m, TA bm1, TA d) {
        return fma(b, m, bm1 * d);
    }
    __device__ __forceinline__ static T add(T a, T b) { return a + b; }
    __device__ __forceinline__ static T update(T vdt2, T zp, T xp, T s, T p, T po) {
        return fma(vdt2, zp + xp + s, fma(T(2), p, -po));
    }
};
template <>
struct Arith<double, false> : ArithFast<double> {};
template <>
struct Arith<float, false> : ArithFast<float> {};

// Combines a derivative d (type T) with a memory variable of type TA.
template <typename T, typename TA, bool STRICT>
__device__ __forceinline__ T add_mem(T d, TA m) {
    if constexpr (STRICT) {
        return __dadd_rn(d, m);
    } else {
        return static_cast<T>(static_cast<TA>(d) + m);
    }
}

template <typename T, typename TA, bool STRICT>
__device__ __forceinline__ TA mem_update(TA b, TA m, TA bm1, T d) {
    if constexpr (STRICT) {
        return __dadd_rn(__dmul_rn(b, m), __dmul_rn(bm1, d));
    } else {
        return fma(b, m, bm1 * static_cast<TA>(d));
    }
}


template <typename T, typename TA, int N, bool STRICT>
__global__ void cpml2d_step_kernel(const Step2D<T, TA> p) {
    constexpr int L = 2 * N - 1;
    using A = Arith<T, STRICT>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int BZ = blockDim.x;
    T* Ps = reinterpret_cast<T*>(smem_raw);  // P(z0-L .. z0+BZ+L-1, j)
    T* zAs = Ps + BZ + 2 * L;                // zA(z0-N .. z0+BZ+N-2, j)

    const int tid = threadIdx.x;
    const int z0 = blockIdx.x * BZ;
    const int i = z0 + tid;
    const bool row_ok = i < p.nz;
    const int x0 = blockIdx.y * p.W;
    const int x1 = min(x0 + p.W, p.nx);
    const int nz = p.nz, nx = p.nx, nB = p.nB;
    const int zband0 = nz - nB;
    const int64_t ldp = p.ldp;

    T cz[N], cx[N];
#pragma unroll
    for (int k = 0; k < N; ++k) {
        cz[k] = p.cz[k];
        cx[k] = p.cx[k];
    }

    // point sources of this step that fall in this block's rows
    double src_amp[kMaxPointSources];
#pragma unroll
    for (int s = 0; s < kMaxPointSources; ++s) src_amp[s] = (s < p.nsrc) ? p.src_wavelet[(int64_t)s * p.nt + p.t] : 0.0;

    T pq[2 * N];  // P(i, k-2N+1 .. k)
    T aq[2 * N];  // xA(i, k-N-2N+1 .. k-N)
#pragma unroll
    for (int q = 0; q < 2 * N; ++q) {
        pq[q] = T(0);
        aq[q] = T(0);
    }

    const T* Prow = p.P + i;
    for (int k = x0 - L; k < x1 + L; ++k) {
#pragma unroll
        for (int q = 0; q < 2 * N - 1; ++q) pq[q] = pq[q + 1];
        pq[2 * N - 1] = Prow[(int64_t)k * ldp];
        if (k < x0) continue;

        // ---- xA at column jx = k - N (x derivative at jx + 1/2) ----
        {
            const int jx = k - N;
            T a[N], b[N];
#pragma unroll
            for (int m = 0; m < N; ++m) {
                a[m] = pq[N + m];
                b[m] = pq[N - 1 - m];
            }
            T d = A::template dsum<N>(cx, p.dx, a, b);
            T xa = d;
            if (row_ok && jx >= 0 && jx < nx && (jx < nB || jx >= nx - nB)) {
                const int c = jx < nB ? jx : nB + jx - (nx - nB);
                const int64_t q = i + (int64_t)c * nz;
                const TA phi = mem_update<T, TA, STRICT>(p.xb[q], p.xphi_in[q], p.xbm1[q], d);
                if (jx >= x0 && jx < x1) p.xphi_out[q] = phi;
                xa = add_mem<T, TA, STRICT>(d, phi);
            }
#pragma unroll
            for (int q = 0; q < 2 * N - 1; ++q) aq[q] = aq[q + 1];
            aq[2 * N - 1] = xa;
        }
        if (k < x0 + L) continue;

        // ---- output column j ----
        const int j = k - L;
        const T pc = pq[0];
        Ps[L + tid] = pc;
        if (tid < L) {
            Ps[tid] = p.P[(int64_t)(z0 - L + tid) + (int64_t)j * ldp];
            Ps[BZ + L + tid] = p.P[(int64_t)(z0 + BZ + tid) + (int64_t)j * ldp];
        }
        __syncthreads();
        for (int rr = tid; rr < BZ + L; rr += BZ) {
            const int r = z0 - N + rr;
            T a[N], b[N];
#pragma unroll
            for (int m = 0; m < N; ++m) {
                a[m] = Ps[rr + N + m];
                b[m] = Ps[rr + N - 1 - m];
            }
            T d = A::template dsum<N>(cz, p.dz, a, b);
            T za = d;
            if (r >= zband0 && r < nz && r >= 0) {
                const int64_t q = (r - zband0) + (int64_t)j * nB;
                const TA phi = mem_update<T, TA, STRICT>(p.zb[q], p.zphi_in[q], p.zbm1[q], d);
                if (rr >= N && rr < N + BZ) p.zphi_out[q] = phi;
                za = add_mem<T, TA, STRICT>(d, phi);
            }
            zAs[rr] = za;
        }
        __syncthreads();

        if (row_ok) {
            T a[N], b[N];
#pragma unroll
            for (int m = 0; m < N; ++m) {
                a[m] = zAs[tid + N + m];
                b[m] = zAs[tid + N - 1 - m];
            }
            const T dzm = A::template dsum<N>(cz, p.dz, a, b);
            T zp = dzm;
            if (i >= zband0) {
                const int64_t q = (i - zband0) + (int64_t)j * nB;
                const TA psi = mem_update<T, TA, STRICT>(p.zb[q], p.zpsi[q], p.zbm1[q], dzm);
                p.zpsi[q] = psi;
                zp = add_mem<T, TA, STRICT>(dzm, psi);
            }
#pragma unroll
            for (int m = 0; m < N; ++m) {
                a[m] = aq[N + m];
                b[m] = aq[N - 1 - m];
            }
            const T dxm = A::template dsum<N>(cx, p.dx, a, b);
            T xp = dxm;
            if (j < nB || j >= nx - nB) {
                const int c = j < nB ? j : nB + j - (nx - nB);
                const int64_t q = i + (int64_t)c * nz;
                const TA psi = mem_update<T, TA, STRICT>(p.xb[q], p.xpsi[q], p.xbm1[q], dxm);
                p.xpsi[q] = psi;
                xp = add_mem<T, TA, STRICT>(dxm, psi);
            }

            double sv = 0.0;
            if (p.src_dense) sv = p.src_dense[i + (int64_t)j * nz];
            if (p.src_row && i == 0) sv = p.src_row[j] - (p.src_row_sub ? p.src_row_sub[j] : 0.0);
#pragma unroll
            for (int s = 0; s < kMaxPointSources; ++s)
                if (s < p.nsrc && i == p.src_iz[s] && j == p.src_ix[s]) sv += src_amp[s];

            const int64_t pidx = i + (int64_t)j * ldp;
            const int64_t q = i + (int64_t)j * nz;
            const T po = p.Pold[pidx];
            const T pn = A::update(p.vdt2[q], zp, xp, static_cast<T>(sv), pc, po);
            p.Pold[pidx] = pn;

            if (p.rec && i == 0) p.rec[j] = static_cast<double>(pn);
            if (p.snap) p.snap[q] = static_cast<double>(pn);
        }
    }
}

template <typename T, typename TA, bool STRICT, int N>
void launch_n(const Step2D<T, TA>& p, int bz, cudaStream_t stream) {
    constexpr int L = 2 * N - 1;
    dim3 grid((p.nz + bz - 1) / bz, (p.nx + p.W - 1) / p.W);
    const size_t smem = sizeof(T) * (2 * bz + 3 * L);
    cpml2d_step_kernel<T, TA, N, STRICT><<<grid, bz, smem, stream>>>(p);
    count_launch();
}

template <typename T, typename TA, bool STRICT>
void launch_dispatch(const Step2D<T, TA>& p, int N, int bz, cudaStream_t stream) {
    switch (N) {
        case 1: launch_n<T, TA, STRICT, 1>(p, bz, stream); break;
        case 2: launch_n<T, TA, STRICT, 2>(p, bz, stream); break;
        case 3: launch_n<T, TA, STRICT, 3>(p, bz, stream); break;
        case 4: launch_n<T, TA, STRICT, 4>(p, bz, stream); break;
        case 5: launch_n<T, TA, STRICT, 5>(p, bz, stream); break;
        case 6: launch_n<T, TA, STRICT, 6>(p, bz, stream); break;
        case 7: launch_n<T, TA, STRICT, 7>(p, bz, stream); break;
        case 8: launch_n<T, TA, STRICT, 8>(p, bz, stream); break;
        default: SSSI_REQUIRE(false, SSSI_ERR_ARG, "nDiffOrder %d out of range 1..8", N);
    }
    SSSI_CHECK_CUDA(cudaGetLastError());
}

// FP16 copy of a padded FP32 field, one power-of-two scale per 32 x 32 block
// (the block maxima amax[bz + bx * nbz], nbz = ceil(nz / 32)), with the error
// feedback of the batched step: err (nz x nx) is added before rounding and
// receives the new rounding error.
__global__ void pack_f16_kernel(const float* P, int64_t ldp, int nz, int nx, const unsigned* amax, __half* out,
                                float* err) {
    const int64_t n = (int64_t)nz * nx;
    const int nbz = (nz + 31) >> 5;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = q % nz, j = q / nz;
        const float scale = fp16_scale_from_amax(amax[(i >> 5) + (j >> 5) * nbz]);
        const float x = __fadd_rn(P[i + j * ldp], err[q]);
        const __half h = __float2half_rn(__fmul_rn(x, scale));
        err[q] = __fsub_rn(x, __fmul_rn(__half2float(h), 1.0f / scale));
        out[q] = h;
    }
}

}  // namespace

template <typename T, typename TA>
void launch_cpml2d_step(const Step2D<T, TA>& p, int N, bool strict, int bz, cudaStream_t stream) {
    if constexpr (std::is_same<T, double>::value && std::is_same<TA, double>::value) {
        if (strict)
            launch_dispatch<T, TA, true>(p, N, bz, stream);
        else
            launch_dispatch<T, TA, false>(p, N, bz, stream);
    } else {
        SSSI_REQUIRE(!strict, SSSI_ERR_ARG, "strict arithmetic exists only in FP64");
        launch_dispatch<T, TA, false>(p, N, bz, stream);
    }
}

template <typename T, typename TA>
cudaError_t launch_cpml2d_step_nothrow(const Step2D<T, TA>& p, int N, bool strict, int bz, cudaStream_t stream) {
    if (N < 1 || N > kMaxOrder) return cudaErrorInvalidValue;
    if constexpr (std::is_same<T, double>::value && std::is_same<TA, double>::value) {
        if (strict) {
            switch (N) {
                case 1: launch_n<T, TA, true, 1>(p, bz, stream); break;
                case 2: launch_n<T, TA, true, 2>(p, bz, stream); break;
                case 3: launch_n<T, TA, true, 3>(p, bz, stream); break;
                case 4: launch_n<T, TA, true, 4>(p, bz, stream); break;
                case 5: launch_n<T, TA, true, 5>(p, bz, stream); break;
                case 6: launch_n<T, TA, true, 6>(p, bz, stream); break;
                case 7: launch_n<T, TA, true, 7>(p, bz, stream); break;
                default: launch_n<T, TA, true, 8>(p, bz, stream); break;
            }
            return cudaGetLastError();
        }
    } else {
        if (strict) return cudaErrorInvalidValue;
    }
    switch (N) {
        case 1: launch_n<T, TA, false, 1>(p, bz, stream); break;
        case 2: launch_n<T, TA, false, 2>(p, bz, stream); break;
        case 3: launch_n<T, TA, false, 3>(p, bz, stream); break;
        case 4: launch_n<T, TA, false, 4>(p, bz, stream); break;
        case 5: launch_n<T, TA, false, 5>(p, bz, stream); break;
        case 6: launch_n<T, TA, false, 6>(p, bz, stream); break;
        case 7: launch_n<T, TA, false, 7>(p, bz, stream); break;
        default: launch_n<T, TA, false, 8>(p, bz, stream); break;
    }
    return cudaGetLastError();
}

void launch_pack_f16(const float* P, int64_t ldp, int nz, int nx, const unsigned* amax, __half* out, float* err,
                     cudaStream_t stream) {
    pack_f16_kernel<<<152 * 4, 256, 0, stream>>>(P, ldp, nz, nx, amax, out, err);
    count_launch();
    SSSI_CHECK_CUDA(cudaGetLastError());
}

// ---------------------------------------------------------------- state
template <typename T, typename TA>
Cpml2d<T, TA>::Cpml2d(const double* v, int64_t nz, int64_t nx, int N, int nB, double dz, double dx, double dt,
                      bool strict, cudaStream_t stream)
    : nz_(nz), nx_(nx), N_(N), L_(2 * N - 1), nB_(nB), strict_(strict), stream_(stream) {
    SSSI_REQUIRE(N >= 1 && N <= kMaxOrder, SSSI_ERR_ARG, "nDiffOrder must be in 1..%d (got %d)", kMaxOrder, N);
    SSSI_REQUIRE(nz >= 1 && nx >= 1, SSSI_ERR_ARG, "empty model (%lld x %lld)", (long long)nz, (long long)nx);
    SSSI_REQUIRE(nB >= 0 && nB <= nz && 2 * (int64_t)nB <= nx, SSSI_ERR_ARG,
                 "nBoundary %d does not fit the model (%lld x %lld): need nBoundary <= nz and 2*nBoundary <= nx", nB,
                 (long long)nz, (long long)nx);
    SSSI_REQUIRE(nz < (1LL << 30) && nx < (1LL << 30), SSSI_ERR_ARG, "model too large");
    constexpr int al = Scalar<T>::kAlign;
    const int64_t oz = (L_ + al - 1) / al * al;             // top padding rows
    const int64_t nz_alloc = (nz + 255) / 256 * 256;        // rows touched by the last block (bz <= 256)
    ldp_ = (oz + nz_alloc + L_ + al - 1) / al * al;
    origin_ = oz + (int64_t)L_ * ldp_;
    const size_t pbytes = sizeof(T) * (size_t)ldp_ * (size_t)(nx + 2 * L_);
    for (auto& b : P_) b.allocate(pbytes);

    // host-side coefficients
    double c[kMaxOrder];
    staggered_coefficients(N, c);
    for (int k = 0; k < kMaxOrder; ++k) {
        tmpl_.cz[k] = tmpl_.cx[k] = T(0);
    }
    for (int k = 0; k < N; ++k) {
        if (strict) {
            tmpl_.cz[k] = static_cast<T>(c[k]);
            tmpl_.cx[k] = static_cast<T>(c[k]);
        } else {
            tmpl_.cz[k] = static_cast<T>(c[k] / dz);
            tmpl_.cx[k] = static_cast<T>(c[k] / dx);
        }
    }
    tmpl_.dz = make_divisor<T>(dz);
    tmpl_.dx = make_divisor<T>(dx);

    // (v dt)^2 and damping bands
    const int64_t n = nz * nx;
    std::vector<T> vdt2(n);
    for (int64_t q = 0; q < n; ++q) vdt2[q] = static_cast<T>((v[q] * dt) * (v[q] * dt));
    vdt2_.allocate(sizeof(T) * n);
    SSSI_CHECK_CUDA(cudaMemcpyAsync(vdt2_.get(), vdt2.data(), sizeof(T) * n, cudaMemcpyHostToDevice, stream));

    Bands2D bands = damping_bands_2d(v, nz, nx, nB, dz, dx, dt);
    auto upload = [&](DeviceBuffer& buf, const std::vector<double>& src) {
        std::vector<TA> tmp(src.begin(), src.end());
        buf.allocate(sizeof(TA) * std::max<size_t>(tmp.size(), 1));
        if (!tmp.empty())
            SSSI_CHECK_CUDA(cudaMemcpyAsync(buf.get(), tmp.data(), sizeof(TA) * tmp.size(), cudaMemcpyHostToDevice,
                                            stream));
        SSSI_CHECK_CUDA(cudaStreamSynchronize(stream));  // tmp goes out of scope
    };
    upload(zb_, bands.zb);
    upload(zbm1_, bands.zbm1);
    upload(xb_, bands.xb);
    upload(xbm1_, bands.xbm1);
    const size_t zbytes = sizeof(TA) * std::max<size_t>((size_t)nB * nx, 1);
    const size_t xbytes = sizeof(TA) * std::max<size_t>((size_t)nz * 2 * nB, 1);
    zphi_[0].allocate(zbytes);
    zphi_[1].allocate(zbytes);
    zpsi_.allocate(zbytes);
    xphi_[0].allocate(xbytes);
    xphi_[1].allocate(xbytes);
    xpsi_.allocate(xbytes);

    tmpl_.nz = (int)nz;
    tmpl_.nx = (int)nx;
    tmpl_.nB = nB;
    tmpl_.ldp = ldp_;
    tmpl_.vdt2 = vdt2_.as<T>();
    tmpl_.zb = zb_.as<TA>();
    tmpl_.zbm1 = zbm1_.as<TA>();
    tmpl_.xb = xb_.as<TA>();
    tmpl_.xbm1 = xbm1_.as<TA>();
    tmpl_.zpsi = zpsi_.as<TA>();
    tmpl_.xpsi = xpsi_.as<TA>();
    reset();
}

template <typename T, typename TA>
void Cpml2d<T, TA>::reset() {
    for (auto& b : P_) b.zero(stream_);
    for (auto* b : {&zphi_[0], &zphi_[1], &zpsi_, &xphi_[0], &xphi_[1], &xpsi_}) b->zero(stream_);
    cur_ = 0;
    phase_ = 0;
}

template <typename T, typename TA>
void Cpml2d<T, TA>::set_point_sources(int nsrc, const int64_t* iz, const int64_t* ix, const T* d_wavelet, int nt) {
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

template <typename T, typename TA>
void Cpml2d<T, TA>::step(const StepIO<T>& io) {
    Step2D<T, TA> p = tmpl_;
    p.W = w_;
    p.t = io.t;
    p.P = field(cur_);
    p.Pold = field(1 - cur_);
    p.zphi_in = zphi_[phase_].template as<TA>();
    p.zphi_out = zphi_[1 - phase_].template as<TA>();
    p.xphi_in = xphi_[phase_].template as<TA>();
    p.xphi_out = xphi_[1 - phase_].template as<TA>();
    p.src_dense = io.src_dense;
    p.src_row = io.src_row;
    p.src_row_sub = nullptr;
    p.rec = io.rec;
    p.snap = io.snap;
    if (p.nsrc == 0) p.src_wavelet = nullptr;
    launch_cpml2d_step<T, TA>(p, N_, strict_, bz_, stream_);
    cur_ = 1 - cur_;
    phase_ = 1 - phase_;
}

template class Cpml2d<double, double>;
template void launch_cpml2d_step<double, double>(const Step2D<double, double>&, int, bool, int, cudaStream_t);
template cudaError_t launch_cpml2d_step_nothrow<double, double>(const Step2D<double, double>&, int, bool, int,
                                                                cudaStream_t);

}  // namespace sssi
