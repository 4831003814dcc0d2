// sssi_fwdTimeCpmlFor2dAwNoAlloc: 2D forward modelling that allocates nothing.
//
// Who needs it: some callers must not allocate memory once they are running.
// A service that has already handed the whole GPU to its own memory pool gets
// out-of-memory from any extra cudaMalloc; a latency-bound loop cannot afford
// the device-wide synchronisation that cudaMalloc and cudaFree imply; a host
// application may forbid heap use after start-up.  For them this entry point
// takes inputs and outputs in device memory that the caller owns and keeps all
// of its working state (two wavefields, (v dt)^2, the CPML band coefficients
// and memory variables) in one fixed array of kScratchBytes that is compiled
// into the library.  It calls no cudaMalloc, cudaFree or other allocating
// routine, allocates no host heap memory and throws no C++ exception.
//
// Costs and rules of the fixed array:
//   - the array is reserved on a GPU when this part of the library is first
//     loaded there, which with CUDA's default lazy module loading is the
//     first call of this function on that GPU; from then on the GPU holds
//     kScratchBytes of device memory until the process exits.  A caller that
//     hands all free GPU memory to its own pool should make one call first
//     (a zero-step call, nt = 0, is enough);
//   - every call uses the same array, so calls whose work overlaps on the GPU
//     (two host threads, or two streams) race and corrupt each other; callers
//     must serialise them (host threads are serialised inside the call, the
//     GPU work of calls on different streams is not);
//   - the array keeps the previous call's contents; each call clears the parts
//     that must start at zero (both wavefields and the CPML memory variables)
//     and overwrites the rest;
//   - the device address of the array is looked up on every call, with the
//     calling thread's current device (cudaGetSymbolAddress), so it stays right
//     after a device reset;
//   - the call blocks until its work is done (it synchronises its stream), so
//     it must not be called while any stream of the calling thread is being
//     captured into a CUDA graph.
//
// The band damping factors are computed on the host with the same formula and
// the same libm exp as the allocating entry points, through one fixed host
// staging array, so the strict FP64 mode is bit-identical to them.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstring>
#include <mutex>

#include "cpml2d.cuh"

namespace sssi {

namespace {

constexpr size_t kScratchBytes = size_t(SSSI_NOALLOC_SCRATCH_BYTES);

// The working state of the entry point.  Host code must not use this name as
// an address: it looks the device address up with cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Host staging for the band damping factors: the band strip of v comes down,
// is turned into b = exp(-d dt) (then b - 1) in place, and goes up again.  The
// layout check bounds every band array to a fifth of the device array.
constexpr size_t kStageDoubles = kScratchBytes / 5 / sizeof(double);
static double g_noalloc_stage[kStageDoubles];

// Held for a whole call: the staging array and the device array are shared.
std::mutex g_noalloc_mu;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    set_error("%s", buf);
    return code;
}

// Device address of g_noalloc_scratch on the current device.
cudaError_t scratch_address(unsigned char** out) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    *out = static_cast<unsigned char*>(p);
    return cudaSuccess;
}

bool on_device(const void* p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Staggered coefficients with the LU of staggered_coefficients(), on the stack.
void coefficients_on_stack(int N, double* c) {
    double A[kMaxOrder * kMaxOrder], x[kMaxOrder];
    int piv[kMaxOrder];
    for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) A[i + j * N] = std::pow(2.0 * (j + 1) - 1.0, 2 * (i + 1) - 1);
    for (int i = 0; i < N; ++i) x[i] = 0.0;
    x[0] = 1.0;
    for (int k = 0; k < N; ++k) {
        int p = k;
        double best = std::fabs(A[k + k * N]);
        for (int i = k + 1; i < N; ++i)
            if (std::fabs(A[i + k * N]) > best) {
                best = std::fabs(A[i + k * N]);
                p = i;
            }
        piv[k] = p;
        if (p != k)
            for (int j = 0; j < N; ++j) {
                const double t = A[k + j * N];
                A[k + j * N] = A[p + j * N];
                A[p + j * N] = t;
            }
        if (A[k + k * N] != 0.0) {
            const double r = 1.0 / A[k + k * N];
            for (int i = k + 1; i < N; ++i) A[i + k * N] *= r;
        }
        for (int j = k + 1; j < N; ++j) {
            const double t = -A[k + j * N];
            for (int i = k + 1; i < N; ++i) A[i + j * N] += A[i + k * N] * t;
        }
    }
    for (int k = 0; k < N; ++k)
        if (piv[k] != k) {
            const double t = x[k];
            x[k] = x[piv[k]];
            x[piv[k]] = t;
        }
    for (int k = 0; k < N; ++k)
        if (x[k] != 0.0)
            for (int i = k + 1; i < N; ++i) x[i] -= x[k] * A[i + k * N];
    for (int k = N - 1; k >= 0; --k)
        if (x[k] != 0.0) {
            x[k] /= A[k + k * N];
            for (int i = 0; i < k; ++i) x[i] -= x[k] * A[i + k * N];
        }
    for (int i = 0; i < N; ++i) c[i] = x[i];
}

// Where each piece of state lives inside the array (byte offsets, 256-aligned).
struct Layout {
    int64_t ldp, origin;
    size_t P[2], vdt2, zb, zbm1, zphi[2], zpsi, xb, xbm1, xphi[2], xpsi, total;
    size_t field_bytes, zband_bytes, xband_bytes;
};

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

Layout plan(int64_t nz, int64_t nx, int L, int nB, int bz) {
    Layout g{};
    const int64_t oz = 16;  // >= L for every supported order; 128-byte aligned row 0
    const int64_t nz_alloc = (nz + bz - 1) / bz * bz;
    g.ldp = (oz + nz_alloc + L + 15) / 16 * 16;
    g.origin = oz + (int64_t)L * g.ldp;
    g.field_bytes = sizeof(double) * (size_t)g.ldp * (size_t)(nx + 2 * L);
    g.zband_bytes = sizeof(double) * std::max<size_t>((size_t)nB * nx, 1);
    g.xband_bytes = sizeof(double) * std::max<size_t>((size_t)nz * 2 * nB, 1);
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t at = off;
        off = align256(off + bytes);
        return at;
    };
    g.P[0] = take(g.field_bytes);
    g.P[1] = take(g.field_bytes);
    g.vdt2 = take(sizeof(double) * (size_t)nz * nx);
    g.zb = take(g.zband_bytes);
    g.zbm1 = take(g.zband_bytes);
    g.zphi[0] = take(g.zband_bytes);
    g.zphi[1] = take(g.zband_bytes);
    g.zpsi = take(g.zband_bytes);
    g.xb = take(g.xband_bytes);
    g.xbm1 = take(g.xband_bytes);
    g.xphi[0] = take(g.xband_bytes);
    g.xphi[1] = take(g.xband_bytes);
    g.xpsi = take(g.xband_bytes);
    g.total = off;
    return g;
}

// (v dt)^2 on the device from the caller's velocity, rounded as the
// allocating entry points round it: (v*dt) * (v*dt).
__global__ void noalloc_vdt2_kernel(const double* v, int64_t n, double dt, double* vdt2) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += stride) {
        const double vdt = __dmul_rn(v[q], dt);
        vdt2[q] = __dmul_rn(vdt, vdt);
    }
}

// Damping factors of one band, C-gateway formulas (fwdTimeCpmlFor2dAw_mex.c:100-145)
// through damp_c_order and the host's exp, exactly as damping_bands_2d_strips
// computes them: the band strip of v (rows x cols, pitch ld doubles, at vsrc)
// comes down into the staging array, b = exp(-d dt) goes up to b_out, then
// b - 1 to bm1_out.  u_of(r, c) is the distance into the band, L its width.
template <class U>
cudaError_t band_factors(const double* vsrc, int64_t ld, int64_t rows, int64_t cols, U u_of, double L, double dt,
                         double* b_out, double* bm1_out, cudaStream_t s) {
    const int64_t n = rows * cols;
    if (n == 0) return cudaSuccess;
    if ((size_t)n > kStageDoubles) return cudaErrorInvalidValue;
    double* h = g_noalloc_stage;
    cudaError_t e = cudaMemcpy2DAsync(h, sizeof(double) * rows, vsrc, sizeof(double) * ld, sizeof(double) * rows,
                                      cols, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    for (int64_t c = 0; c < cols; ++c)
        for (int64_t r = 0; r < rows; ++r) {
            const double d = damp_c_order(u_of(r, c), h[r + c * rows], L);
            h[r + c * rows] = std::exp(-d * dt);
        }
    e = cudaMemcpyAsync(b_out, h, sizeof(double) * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    for (int64_t q = 0; q < n; ++q) h[q] = h[q] - 1;
    e = cudaMemcpyAsync(bm1_out, h, sizeof(double) * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return e;
}

int run(const double* v, const double* source, int64_t nz, int64_t nx, int64_t nt, int N, int nB, double dz,
        double dx, double dt, double* data, double* snapshot, int mode) {
    if (!(nz > 0 && nx > 0 && nt >= 0)) return fail(SSSI_ERR_ARG, "bad sizes nz=%lld nx=%lld nt=%lld", (long long)nz,
                                                     (long long)nx, (long long)nt);
    // bounds before any size arithmetic: the layout sums and the per-step
    // offsets t * nz * nx must not wrap
    if (nz >= (int64_t(1) << 30) || nx >= (int64_t(1) << 30) || nt >= (int64_t(1) << 31) ||
        nz * nx > INT64_MAX / std::max<int64_t>(nt, 1))
        return fail(SSSI_ERR_ARG, "sizes out of range: nz=%lld nx=%lld nt=%lld (nz, nx < 2^30, nt < 2^31)",
                    (long long)nz, (long long)nx, (long long)nt);
    if (N < 1 || N > kMaxOrder) return fail(SSSI_ERR_ARG, "nDiffOrder must be in 1..%d (got %d)", kMaxOrder, N);
    if (nB < 0 || nB > nz || 2 * (int64_t)nB > nx)
        return fail(SSSI_ERR_ARG, "nBoundary %d does not fit the model (%lld x %lld)", nB, (long long)nz,
                    (long long)nx);
    if (!(dz > 0 && dx > 0 && dt > 0)) return fail(SSSI_ERR_ARG, "dz, dx, dt must be positive");
    if (mode != SSSI_MODE_FP64_STRICT && mode != SSSI_MODE_FP64)
        return fail(SSSI_ERR_ARG, "the no-allocation entry point computes in FP64 only (mode %d)", mode);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(SSSI_ERR_CUDA, "no CUDA device available");
    }
    if (!v || !on_device(v)) return fail(SSSI_ERR_ARG, "v must be device memory (this entry point copies nothing)");
    if (source && !on_device(source)) return fail(SSSI_ERR_ARG, "source must be device memory");
    if (data && !on_device(data)) return fail(SSSI_ERR_ARG, "data must be device memory");
    if (snapshot && !on_device(snapshot)) return fail(SSSI_ERR_ARG, "snapshot must be device memory");

    const int L = 2 * N - 1;
    const int bz = nz >= 512 ? 128 : (nz >= 96 ? 64 : 32);
    const int W = 32;
    const Layout g = plan(nz, nx, L, nB, bz);
    if (g.total > kScratchBytes)
        return fail(SSSI_ERR_ARG,
                    "a %lld x %lld grid at nDiffOrder %d needs %zu bytes of working memory; the no-allocation "
                    "entry point has a fixed %zu bytes (use sssi_fwdTimeCpmlFor2dAw for larger grids)",
                    (long long)nz, (long long)nx, N, g.total, kScratchBytes);

    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    unsigned char* base = nullptr;
    cudaError_t e = scratch_address(&base);
    if (e != cudaSuccess) return fail(SSSI_ERR_CUDA, "cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
    cudaStream_t s = current_stream();

    // parts that must start at zero; the rest is overwritten below
    const size_t zero_at[] = {g.P[0], g.P[1], g.zphi[0], g.zphi[1], g.zpsi, g.xphi[0], g.xphi[1], g.xpsi};
    const size_t zero_len[] = {g.field_bytes, g.field_bytes, g.zband_bytes, g.zband_bytes,
                               g.zband_bytes, g.xband_bytes, g.xband_bytes, g.xband_bytes};
    for (int k = 0; k < 8; ++k) {
        e = cudaMemsetAsync(base + zero_at[k], 0, zero_len[k], s);
        if (e != cudaSuccess) return fail(SSSI_ERR_CUDA, "cudaMemsetAsync failed: %s", cudaGetErrorString(e));
    }
    auto at = [&](size_t off) { return reinterpret_cast<double*>(base + off); };
    noalloc_vdt2_kernel<<<152 * 4, 256, 0, s>>>(v, nz * nx, dt, at(g.vdt2));
    count_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(SSSI_ERR_CUDA, "set-up kernel launch failed: %s", cudaGetErrorString(e));
    // bottom band: rows nz-nB .. nz-1, u = (r+1) dz; side bands: columns 0 .. nB-1
    // (u = (nB-c) dx) and nx-nB .. nx-1 (u = (c+1) dx), each nz rows
    const double Lz = nB * dz, Lx = nB * dx;
    e = band_factors(v + (nz - nB), nz, nB, nx, [&](int64_t r, int64_t) { return (r + 1) * dz; }, Lz, dt,
                     at(g.zb), at(g.zbm1), s);
    if (e == cudaSuccess)
        e = band_factors(v, nz, nz, nB, [&](int64_t, int64_t c) { return (nB - c) * dx; }, Lx, dt, at(g.xb),
                         at(g.xbm1), s);
    if (e == cudaSuccess)
        e = band_factors(v + (nx - nB) * nz, nz, nz, nB, [&](int64_t, int64_t c) { return (c + 1) * dx; }, Lx, dt,
                         at(g.xb) + nz * nB, at(g.xbm1) + nz * nB, s);
    if (e != cudaSuccess) return fail(SSSI_ERR_CUDA, "damping set-up failed: %s", cudaGetErrorString(e));

    double c[kMaxOrder];
    coefficients_on_stack(N, c);
    const bool strict = mode == SSSI_MODE_FP64_STRICT;
    Step2D<double, double> p{};
    p.nz = (int)nz;
    p.nx = (int)nx;
    p.nB = nB;
    p.W = W;
    p.ldp = g.ldp;
    p.vdt2 = at(g.vdt2);
    p.zb = at(g.zb);
    p.zbm1 = at(g.zbm1);
    p.zpsi = at(g.zpsi);
    p.xb = at(g.xb);
    p.xbm1 = at(g.xbm1);
    p.xpsi = at(g.xpsi);
    for (int k = 0; k < N; ++k) {
        p.cz[k] = strict ? c[k] : c[k] / dz;
        p.cx[k] = strict ? c[k] : c[k] / dx;
    }
    p.dz = make_divisor<double>(dz);
    p.dx = make_divisor<double>(dx);
    const int64_t n = nz * nx;
    int cur = 0;
    for (int64_t t = 0; t < nt; ++t) {
        const int ph = (int)(t & 1);
        p.t = (int)t;
        p.P = at(g.P[cur]) + g.origin;
        p.Pold = at(g.P[1 - cur]) + g.origin;
        p.zphi_in = at(g.zphi[ph]);
        p.zphi_out = at(g.zphi[1 - ph]);
        p.xphi_in = at(g.xphi[ph]);
        p.xphi_out = at(g.xphi[1 - ph]);
        p.src_dense = source ? source + t * n : nullptr;
        p.rec = data ? data + t * nx : nullptr;
        p.snap = snapshot ? snapshot + t * n : nullptr;
        e = launch_cpml2d_step_nothrow<double, double>(p, N, strict, bz, s);
        if (e != cudaSuccess) return fail(SSSI_ERR_CUDA, "step launch failed: %s", cudaGetErrorString(e));
        cur = 1 - cur;
    }
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(SSSI_ERR_CUDA, "propagation failed: %s", cudaGetErrorString(e));
    return SSSI_OK;
}

}  // namespace
}  // namespace sssi

extern "C" int sssi_fwdTimeCpmlFor2dAwNoAlloc(const double* v, const double* source, int64_t nz, int64_t nx,
                                              int64_t nt, int nDiffOrder, int nBoundary, double dz, double dx,
                                              double dt, double* data, double* snapshot, int mode) {
    sssi::clear_error();
    return sssi::run(v, source, nz, nx, nt, nDiffOrder, nBoundary, dz, dx, dt, data, snapshot, mode);
}
