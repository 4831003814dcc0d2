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
//   - every GPU that loads this part of the library holds kScratchBytes of
//     device memory until the process exits;
//   - every call uses the same array, so calls whose work overlaps on the GPU
//     (two host threads, or two streams) race and corrupt each other; callers
//     must serialise them;
//   - the array keeps the previous call's contents; each call clears the parts
//     that must start at zero (both wavefields and the CPML memory variables)
//     and overwrites the rest;
//   - the device address of the array is looked up once per device, on the
//     first call made with that device current (cudaGetSymbolAddress); make
//     that first call before any stream capture begins.
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <mutex>

#include "cpml2d.cuh"

namespace sssi {

namespace {

constexpr size_t kScratchBytes = size_t(SSSI_NOALLOC_SCRATCH_BYTES);
constexpr int kMaxDevices = 64;

// The working state of the entry point.  Host code must not use this name as
// an address: it looks the device address up with cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kMaxDevices] = {};

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    set_error("%s", buf);
    return code;
}

// Device address of g_noalloc_scratch on the current device (looked up once).
cudaError_t scratch_address(unsigned char** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_noalloc_ptr[dev] = p;
    }
    *out = static_cast<unsigned char*>(g_noalloc_ptr[dev]);
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

// (v dt)^2 and the damping factors of the three CPML bands, computed on the
// device from the caller's velocity (C-gateway formulas, fwd...mex.c:100-145).
__global__ void noalloc_setup_kernel(const double* v, int nz, int nx, int nB, double dz, double dx, double dt,
                                     double logR, double* vdt2, double* zb, double* zbm1, double* xb, double* xbm1) {
    const int64_t n = (int64_t)nz * nx;
    const int64_t nzb = (int64_t)nB * nx;
    const int64_t nxb = (int64_t)nz * 2 * nB;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n + nzb + nxb; q += stride) {
        if (q < n) {
            const double vdt = v[q] * dt;
            vdt2[q] = vdt * vdt;
        } else if (q < n + nzb) {
            const int64_t k = q - n;
            const int r = (int)(k % nB);
            const int64_t j = k / nB;
            const double L = nB * dz, u = (r + 1) * dz;
            const double d0 = -(3.0 * v[(nz - nB + r) + j * nz]) / (2 * L) * logR;
            const double d = d0 * (u / L) * (u / L);
            const double e = exp(-d * dt);
            zb[k] = e;
            zbm1[k] = e - 1;
        } else {
            const int64_t k = q - n - nzb;
            const int64_t i = k % nz;
            const int c = (int)(k / nz);
            const int64_t j = c < nB ? c : nx - nB + (c - nB);
            const double L = nB * dx, u = c < nB ? (nB - c) * dx : (c - nB + 1) * dx;
            const double d0 = -(3.0 * v[i + j * nz]) / (2 * L) * logR;
            const double d = d0 * (u / L) * (u / L);
            const double e = exp(-d * dt);
            xb[k] = e;
            xbm1[k] = e - 1;
        }
    }
}

int run(const double* v, const double* source, int64_t nz, int64_t nx, int64_t nt, int N, int nB, double dz,
        double dx, double dt, double* data, double* snapshot, int mode) {
    if (!(nz > 0 && nx > 0 && nt >= 0)) return fail(SSSI_ERR_ARG, "bad sizes nz=%lld nx=%lld nt=%lld", (long long)nz,
                                                     (long long)nx, (long long)nt);
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
    noalloc_setup_kernel<<<152 * 4, 256, 0, s>>>(v, (int)nz, (int)nx, nB, dz, dx, dt, std::log(1e-6), at(g.vdt2),
                                                  at(g.zb), at(g.zbm1), at(g.xb), at(g.xbm1));
    count_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(SSSI_ERR_CUDA, "set-up kernel launch failed: %s", cudaGetErrorString(e));

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
    p.dz = dz;
    p.dx = dx;
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
