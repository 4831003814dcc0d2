// Host-side set-up of the CPML finite-difference step: staggered-grid
// coefficients and damping profiles.  Compiled with -ffp-contract=off so every
// expression rounds exactly as written (the reference C is built that way on
// x86-64, where nothing is fused).
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstring>

#include "sssi_internal.h"

namespace sssi {

void staggered_coefficients(int N, double* c) {
    // A_ij = (2j+1)^(2i+1) (0-based), b = e1; LU with partial pivoting:
    // unblocked right-looking elimination that scales the pivot column by the
    // reciprocal pivot, then row interchanges on b, unit-lower forward
    // substitution and upper back substitution (column oriented).
    std::vector<double> A(static_cast<size_t>(N) * N), x(N, 0.0);
    std::vector<int> piv(N);
    for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) A[i + j * N] = std::pow(2.0 * (j + 1) - 1.0, 2 * (i + 1) - 1);
    x[0] = 1.0;
    for (int k = 0; k < N; ++k) {
        int p = k;
        double best = std::fabs(A[k + k * N]);
        for (int i = k + 1; i < N; ++i) {
            if (std::fabs(A[i + k * N]) > best) {
                best = std::fabs(A[i + k * N]);
                p = i;
            }
        }
        piv[k] = p;
        if (p != k)
            for (int j = 0; j < N; ++j) std::swap(A[k + j * N], A[p + j * N]);
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
        if (piv[k] != k) std::swap(x[k], x[piv[k]]);
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

double damp_c_order(double u, double v, double L) {
    const double logR = std::log(1e-6);
    const double d0 = -(3.0 * v) / (2 * L) * logR;
    return d0 * (u / L) * (u / L);
}

double damp_m_order(double u, double v, double L) {
    const double logR = std::log(1e-6);
    const double d0 = -(3 * v) / (2 * L) * logR;
    const double q = u / L;
    return d0 * (q * q);
}

Bands2D damping_bands_2d_strips(const double* bottom, const double* sides, int64_t nz, int64_t nx, int nB, double dz,
                                double dx, double dt) {
    Bands2D b;
    b.zb.resize(static_cast<size_t>(nB) * nx);
    b.zbm1.resize(b.zb.size());
    b.xb.resize(static_cast<size_t>(nz) * 2 * nB);
    b.xbm1.resize(b.xb.size());
    // bottom band: u = (r+1)*dz, velocity of the damped cell (fwd...mex.c:127-145)
    for (int64_t j = 0; j < nx; ++j)
        for (int r = 0; r < nB; ++r) {
            const double d = damp_c_order((r + 1) * dz, bottom[r + j * nB], nB * dz);
            const double e = std::exp(-d * dt);
            b.zb[r + j * nB] = e;
            b.zbm1[r + j * nB] = e - 1;
        }
    // left band u = (nB-j)*dx, right band u = (j-(nx-nB)+1)*dx (fwd...mex.c:100-124)
    for (int c = 0; c < 2 * nB; ++c) {
        const double u = c < nB ? (nB - c) * dx : (c - nB + 1) * dx;
        for (int64_t i = 0; i < nz; ++i) {
            const double d = damp_c_order(u, sides[i + c * nz], nB * dx);
            const double e = std::exp(-d * dt);
            b.xb[i + c * nz] = e;
            b.xbm1[i + c * nz] = e - 1;
        }
    }
    return b;
}

Bands2D damping_bands_2d(const double* v, int64_t nz, int64_t nx, int nB, double dz, double dx, double dt) {
    std::vector<double> bottom(static_cast<size_t>(nB) * nx), sides(static_cast<size_t>(nz) * 2 * nB);
    for (int64_t j = 0; j < nx; ++j)
        for (int r = 0; r < nB; ++r) bottom[r + j * nB] = v[nz - nB + r + j * nz];
    for (int c = 0; c < 2 * nB; ++c) {
        const int64_t j = c < nB ? c : nx - nB + (c - nB);
        std::copy(v + j * nz, v + (j + 1) * nz, sides.begin() + c * nz);
    }
    return damping_bands_2d_strips(bottom.data(), sides.data(), nz, nx, nB, dz, dx, dt);
}

Bands3D damping_bands_3d(const double* vslice, const double* vtop, int64_t nz, int64_t nx, int64_t ny, int nB,
                         double dt) {
    Bands3D b;
    const double L = static_cast<double>(nB);
    b.zb.resize(static_cast<size_t>(nB) * nx);
    b.zbm1.resize(b.zb.size());
    b.xb.resize(static_cast<size_t>(nz) * 2 * nB);
    b.xbm1.resize(b.xb.size());
    b.yb.resize(static_cast<size_t>(nx) * 2 * nB);
    b.ybm1.resize(b.yb.size());
    for (int64_t j = 0; j < nx; ++j)
        for (int r = 0; r < nB; ++r) {
            const double d = damp_m_order(static_cast<double>(r + 1), vslice[(nz - nB + r) + j * nz], L);
            const double e = std::exp(-d * dt);
            b.zb[r + j * nB] = e;
            b.zbm1[r + j * nB] = e - 1;
        }
    for (int c = 0; c < 2 * nB; ++c) {
        const int64_t j = c < nB ? c : nx - nB + (c - nB);
        const double u = c < nB ? static_cast<double>(nB - c) : static_cast<double>(c - nB + 1);
        for (int64_t i = 0; i < nz; ++i) {
            const double d = damp_m_order(u, vslice[i + j * nz], L);
            const double e = std::exp(-d * dt);
            b.xb[i + c * nz] = e;
            b.xbm1[i + c * nz] = e - 1;
        }
    }
    for (int c = 0; c < 2 * nB; ++c) {
        const int64_t k = c < nB ? c : ny - nB + (c - nB);
        const double u = c < nB ? static_cast<double>(nB - c) : static_cast<double>(c - nB + 1);
        for (int64_t j = 0; j < nx; ++j) {
            const double d = damp_m_order(u, vtop[j + k * nx], L);
            const double e = std::exp(-d * dt);
            b.yb[j + c * nx] = e;
            b.ybm1[j + c * nx] = e - 1;
        }
    }
    return b;
}

// Composed second-derivative coefficients a_0..a_l of D-(D+ .) for weights w:
// coefficient of P(i+m) (= that of P(i-m)).
void composed_coefficients(const double* w, int N, double* a) {
    const int L = 2 * N - 1;
    for (int m = 0; m <= L; ++m) a[m] = 0.0;
    for (int k = 0; k < N; ++k)
        for (int n = 0; n < N; ++n) {
            const double ww = w[k] * w[n];
            a[k + n + 1] += ww;  // +P(i+k+n+1) and its mirror +P(i-1-k-n)
            // -P(i+k-n) and -P(i-k+n): over ordered pairs each |k-n| > 0 is met
            // twice (once per sign), while k = n puts both terms on P(i)
            const int d = k - n;
            a[d < 0 ? -d : d] -= (d == 0 ? 2.0 : 1.0) * ww;
        }
}



}  // namespace sssi

extern "C" int sssi_dCoef(int order, double* coeff) {
    return sssi::guarded([&] {
        SSSI_REQUIRE(order >= 1 && order <= 8, SSSI_ERR_ARG, "dCoef: order must be in 1..8 (got %d)", order);
        SSSI_REQUIRE(coeff != nullptr, SSSI_ERR_ARG, "dCoef: coeff is NULL");
        sssi::staggered_coefficients(order, coeff);
    });
}

extern "C" int sssi_dampPml(const double* u, const double* v, int64_t count, double L, double* d) {
    return sssi::guarded([&] {
        SSSI_REQUIRE(count >= 0 && (count == 0 || (u && v && d)), SSSI_ERR_ARG, "dampPml: bad arguments");
        for (int64_t q = 0; q < count; ++q) d[q] = sssi::damp_c_order(u[q], v[q], L);
    });
}
