// 2D acoustic CPML step: kernel parameters and the propagator state object.
#pragma once

#include <cuda_fp16.h>

#include "divide.cuh"
#include "sssi_internal.h"

namespace sssi {

constexpr int kMaxOrder = 8;
constexpr int kMaxPointSources = 8;

// Everything one launch of the fused 2D step needs.  The wavefield is stored
// padded: element (i, j) of the interior (0 <= i < nz, 0 <= j < nx) lives at
// P[i + j*ldp] with P pointing at interior (0, 0); rows -l..-1 and nz..nz+l-1
// and columns -l..-1 and nx..nx+l-1 exist and hold zero forever.
template <typename T, typename TA>
struct Step2D {
    int nz, nx, nB;
    int W;        // columns marched by one block
    int64_t ldp;  // padded column length
    int t;        // time index of this step (source wavelets, imaging)
    int nt;       // wavelet length
    const T* P;   // current field
    T* Pold;      // previous field, overwritten in place with the new field
    const T* vdt2;  // (v*dt)^2, nz x nx

    // bottom CPML band, nB x nx: element (r, j) at r + j*nB, r = i - (nz-nB)
    const TA* zb;
    const TA* zbm1;
    const TA* zphi_in;
    TA* zphi_out;
    TA* zpsi;
    // side CPML bands, nz x 2nB: element (i, c) at i + c*nz, c = j (left) or nB + j-(nx-nB) (right)
    const TA* xb;
    const TA* xbm1;
    const TA* xphi_in;
    TA* xphi_out;
    TA* xpsi;

    // strict: c_k and the divisors; fast: w_k = c_k/d (divisors unused)
    T cz[kMaxOrder];
    T cx[kMaxOrder];
    Divisor<T> dz, dx;

    // sources added inside vdt2*(Pz + Px + src)
    const double* src_dense;  // nz x nx slice of this step, or null
    const double* src_row;    // nx values injected on row 0, or null
    const double* src_row_sub;  // subtracted from src_row (dataTrue - dataSmooth), or null
    int nsrc;
    int src_iz[kMaxPointSources];
    int src_ix[kMaxPointSources];
    const double* src_wavelet;  // nsrc x nt (row s at s*nt)

    // outputs of this step
    double* rec;   // nx: new field on row 0
    double* snap;  // nz x nx: new field
};

// Power-of-two scale that maps max|P| into [2^14, 2^15) for FP16 storage.
__host__ __device__ inline float fp16_scale_from_amax(unsigned amax_bits) {
    const int e = static_cast<int>((amax_bits >> 23) & 0xffu) - 127;  // amax in [2^e, 2^(e+1))
    if (amax_bits == 0u) return 1.0f;
    int ebias = 127 + 14 - e;
    if (ebias < 1) ebias = 1;
    if (ebias > 254) ebias = 254;
    union {
        unsigned u;
        float f;
    } c;
    c.u = static_cast<unsigned>(ebias) << 23;
    return c.f;
}

template <typename T>
struct Scalar;
template <>
struct Scalar<double> {
    static constexpr int kAlign = 16;  // elements per 128 bytes
};
template <>
struct Scalar<float> {
    static constexpr int kAlign = 32;
};

// Per-step inputs/outputs chosen by the caller, in the propagator's element
// type (conversions to and from double happen outside the step kernels).
template <typename T>
struct StepIO {
    const T* src_dense = nullptr;  // nz x nx source slice of this step
    const T* src_row = nullptr;    // nx values injected on row 0
    T* rec = nullptr;              // nx: new field on row 0
    T* snap = nullptr;             // nz x nx: new field
    int t = 0;
};

// Device state of one 2D propagation: two padded wavefields (current / old),
// (v dt)^2, the CPML band coefficients and memory variables.
template <typename T, typename TA>
class Cpml2d {
  public:
    using value_type = T;
    // v: nz x nx host array (column-major).
    Cpml2d(const double* v, int64_t nz, int64_t nx, int N, int nB, double dz, double dx, double dt, bool strict,
           cudaStream_t stream);

    void reset();  // zero fields and memory variables
    void set_point_sources(int nsrc, const int64_t* iz, const int64_t* ix, const T* d_wavelet, int nt);
    void step(const StepIO<T>& io);

    // Field after the last step (padded storage; interior (0,0) at offset).
    const T* current() const { return field(cur_); }
    const T* previous() const { return field(1 - cur_); }
    T* field(int k) const { return P_[k].as<T>() + origin_; }
    int64_t ldp() const { return ldp_; }
    int64_t padded_cols() const { return nx_ + 2 * L_; }
    int64_t origin() const { return origin_; }
    T* base(int k) const { return P_[k].as<T>(); }
    int L() const { return L_; }
    int64_t nz() const { return nz_; }
    int64_t nx() const { return nx_; }

    void set_launch(int bz, int w) {
        bz_ = bz;
        w_ = w;
    }
    void check_errors() {}

  private:
    int64_t nz_, nx_;
    int N_, L_, nB_;
    bool strict_;
    cudaStream_t stream_;
    int64_t ldp_ = 0, origin_ = 0;
    int cur_ = 0, phase_ = 0;
    int bz_ = 128, w_ = 64;
    DeviceBuffer P_[2], vdt2_, zb_, zbm1_, zphi_[2], zpsi_, xb_, xbm1_, xphi_[2], xpsi_;
    Step2D<T, TA> tmpl_{};
};

// Launches one step of the kernel instance for (T, TA, N, strict).
template <typename T, typename TA>
void launch_cpml2d_step(const Step2D<T, TA>& p, int N, bool strict, int bz, cudaStream_t stream);

// Same launch, reporting failure as a return value instead of an exception.
template <typename T, typename TA>
cudaError_t launch_cpml2d_step_nothrow(const Step2D<T, TA>& p, int N, bool strict, int bz, cudaStream_t stream);

// Packs field P (padded, interior origin) into FP16 with the scale from *amax.
// FP16 copy of the padded FP32 field P (nz x nx interior, column pitch ldp)
// with one power-of-two scale per 32 x 32 block, from the block maxima amax
// (index bz + bx * ceil(nz / 32)); err (nz x nx) carries each cell's rounding
// error from one stored step to the next.
void launch_pack_f16(const float* P, int64_t ldp, int nz, int nx, const unsigned* amax, __half* out, float* err,
                     cudaStream_t stream);

}  // namespace sssi
