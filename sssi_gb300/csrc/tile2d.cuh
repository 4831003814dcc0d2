// Tiled 2D CPML step (FP32 and fused FP64) for sm_103a.
//
// One persistent launch advances the grid by one time step.  Each CTA walks a
// strided list of TZ x TX tiles.  For every tile a single thread issues three
// TMA box copies into shared memory -- the current field with its halo (the
// P box: rows z0-HZ .. z0+TZ+HZ, columns x0-l .. x0+TX+l), the previous field
// and (v dt)^2 (TZ x TX each) -- double-buffered, so the copies of tile k+1
// overlap the arithmetic of tile k.  Each thread owns a block of 4 rows x RX
// columns and reads shared memory in 16-byte vectors: the z stencil of a
// column comes from one register window, the x stencil from RX + 2l column
// vectors streamed through registers.
//
// Interior tiles use the composed second-derivative stencil
//     Lz P(i) = a_0 P(i) + sum_{m=1..l} a_m (P(i+m) + P(i-m)),
// which is the staggered pair D-(D+ P) of the reference multiplied out (exact
// in real arithmetic wherever the CPML memory variables are zero).  Tiles whose
// stencil reaches a damped band use the two-stage form with the memory
// variables: A = D+P + phi, phi = b phi + (b-1) D+P, and D-A + psi.  In FP32
// the memory variables are carried as compensated (hi, lo) pairs; in FP64 as
// doubles.
#pragma once

#include "cpml2d.cuh"
#include "tma.cuh"

namespace sssi {

template <typename T>
struct TileShape;
// TZ x TX cells per tile; each thread owns 4 rows x RX columns; kMinBlocks
// CTAs per SM is the register budget the compiler is held to.
template <>
struct TileShape<float> {
    static constexpr int TZ = 64, TX = 32, RX = 2;
    static constexpr int kThreads = (TZ / 4) * (TX / RX), kMinBlocks = 2;
};
template <>
struct TileShape<double> {
    static constexpr int TZ = 32, TX = 32, RX = 2;
    static constexpr int kThreads = (TZ / 4) * (TX / RX), kMinBlocks = 2;
};

template <typename T>
struct MemVar;
template <>
struct MemVar<double> {
    using type = double;
};
template <>
struct MemVar<float> {
    using type = float2;  // compensated sum hi + lo
};

// Rows of halo above and below a tile in the P box: l rounded up to 4 so that
// every row window starts on a 16-byte boundary.
__host__ __device__ constexpr int tile_halo_rows(int N) { return ((2 * N - 1) + 3) / 4 * 4; }

template <typename T>
struct TileStep {
    using M = typename MemVar<T>::type;
    int nz, nx, nB;
    int ntz, ntx;  // tiles along z and x
    int oz;        // storage row of interior row 0
    int64_t ldp;
    int t, nt;
    T* Pnew;  // previous field, overwritten in place (interior origin)
    // bottom band nB x nx / side bands nz x 2nB (layouts as in Step2D)
    const T* zb;
    const T* zbm1;
    const M* zphi_in;
    M* zphi_out;
    M* zpsi;
    const T* xb;
    const T* xbm1;
    const M* xphi_in;
    M* xphi_out;
    M* xpsi;
    T az[16], ax[16];  // composed coefficients a_0 .. a_l
    T wz[8], wx[8];    // first-derivative weights c_k / d
    // sources, in T
    const T* src_dense;    // nz x nx slice of this step
    const T* src_row;      // nx values injected on row 0
    int nsrc;
    int src_iz[kMaxPointSources];
    int src_ix[kMaxPointSources];
    const T* src_wavelet;  // nsrc x nt
    // outputs, in T, and the RTM epilogue
    T* rec;
    T* snap;
    __half* pack;
    const unsigned* pack_amax;
    float* pack_inv_scale_out;
    unsigned* amax;
    const double* img_f64;
    const __half* img_f16;
    const float* img_inv_scale;
    double* img_m;   // FP64 image sums (fp64 mode)
    double* img_s2;
    float2* img_m2;  // compensated FP32 image sums (fp32 mode, with img_f16)
    float2* img_s22;
    int* err;  // set when a TMA copy does not arrive in time
};

// Device state of one 2D propagation on the tiled kernel.  Same interface as
// Cpml2d, so the C-ABI drivers are written once for both.
template <typename T>
class Tile2d {
  public:
    using value_type = T;
    using M = typename MemVar<T>::type;
    Tile2d(const double* v, int64_t nz, int64_t nx, int N, int nB, double dz, double dx, double dt, bool strict,
           cudaStream_t stream);
    void reset();
    void set_point_sources(int nsrc, const int64_t* iz, const int64_t* ix, const T* d_wavelet, int nt);
    void step(const StepIO<T>& io);
    void set_launch(int, int) {}
    // Throws if a kernel reported a failed TMA wait since the last reset.
    void check_errors();

    const T* current() const { return field(cur_); }
    const T* previous() const { return field(1 - cur_); }
    T* field(int k) const { return P_[k].as<T>() + origin_; }
    int64_t ldp() const { return ldp_; }
    int64_t padded_cols() const { return nx_ + 2 * L_; }
    int64_t origin() const { return origin_; }
    int L() const { return L_; }
    int64_t nz() const { return nz_; }
    int64_t nx() const { return nx_; }
    int grid() const { return grid_; }

  private:
    int64_t nz_, nx_;
    int N_, L_, nB_;
    cudaStream_t stream_;
    int64_t ldp_ = 0, origin_ = 0, oz_ = 0;
    int cur_ = 0, phase_ = 0;
    int grid_ = 0;
    DeviceBuffer P_[2], vdt2_, zb_, zbm1_, zphi_[2], zpsi_, xb_, xbm1_, xphi_[2], xpsi_, err_;
    CUtensorMap tm_box_[2], tm_tile_[2], tm_v_;
    TileStep<T> tmpl_{};
};

// Per-order pieces, explicitly instantiated in tile2d_{f32,f64}_{a,b}.cu.
template <typename T, int N>
void launch_tile2d_n(const CUtensorMap& tm_cur, const CUtensorMap& tm_old, const CUtensorMap& tm_v,
                     const TileStep<T>& p, int grid, cudaStream_t stream);
template <typename T, int N>
size_t tile2d_smem_n();
template <typename T, int N>
int tile2d_occupancy_n();

// Launches one step for order N (1..8).
template <typename T>
void launch_tile2d(int N, const CUtensorMap& tm_cur, const CUtensorMap& tm_old, const CUtensorMap& tm_v,
                   const TileStep<T>& p, int grid, cudaStream_t stream);

// CTAs of the tiled kernel for order N that fit on one SM.
template <typename T>
int tile2d_ctas_per_sm(int N);

}  // namespace sssi
