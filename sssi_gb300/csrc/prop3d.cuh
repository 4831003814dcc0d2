// 3D CPML propagation (fwdTimeCpmlFor3dAw.m): one launch per time step over
// the whole volume, persistent blocks marching along y.
//
// Work item: a TZ x TX tile of the (z, x) plane and a chunk of planes along
// y (chunks cut per tile by estimated cost, so that the items fill the GPU and
// tiles next to the damped bands get shorter chunks).  For each output plane the block copies that plane's P tile with its z
// and x halo, and its P_old and (v dt)^2 tiles, into shared memory (TMA, ring
// of kStages planes), together with the tile's own cells of P at plane
// y+2N-1, which enter the y queue; the z and x
// second derivatives come from it (composed stencil, or the two-stage form
// with the memory variables in tiles that reach a damped band).  The y
// derivatives always use the two-stage form out of per-thread register
// queues: P at planes y .. y+2N-1 and A_y = D+_y P (+ phi_y) at planes
// y-N .. y+N-1, so each plane of the chunk is read once per thread.
//
// Layout in HBM:
//   fields P (two buffers), (v dt)^2: padded Nzp x Nxp x Nyp, column-major
//   (z fastest), interior origin at (HZ, L, L); HZ is a multiple of 4, so
//   rows stay 16-byte aligned for vector loads and TMA coordinates;
//   band coefficients b, b-1 (2D): z: nB x nx, x: nz x 2nB, y: nx x 2nB
//   (the MATLAB profiles vary in two dimensions only);
//   memory variables phi (two buffers: halo cells are read by neighbouring
//   items while their owners update them) and psi: z: nB x nx x ny,
//   x: nz x 2nB x ny, y: nz x nx x 2nB.
#pragma once

#include <cuda_fp16.h>
#include <cudaTypedefs.h>

#include "sssi_internal.h"
#include "tile2d.cuh"

namespace sssi {

template <typename T>
struct Shape3D;
template <>
struct Shape3D<float> {
    static constexpr int TZ = 32, TX = 32, RZ = 4;  // tile, rows per thread
    static constexpr int kThreads = (TZ / RZ) * TX;
    static constexpr int kMinBlocks = 2;
};
template <>
struct Shape3D<double> {
    static constexpr int TZ = 16, TX = 32, RZ = 2;
    static constexpr int kThreads = (TZ / RZ) * TX;
    static constexpr int kMinBlocks = 1;
};

// CPML memory variables of the 3D propagator: one word of the field's type.
// (The 2D FP32 forms carry theirs as compensated pairs for the RTM residual;
// the 3D propagator models forward only, where plain FP32 memory variables
// leave the receivers within a few 1e-7 of FP64.)
template <typename T>
struct MemVar3 {
    using type = T;
};

// Candidate work-item schedules of a 3D propagation, timed on its first steps.
constexpr int kSchedules3 = kSchedules3Max;

template <typename T>
struct Desc3 {
    using M = typename MemVar3<T>::type;
    CUtensorMap tm_plane[2];  // plane tile of field k with its z/x halo
    CUtensorMap tm_tile[2];   // plane tile of field k without halo (P_old)
    CUtensorMap tm_v;         // plane tile of (v dt)^2
    T* field[2];              // interior origin of field k; field (t & 1) is current at step t
    const T* vdt2;            // interior origin of (v dt)^2
    int64_t ldz;              // Nzp: stride of x
    int64_t ldxy;             // Nzp * Nxp: stride of y
    int nz, nx, ny, nB, nt;
    int ntz, ntx;          // tiles along z and x
    int zs;                // tile rows start at row -zs (Prop3d: the bottom band's rows in one tile row)
    const int2* order[kSchedules3];  // work items (tile, y0 | y1 << 16: planes y0 .. y1-1), most expensive
                                     // first, of each candidate schedule (Const3::sched picks one)
    int* next;             // two counters: items taken at steps of parity 0 / 1
    // band coefficients (2D) and memory variables (3D), see the file header
    const T *zb, *zbm1, *xb, *xbm1, *yb, *ybm1;
    M *zphi[2], *zpsi, *xphi[2], *xpsi, *yphi[2], *ypsi;
    // sources: dense slices (nz x nx x ny per step, from dense_t0 on), points
    const T* src_dense;
    int dense_t0;
    int nsrc;
    int src_iz[kMaxPointSources], src_ix[kMaxPointSources], src_iy[kMaxPointSources];
    const T* src_wavelet;    // nsrc x nt
    T* rec;                  // nx x ny per step: the top interior face after the step
    T* snap;                 // nz x nx x ny per step from snap_t0 on
    int snap_t0;
};

template <typename T>
struct Const3 {
    T az[16], ax[16];  // composed second-derivative coefficients (z, x)
    T wz[8], wx[8], wy[8];
    // D- along y over the A_y queue: row u (queue position of the step) holds
    // the weight of each of the 2N slots, so the slots are read in a fixed order
    T wyq[16 * 16];
    // FP32: the same coefficients as pairs {c, c}, operands of the two-cell
    // (packed) instructions
    float2 az2[16], ax2[16], wy2[8], wyq2[16 * 16];
    int nitems;
    int sched;             // the schedule in use (Desc3::order)
    const int* step_base;  // the launch computes step *step_base + step_offset
    int step_offset;
    int* err;
};

// Host driver of one 3D propagation.
template <typename T>
class Prop3d {
  public:
    using M = typename MemVar3<T>::type;
    Prop3d(const double* v, int64_t nz, int64_t nx, int64_t ny, int N, int nB, double dz, double dx, double dy,
           double dt, int nt, cudaStream_t stream);
    ~Prop3d();
    Prop3d(const Prop3d&) = delete;
    Prop3d& operator=(const Prop3d&) = delete;

    Desc3<T>& desc() { return desc_; }
    void set_point_sources(int nsrc, const int64_t* iz, const int64_t* ix, const int64_t* iy, const T* d_wavelet);
    // Stream of the later launches and copies (set up on another stream, the
    // caller orders this one after it).
    void set_stream(cudaStream_t s) { stream_ = s; }
    void sync_desc();
    // Whole runs of kGraphSteps go through a CUDA graph.  The first steps of a
    // long run time the candidate schedules (even chunks along y with about
    // three items per resident block, or chunks cut by estimated cost per tile
    // with about three, two or four); the fastest is kept.
    void run(int nsteps);
    void check_errors();
    int schedule() const { return cc_.sched; }
    float tune_ms(int c) const { return tune_ms_[c]; }
    const T* current_field() const { return desc_.field[step_ & 1]; }
    int step() const { return step_; }
    static constexpr int kGraphSteps = 16;

  private:
    void launch_step(const int* base, int offset, cudaStream_t s);
    void use_schedule(int c);
    int N_;
    cudaStream_t stream_;
    Desc3<T> desc_{};
    Const3<T> cc_{};
    DeviceBuffer P_[2], vdt2_, zb_, zbm1_, xb_, xbm1_, yb_, ybm1_, zphi_[2], zpsi_, xphi_[2], xpsi_, yphi_[2], ypsi_;
    DeviceBuffer d_desc_, d_ctr_, d_order_[kSchedules3], d_next_;
    int nitems_[kSchedules3] = {}, grid_c_[kSchedules3] = {};
    int grid_ = 0, step_ = 0;
    cudaGraphExec_t graph_ = nullptr;
    // schedule tuning: phase 0 warm-up, 1 .. kSchedules3 timing schedule
    // phase-1, kTuneWait waiting for the timings, kTuneDone done
    static constexpr int kTuneSteps = 6, kTuneMinSteps = 64;
    static constexpr int kTuneWait = kSchedules3 + 1, kTuneDone = kSchedules3 + 2;
    int tune_ = 0, tune_left_ = 2;
    cudaEvent_t tev_[2 * kSchedules3] = {};  // start and end of each timed run
    float tune_ms_[kSchedules3] = {};        // the timed runs (ms), 0 until tuned
};

template <typename T, int N>
void launch_prop3d_n(const Desc3<T>* d, const Const3<T>& c, int grid, cudaStream_t stream);
template <typename T, int N>
int prop3d_occupancy_n();

}  // namespace sssi
