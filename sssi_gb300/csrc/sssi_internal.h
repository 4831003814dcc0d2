// Internal declarations shared by the translation units of libsssi_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <cmath>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "sssi_gb300.h"

namespace sssi {

// ---------------------------------------------------------------- errors
// Every C-ABI entry point returns a status code; the text of the last failure
// of the calling thread is kept for sssi_last_error().
void set_error(const char* fmt, ...);
void clear_error();

struct Error {
    int code;
};

#define SSSI_CHECK_CUDA(expr)                                                                   \
    do {                                                                                        \
        cudaError_t e_ = (expr);                                                                \
        if (e_ != cudaSuccess) {                                                                \
            ::sssi::set_error("%s failed: %s (%s:%d)", #expr, cudaGetErrorString(e_), __FILE__, \
                              __LINE__);                                                        \
            throw ::sssi::Error{SSSI_ERR_CUDA};                                                 \
        }                                                                                       \
    } while (0)

#define SSSI_REQUIRE(cond, code, ...)      \
    do {                                   \
        if (!(cond)) {                     \
            ::sssi::set_error(__VA_ARGS__); \
            throw ::sssi::Error{code};     \
        }                                  \
    } while (0)

// Runs f, translating exceptions into a status code (C-ABI boundary helper).
template <typename F>
int guarded(F&& f) {
    clear_error();
    try {
        f();
        return SSSI_OK;
    } catch (const Error& e) {
        return e.code;
    } catch (const std::bad_alloc&) {
        set_error("host allocation failed");
        return SSSI_ERR_NOMEM;
    } catch (...) {
        set_error("unexpected C++ exception");
        return SSSI_ERR_INTERNAL;
    }
}

// ---------------------------------------------------------------- runtime
void count_launch(int n = 1);
// The test knob of sssi_debug_withhold_copy (step < 0: off).
void debug_withhold(int* step, unsigned* wait_limit);
// The test knob of sssi_debug_tile_shape (-1: the tuner chooses).
int forced_tile_shape();
// The last 3D schedule choice and the timed runs behind it (sssi_debug_schedule3d).
constexpr int kSchedules3Max = 4;
void record_schedule3d(int chosen, const float* ms, int n);
// One-thread kernels that set / advance a device int (graph step bases).
void launch_store_int(int* p, int v, cudaStream_t s);
void launch_add_int(int* p, int v, cudaStream_t s);
// A non-blocking stream used only to record CUDA graphs (capture runs nothing;
// the legacy default stream cannot be captured), and the lock held while
// recording on it.
cudaStream_t capture_stream();
std::mutex& capture_mutex();
cudaStream_t current_stream();
bool is_device_pointer(const void* p);
void ensure_device();

// Device memory from a per-process cache keyed by size: buffers are returned to
// the cache at the end of a call and reused by the next call of the same shape.
class DeviceBuffer {
  public:
    DeviceBuffer() = default;
    explicit DeviceBuffer(size_t bytes) { allocate(bytes); }
    ~DeviceBuffer() { release(); }
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    DeviceBuffer(DeviceBuffer&& o) noexcept : ptr_(o.ptr_), bytes_(o.bytes_) {
        o.ptr_ = nullptr;
        o.bytes_ = 0;
    }
    DeviceBuffer& operator=(DeviceBuffer&& o) noexcept {
        if (this != &o) {
            release();
            ptr_ = o.ptr_;
            bytes_ = o.bytes_;
            o.ptr_ = nullptr;
            o.bytes_ = 0;
        }
        return *this;
    }
    void allocate(size_t bytes);
    void release();
    void zero(cudaStream_t s);
    template <typename T>
    T* as() const {
        return static_cast<T*>(ptr_);
    }
    void* get() const { return ptr_; }
    size_t bytes() const { return bytes_; }

  private:
    void* ptr_ = nullptr;
    size_t bytes_ = 0;
};

// Phase boundaries of the current call (no-ops unless timing is enabled).
void timing_begin(cudaStream_t s);
void timing_mark(cudaStream_t s);
void timing_end(cudaStream_t s);

// Releases every cached buffer (sssi_release_cache).
void pool_trim();
size_t pool_cached_bytes();

// Pinned host staging buffer (reused across calls).
class PinnedBuffer {
  public:
    PinnedBuffer() = default;
    ~PinnedBuffer();
    void reserve(size_t bytes);
    void* get() const { return ptr_; }

  private:
    void* ptr_ = nullptr;
    size_t bytes_ = 0;
};

// ---------------------------------------------------------------- host setup
// Staggered-grid coefficients of half-order N: A c = e1, A_ij = (2j-1)^(2i-1),
// by LU with partial pivoting (finiteDifference.c:24-82).
void staggered_coefficients(int N, double* c);

// d = (-(3 v)/(2 L) * log(1e-6)) * (u/L) * (u/L)   (finiteDifference.c:253-280)
double damp_c_order(double u, double v, double L);
// d = d0 .* (u/L).^2                              (src/dampPml.m:16-18)
double damp_m_order(double u, double v, double L);

// (v dt)^2 of the nz x nx x ny device model v into a padded layout (interior
// origin `out`, strides ldz along x and ldxy along y), on stream s.
template <typename T>
void launch_vdt2(const double* v, int64_t nz, int64_t nx, int64_t ny, double dt, T* out, int64_t ldz, int64_t ldxy,
                 cudaStream_t s);

// Damping factors of the CPML bands of a 2D grid, C-gateway conventions
// (fwdTimeCpmlFor2dAw_mex.c:100-145).  Bottom band: nB x nx (row r = i-(nz-nB)),
// side bands: nz x 2nB (column c = j for the left band, nB + j-(nx-nB) for the right).
struct Bands2D {
    std::vector<double> zb, zbm1;  // nB x nx
    std::vector<double> xb, xbm1;  // nz x 2nB
};
Bands2D damping_bands_2d(const double* v, int64_t nz, int64_t nx, int nB, double dz, double dx, double dt);
// The same from the velocities the bands read: bottom = rows nz-nB .. nz-1
// (nB x nx), sides = columns 0 .. nB-1 then nx-nB .. nx-1 (nz x 2nB).
Bands2D damping_bands_2d_strips(const double* bottom, const double* sides, int64_t nz, int64_t nx, int nB, double dz,
                                double dx, double dt);

// Damping factors of the 3D MATLAB file (src/fwdTimeCpmlFor3dAw.m:45-70):
// cell units (L = nB), x profiles from the y=0 slice, y profiles from the top row,
// z profiles from the y=0 slice.  Bottom band: nB x nx (same for every y);
// x bands: nz x 2nB (same for every y); y bands: nx x 2nB (same for every z).
struct Bands3D {
    std::vector<double> zb, zbm1;  // nB x nx
    std::vector<double> xb, xbm1;  // nz x 2nB
    std::vector<double> yb, ybm1;  // nx x 2nB
};
// vslice: v on the y = 0 slice (nz x nx); vtop: v on row 0 of every column
// (nx x ny) -- the only velocities the profiles read.
Bands3D damping_bands_3d(const double* vslice, const double* vtop, int64_t nz, int64_t nx, int64_t ny, int nB,
                         double dt);

// Composed second-derivative coefficients a_0..a_l (l = 2N-1) of D-(D+ .) for
// the first-derivative weights w_0..w_{N-1}: coefficient of P(i+m) (= of P(i-m)).
void composed_coefficients(const double* w, int N, double* a);

// Band coefficients in T.  In FP32, b - 1 comes from expm1 so it keeps full
// relative precision where b is close to 1.
template <typename T>
inline void band_coefficients(const std::vector<double>& b, const std::vector<double>& bm1, std::vector<T>& ob,
                       std::vector<T>& obm1) {
    ob.resize(b.size());
    obm1.resize(b.size());
    for (size_t k = 0; k < b.size(); ++k) {
        ob[k] = static_cast<T>(b[k]);
        if constexpr (std::is_same<T, float>::value)
            obm1[k] = static_cast<float>(std::expm1(std::log(b[k])));
        else
            obm1[k] = bm1[k];
    }
}


}  // namespace sssi
