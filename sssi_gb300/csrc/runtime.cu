// Runtime services of libsssi_gb300: error text, the launch counter, the
// library stream, and the device-buffer cache.
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <map>
#include <mutex>

#include "sssi_internal.h"

namespace sssi {

namespace {
thread_local char g_error[1024] = "";
std::atomic<int64_t> g_launches{0};
cudaStream_t g_stream = nullptr;

// Cached device buffers keyed by exact size.  cudaMalloc/cudaFree synchronise
// the device and cost milliseconds for multi-GB buffers, so buffers of a shape
// used once are kept for the next call with the same shape.
std::mutex g_pool_mu;
std::multimap<size_t, void*> g_pool;
size_t g_pool_bytes = 0;

// phase timing
bool g_timing = false;
std::vector<cudaEvent_t> g_events;
std::vector<int64_t> g_marks;
int g_nmarks = 0;
std::vector<double> g_phase_ms;
std::vector<int64_t> g_phase_launches;
}  // namespace

void timing_begin(cudaStream_t s) {
    g_nmarks = 0;
    g_marks.clear();
    g_phase_ms.clear();
    g_phase_launches.clear();
    if (!g_timing) return;
    timing_mark(s);
}

void timing_mark(cudaStream_t s) {
    if (!g_timing) return;
    if ((int)g_events.size() <= g_nmarks) {
        cudaEvent_t e;
        SSSI_CHECK_CUDA(cudaEventCreate(&e));
        g_events.push_back(e);
    }
    SSSI_CHECK_CUDA(cudaEventRecord(g_events[g_nmarks], s));
    g_marks.push_back(g_launches.load());
    ++g_nmarks;
}

void timing_end(cudaStream_t s) {
    if (!g_timing) return;
    timing_mark(s);
    SSSI_CHECK_CUDA(cudaEventSynchronize(g_events[g_nmarks - 1]));
    for (int k = 1; k < g_nmarks; ++k) {
        float ms = 0.f;
        SSSI_CHECK_CUDA(cudaEventElapsedTime(&ms, g_events[k - 1], g_events[k]));
        g_phase_ms.push_back(ms);
        g_phase_launches.push_back(g_marks[k] - g_marks[k - 1]);
    }
}

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_error, sizeof(g_error), fmt, ap);
    va_end(ap);
}

void clear_error() { g_error[0] = 0; }

void count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

cudaStream_t current_stream() { return g_stream; }

namespace {
__global__ void store_int_kernel(int* p, int v) { *p = v; }
__global__ void add_int_kernel(int* p, int v) { *p += v; }
}  // namespace

void launch_store_int(int* p, int v, cudaStream_t s) {
    store_int_kernel<<<1, 1, 0, s>>>(p, v);
    SSSI_CHECK_CUDA(cudaGetLastError());
}

void launch_add_int(int* p, int v, cudaStream_t s) {
    add_int_kernel<<<1, 1, 0, s>>>(p, v);
    SSSI_CHECK_CUDA(cudaGetLastError());
}

cudaStream_t capture_stream() {
    static cudaStream_t cs = nullptr;
    static std::once_flag once;
    std::call_once(once, [] { SSSI_CHECK_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking)); });
    return cs;
}

std::mutex& capture_mutex() {
    static std::mutex m;
    return m;
}


void ensure_device() {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    SSSI_REQUIRE(e == cudaSuccess && n > 0, SSSI_ERR_CUDA, "no CUDA device available (%s)",
                 e == cudaSuccess ? "0 devices" : cudaGetErrorString(e));
}

bool is_device_pointer(const void* p) {
    if (!p) return false;
    cudaPointerAttributes a{};
    cudaError_t e = cudaPointerGetAttributes(&a, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

void DeviceBuffer::allocate(size_t bytes) {
    release();
    if (bytes == 0) return;
    {
        std::lock_guard<std::mutex> lk(g_pool_mu);
        auto it = g_pool.find(bytes);
        if (it != g_pool.end()) {
            ptr_ = it->second;
            g_pool.erase(it);
            g_pool_bytes -= bytes;
            bytes_ = bytes;
            return;
        }
    }
    cudaError_t e = cudaMalloc(&ptr_, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        // give the cache back to the driver and retry once
        pool_trim();
        e = cudaMalloc(&ptr_, bytes);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        ptr_ = nullptr;
        set_error("cudaMalloc of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
        throw Error{SSSI_ERR_NOMEM};
    }
    bytes_ = bytes;
}

void DeviceBuffer::release() {
    if (!ptr_) return;
    std::lock_guard<std::mutex> lk(g_pool_mu);
    g_pool.emplace(bytes_, ptr_);
    g_pool_bytes += bytes_;
    ptr_ = nullptr;
    bytes_ = 0;
}

void DeviceBuffer::zero(cudaStream_t s) {
    if (ptr_) SSSI_CHECK_CUDA(cudaMemsetAsync(ptr_, 0, bytes_, s));
}

void pool_trim() {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    cudaDeviceSynchronize();
    for (auto& kv : g_pool) cudaFree(kv.second);
    g_pool.clear();
    g_pool_bytes = 0;
}

size_t pool_cached_bytes() {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    return g_pool_bytes;
}

PinnedBuffer::~PinnedBuffer() {
    if (ptr_) cudaFreeHost(ptr_);
}

void PinnedBuffer::reserve(size_t bytes) {
    if (bytes <= bytes_) return;
    if (ptr_) cudaFreeHost(ptr_);
    ptr_ = nullptr;
    bytes_ = 0;
    SSSI_CHECK_CUDA(cudaMallocHost(&ptr_, bytes));
    bytes_ = bytes;
}

}  // namespace sssi

namespace sssi {
namespace {
std::atomic<int> g_debug_step{-1};
std::atomic<unsigned> g_debug_wait{0};
std::atomic<int> g_forced_shape{-1};
std::mutex g_sched3_mutex;
int g_sched3 = -1;
float g_sched3_ms[kSchedules3Max] = {};
}  // namespace

int forced_tile_shape() { return g_forced_shape.load(); }

void record_schedule3d(int chosen, const float* ms, int n) {
    std::lock_guard<std::mutex> lock(g_sched3_mutex);
    g_sched3 = chosen;
    for (int c = 0; c < kSchedules3Max; ++c) g_sched3_ms[c] = c < n ? ms[c] : 0.0f;
}

void debug_withhold(int* step, unsigned* wait_limit) {
    *step = g_debug_step.load();
    *wait_limit = g_debug_wait.load();
}
}  // namespace sssi

extern "C" int sssi_debug_withhold_copy(int step, unsigned wait_limit) {
    sssi::clear_error();
    sssi::g_debug_step.store(step < 0 ? -1 : step);
    sssi::g_debug_wait.store(wait_limit);
    return SSSI_OK;
}

extern "C" int sssi_debug_tile_shape(int shape) {
    sssi::clear_error();
    sssi::g_forced_shape.store(shape < 0 ? -1 : shape);
    return SSSI_OK;
}

extern "C" int sssi_debug_schedule3d(int* schedule, float* ms) {
    sssi::clear_error();
    if (!schedule || !ms) {
        sssi::set_error("sssi_debug_schedule3d: null argument");
        return SSSI_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(sssi::g_sched3_mutex);
    *schedule = sssi::g_sched3;
    for (int c = 0; c < sssi::kSchedules3Max; ++c) ms[c] = sssi::g_sched3_ms[c];
    return SSSI_OK;
}

extern "C" const char* sssi_last_error(void) { return sssi::g_error; }

extern "C" int sssi_version(void) { return 10000 * 0 + 100 * 1 + 0; }

extern "C" int64_t sssi_launch_count(void) { return sssi::g_launches.load(); }

extern "C" int sssi_release_cache(void) {
    return sssi::guarded([] { sssi::pool_trim(); });
}

extern "C" int sssi_enable_timing(int on) {
    return sssi::guarded([&] { sssi::g_timing = on != 0; });
}

extern "C" int sssi_last_timing(double* phase_ms, int64_t* phase_launches, int max_phases, int* n_phases) {
    return sssi::guarded([&] {
        const int n = (int)sssi::g_phase_ms.size();
        if (n_phases) *n_phases = n;
        for (int k = 0; k < n && k < max_phases; ++k) {
            if (phase_ms) phase_ms[k] = sssi::g_phase_ms[k];
            if (phase_launches) phase_launches[k] = sssi::g_phase_launches[k];
        }
    });
}

extern "C" int sssi_set_stream(void* stream) {
    return sssi::guarded([&] { sssi::g_stream = static_cast<cudaStream_t>(stream); });
}
