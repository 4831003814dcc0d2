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
}  // namespace

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_error, sizeof(g_error), fmt, ap);
    va_end(ap);
}

void clear_error() { g_error[0] = 0; }

void count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

cudaStream_t current_stream() { return g_stream; }

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

extern "C" const char* sssi_last_error(void) { return sssi::g_error; }

extern "C" int sssi_version(void) { return 10000 * 0 + 100 * 1 + 0; }

extern "C" int64_t sssi_launch_count(void) { return sssi::g_launches.load(); }

extern "C" int sssi_release_cache(void) {
    return sssi::guarded([] { sssi::pool_trim(); });
}

extern "C" int sssi_set_stream(void* stream) {
    return sssi::guarded([&] { sssi::g_stream = static_cast<cudaStream_t>(stream); });
}
