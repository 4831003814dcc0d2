// MAT-file (Level 5) persistence of the applications' arrays: the seismograms,
// images and snapshots that applications/rtm_2d_acoustic/mainRtmTimeCpmlFor2dAw.m
// saves and loads (:170-183, :250-266, :348-351) with MATLAB's save/load.
//
// The applications write MATLAB's HDF5-based v7.3 files; MATLAB's `load` also
// reads the Level-5 format written here (an 128-byte header, then one
// miMATRIX element per variable: array flags, dimensions, name, real part), and
// `save(..., '-v6')` writes what the reader takes.  The writer streams each
// array from host or device memory to the file through a bounded staging
// buffer, so a device-resident image or record goes to disk without a full
// host copy; the reader fills a host or device array the same way.  Limits of
// the format: a variable's element holds at most 2^32 - 1 bytes (about 536 M
// doubles); compressed (v7) elements are refused with a message.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "sssi_internal.h"

namespace sssi {
namespace {

constexpr uint32_t miINT8 = 1, miUINT8 = 2, miINT16 = 3, miUINT16 = 4, miINT32 = 5, miUINT32 = 6, miSINGLE = 7,
                   miDOUBLE = 9, miINT64 = 12, miUINT64 = 13, miMATRIX = 14, miCOMPRESSED = 15;
constexpr uint32_t mxDOUBLE_CLASS = 6;
constexpr size_t kStage = size_t(64) << 20;  // bytes staged per device copy

struct File {
    FILE* f = nullptr;
    explicit File(const char* path, const char* mode) : f(std::fopen(path, mode)) {}
    ~File() {
        if (f) std::fclose(f);
    }
};

void put(FILE* f, const void* p, size_t n, const char* path) {
    SSSI_REQUIRE(std::fwrite(p, 1, n, f) == n, SSSI_ERR_ARG, "writing %s failed", path);
}

void get(FILE* f, void* p, size_t n, const char* path) {
    SSSI_REQUIRE(std::fread(p, 1, n, f) == n, SSSI_ERR_ARG, "%s: unexpected end of file", path);
}

void pad8(FILE* f, uint64_t n, const char* path) {
    static const char zero[8] = {0};
    if (n % 8) put(f, zero, 8 - n % 8, path);
}

void tag(FILE* f, uint32_t type, uint32_t bytes, const char* path) {
    const uint32_t t[2] = {type, bytes};
    put(f, t, 8, path);
}

// Copies n doubles from src (host or device) to the file, staging device data.
void write_doubles(FILE* f, const double* src, uint64_t n, const char* path) {
    if (n == 0) return;
    if (!is_device_pointer(src)) {
        put(f, src, n * sizeof(double), path);
        return;
    }
    std::vector<double> buf(std::min<uint64_t>(n, kStage / sizeof(double)));
    for (uint64_t q = 0; q < n; q += buf.size()) {
        const uint64_t k = std::min<uint64_t>(buf.size(), n - q);
        SSSI_CHECK_CUDA(cudaMemcpy(buf.data(), src + q, k * sizeof(double), cudaMemcpyDeviceToHost));
        put(f, buf.data(), k * sizeof(double), path);
    }
}

template <typename S>
void convert_chunk(const unsigned char* in, double* out, uint64_t k) {
    for (uint64_t i = 0; i < k; ++i) {
        S v;
        std::memcpy(&v, in + i * sizeof(S), sizeof(S));
        out[i] = (double)v;
    }
}

size_t type_size(uint32_t type) {
    switch (type) {
        case miINT8:
        case miUINT8: return 1;
        case miINT16:
        case miUINT16: return 2;
        case miINT32:
        case miUINT32:
        case miSINGLE: return 4;
        case miDOUBLE:
        case miINT64:
        case miUINT64: return 8;
        default: return 0;
    }
}

// Reads n values of the stored type into dst (host or device) as doubles.
// MATLAB may store a double array in a narrower type when its values allow.
void read_values(FILE* f, uint32_t type, double* dst, uint64_t n, const char* path) {
    const size_t es = type_size(type);
    SSSI_REQUIRE(es != 0, SSSI_ERR_ARG, "%s: unsupported data type %u in a numeric array", path, type);
    const bool dev = is_device_pointer(dst);
    const uint64_t chunk = std::max<uint64_t>(1, kStage / 8);
    std::vector<unsigned char> raw((size_t)std::min<uint64_t>(n, chunk) * es);
    std::vector<double> vals((size_t)std::min<uint64_t>(n, chunk));
    for (uint64_t q = 0; q < n; q += chunk) {
        const uint64_t k = std::min<uint64_t>(chunk, n - q);
        get(f, raw.data(), (size_t)(k * es), path);
        double* out = dev ? vals.data() : dst + q;
        switch (type) {
            case miDOUBLE: std::memcpy(out, raw.data(), (size_t)(k * 8)); break;
            case miSINGLE: convert_chunk<float>(raw.data(), out, k); break;
            case miINT8: convert_chunk<int8_t>(raw.data(), out, k); break;
            case miUINT8: convert_chunk<uint8_t>(raw.data(), out, k); break;
            case miINT16: convert_chunk<int16_t>(raw.data(), out, k); break;
            case miUINT16: convert_chunk<uint16_t>(raw.data(), out, k); break;
            case miINT32: convert_chunk<int32_t>(raw.data(), out, k); break;
            case miUINT32: convert_chunk<uint32_t>(raw.data(), out, k); break;
            case miINT64: convert_chunk<int64_t>(raw.data(), out, k); break;
            default: convert_chunk<uint64_t>(raw.data(), out, k); break;
        }
        if (dev) SSSI_CHECK_CUDA(cudaMemcpy(dst + q, vals.data(), (size_t)(k * 8), cudaMemcpyHostToDevice));
    }
}

// One sub-element tag: type and byte count, in the small-element form when the
// upper 16 bits of the first word are set (data in the following 4 bytes).
struct Sub {
    uint32_t type = 0, bytes = 0;
    bool small = false;
    unsigned char inl[4] = {0, 0, 0, 0};
};

Sub read_sub(FILE* f, const char* path) {
    uint32_t w[2];
    get(f, w, 8, path);
    Sub s;
    if (w[0] >> 16) {
        s.small = true;
        s.type = w[0] & 0xffffu;
        s.bytes = w[0] >> 16;
        std::memcpy(s.inl, &w[1], 4);
    } else {
        s.type = w[0];
        s.bytes = w[1];
    }
    return s;
}

void skip(FILE* f, uint64_t n, const char* path) {
    SSSI_REQUIRE(std::fseek(f, (long)n, SEEK_CUR) == 0, SSSI_ERR_ARG, "%s: seek failed", path);
}

}  // namespace
}  // namespace sssi

using namespace sssi;

extern "C" {

int sssi_mat_write(const char* path, int nvars, const char* const* names, const double* const* arrays,
                   const int* ndims, const int64_t* const* dims) {
    return guarded([&] {
        SSSI_REQUIRE(path && nvars >= 0 && (nvars == 0 || (names && arrays && ndims && dims)), SSSI_ERR_ARG,
                     "sssi_mat_write: path, names, arrays, ndims and dims are required");
        for (int v = 0; v < nvars; ++v) {
            SSSI_REQUIRE(names[v] && std::strlen(names[v]) > 0 && std::strlen(names[v]) <= 63, SSSI_ERR_ARG,
                         "variable %d: a name of 1 to 63 characters is required", v);
            SSSI_REQUIRE(ndims[v] >= 1 && ndims[v] <= 8, SSSI_ERR_ARG, "variable %s: ndims must be 1..8", names[v]);
            uint64_t n = 1;
            constexpr uint64_t kMaxElems = ((uint64_t(1) << 32) - 256) / 8;  // the element's 32-bit byte count
            for (int d = 0; d < ndims[v]; ++d) {
                SSSI_REQUIRE(dims[v][d] >= 0 && dims[v][d] < (int64_t(1) << 31), SSSI_ERR_ARG,
                             "variable %s: dimension %d out of range", names[v], d);
                const uint64_t e = (uint64_t)dims[v][d];
                n = (e != 0 && n > kMaxElems / e) ? kMaxElems + 1 : n * e;
            }
            SSSI_REQUIRE(n <= kMaxElems, SSSI_ERR_ARG,
                         "variable %s exceeds the Level-5 element limit (4 GiB)", names[v]);
            SSSI_REQUIRE(n == 0 || arrays[v], SSSI_ERR_ARG, "variable %s: no data", names[v]);
        }
        File F(path, "wb");
        SSSI_REQUIRE(F.f, SSSI_ERR_ARG, "cannot open %s for writing", path);
        char head[128];
        std::memset(head, ' ', 116);
        const char* text = "MATLAB 5.0 MAT-file, written by libsssi_gb300";
        std::memcpy(head, text, std::strlen(text));
        std::memset(head + 116, 0, 8);  // no subsystem data
        const uint16_t version = 0x0100, endian = ('M' << 8) | 'I';
        std::memcpy(head + 124, &version, 2);
        std::memcpy(head + 126, &endian, 2);
        put(F.f, head, 128, path);
        for (int v = 0; v < nvars; ++v) {
            const int nd = ndims[v] == 1 ? 2 : ndims[v];  // MATLAB arrays have at least two dimensions
            std::vector<int32_t> dv((size_t)nd, 1);
            uint64_t n = 1;
            for (int d = 0; d < ndims[v]; ++d) {
                dv[(size_t)d] = (int32_t)dims[v][d];
                n *= (uint64_t)dims[v][d];
            }
            const uint32_t namelen = (uint32_t)std::strlen(names[v]);
            auto padded = [](uint64_t b) { return (b + 7) / 8 * 8; };
            const uint64_t body = 16 + 8 + padded(4ull * nd) + 8 + padded(namelen) + 8 + padded(n * 8);
            tag(F.f, miMATRIX, (uint32_t)body, path);
            tag(F.f, miUINT32, 8, path);
            const uint32_t flags[2] = {mxDOUBLE_CLASS, 0};
            put(F.f, flags, 8, path);
            tag(F.f, miINT32, 4u * (uint32_t)nd, path);
            put(F.f, dv.data(), 4u * (size_t)nd, path);
            pad8(F.f, 4ull * nd, path);
            tag(F.f, miINT8, namelen, path);
            put(F.f, names[v], namelen, path);
            pad8(F.f, namelen, path);
            tag(F.f, miDOUBLE, (uint32_t)(n * 8), path);
            write_doubles(F.f, arrays[v], n, path);
        }
        SSSI_REQUIRE(std::fflush(F.f) == 0, SSSI_ERR_ARG, "writing %s failed", path);
    });
}

int sssi_mat_read(const char* path, const char* name, double* out, int64_t capacity, int* ndims, int64_t* dims) {
    return guarded([&] {
        SSSI_REQUIRE(path && name && ndims && dims, SSSI_ERR_ARG, "sssi_mat_read: path, name, ndims and dims required");
        File F(path, "rb");
        SSSI_REQUIRE(F.f, SSSI_ERR_ARG, "cannot open %s", path);
        char head[128];
        get(F.f, head, 128, path);
        uint16_t endian;
        std::memcpy(&endian, head + 126, 2);
        SSSI_REQUIRE(endian == (('M' << 8) | 'I'), SSSI_ERR_ARG,
                     "%s: not a little-endian Level-5 MAT-file (v7.3 files are HDF5: save with -v6 instead)", path);
        for (;;) {
            uint32_t w[2];
            if (std::fread(w, 1, 8, F.f) != 8) break;
            const uint32_t type = w[0], bytes = w[1];
            SSSI_REQUIRE(type != miCOMPRESSED, SSSI_ERR_ARG,
                         "%s: compressed (v7) elements are not read here: save with -v6", path);
            if (type != miMATRIX) {
                skip(F.f, (bytes + 7) / 8 * 8, path);
                continue;
            }
            const long start = std::ftell(F.f);
            read_sub(F.f, path);  // the array flags' tag (miUINT32, 8 bytes)
            uint32_t fl[2];
            get(F.f, fl, 8, path);
            const uint32_t cls = fl[0] & 0xffu;
            const bool complex = (fl[0] >> 11) & 1u;
            Sub dsub = read_sub(F.f, path);
            std::vector<int32_t> dv(dsub.bytes / 4);
            if (dsub.small) {
                std::memcpy(dv.data(), dsub.inl, dsub.bytes);
            } else {
                get(F.f, dv.data(), dsub.bytes, path);
                skip(F.f, (dsub.bytes + 7) / 8 * 8 - dsub.bytes, path);
            }
            Sub nsub = read_sub(F.f, path);
            std::string vname;
            if (nsub.small) {
                vname.assign(reinterpret_cast<const char*>(nsub.inl), nsub.bytes);
            } else {
                vname.resize(nsub.bytes);
                get(F.f, &vname[0], nsub.bytes, path);
                skip(F.f, (nsub.bytes + 7) / 8 * 8 - nsub.bytes, path);
            }
            if (vname != name) {
                SSSI_REQUIRE(std::fseek(F.f, start + (long)((bytes + 7) / 8 * 8), SEEK_SET) == 0, SSSI_ERR_ARG,
                             "%s: seek failed", path);
                continue;
            }
            SSSI_REQUIRE(cls >= 6 && cls <= 15 && !complex, SSSI_ERR_ARG,
                         "%s: variable %s is not a real numeric array (class %u)", path, name, cls);
            SSSI_REQUIRE(dv.size() <= 8, SSSI_ERR_ARG, "%s: variable %s has more than 8 dimensions", path, name);
            uint64_t n = 1;
            *ndims = (int)dv.size();
            for (size_t d = 0; d < dv.size(); ++d) {
                dims[d] = dv[d];
                n *= (uint64_t)dv[d];
            }
            if (!out) return;  // a size query
            SSSI_REQUIRE((int64_t)n <= capacity, SSSI_ERR_ARG, "%s: variable %s has %llu elements, capacity %lld",
                         path, name, (unsigned long long)n, (long long)capacity);
            Sub real = read_sub(F.f, path);
            const size_t es = type_size(real.type);
            SSSI_REQUIRE(es != 0 && real.bytes == n * es, SSSI_ERR_ARG, "%s: variable %s: bad real part", path,
                         name);
            if (real.small) {
                std::vector<double> tmp((size_t)n);
                unsigned char in[4];
                std::memcpy(in, real.inl, 4);
                for (uint64_t i = 0; i < n; ++i) {
                    switch (real.type) {
                        case miINT8: tmp[i] = (double)(int8_t)in[i]; break;
                        case miUINT8: tmp[i] = (double)in[i]; break;
                        case miINT16: { int16_t x; std::memcpy(&x, in + 2 * i, 2); tmp[i] = x; break; }
                        case miUINT16: { uint16_t x; std::memcpy(&x, in + 2 * i, 2); tmp[i] = x; break; }
                        case miINT32: { int32_t x; std::memcpy(&x, in, 4); tmp[i] = x; break; }
                        case miUINT32: { uint32_t x; std::memcpy(&x, in, 4); tmp[i] = x; break; }
                        case miSINGLE: { float x; std::memcpy(&x, in, 4); tmp[i] = x; break; }
                        default: SSSI_REQUIRE(false, SSSI_ERR_ARG, "%s: bad small element", path);
                    }
                }
                if (is_device_pointer(out))
                    SSSI_CHECK_CUDA(cudaMemcpy(out, tmp.data(), n * 8, cudaMemcpyHostToDevice));
                else
                    std::memcpy(out, tmp.data(), n * 8);
            } else {
                read_values(F.f, real.type, out, n, path);
            }
            return;
        }
        SSSI_REQUIRE(false, SSSI_ERR_ARG, "%s: no variable named %s", path, name);
    });
}

}  // extern "C"
