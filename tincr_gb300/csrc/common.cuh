// Shared helpers of the tincr_gb300 CUDA library: status handling, device buffers, launch
// accounting.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/tincr_gb300.h"

namespace tincr {

// Exception carrying a tincr_status; caught at the C ABI and turned into a return code.
struct Error {
    int status;
    std::string msg;
};

[[noreturn]] void fail(int status, const std::string &msg);
void check_cuda(cudaError_t e, const char *what);

#define TINCR_CUDA(call) ::tincr::check_cuda((call), #call)

// Counts kernel launches issued by this library (reported to the caller).
extern thread_local long long g_launches;
inline void count_launch(cudaStream_t, const char *) { ++g_launches; }
void check_launch(const char *name);
// Fails with TINCR_NONFINITE if any of the n host values is NaN or infinite.
void check_finite(const double *p, size_t n, const char *what);

// Owning device buffer of T.
template <class T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    explicit DevBuf(size_t count) { alloc(count); }
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
    DevBuf &operator=(DevBuf &&o) noexcept {
        if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
        return *this;
    }
    ~DevBuf() { release(); }
    void alloc(size_t count) {
        if (count == n && p) return;
        release();
        if (count) TINCR_CUDA(cudaMalloc(&p, count * sizeof(T)));
        n = count;
    }
    // grow-only allocation (keeps nothing)
    void reserve(size_t count) { if (count > n) alloc(count); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    T *get() const { return p; }
};

// page-locked host staging buffer (grow-only): uploads from it are plain DMA
struct PinnedBuf {
    double *p = nullptr;
    size_t n = 0;
    PinnedBuf() = default;
    PinnedBuf(const PinnedBuf &) = delete;
    PinnedBuf &operator=(const PinnedBuf &) = delete;
    void reserve(size_t count) {
        if (count <= n && p) return;
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
        TINCR_CUDA(cudaMallocHost(&p, (count ? count : 1) * sizeof(double)));
        n = count ? count : 1;
    }
    ~PinnedBuf() {
        if (p) cudaFreeHost(p);
    }
};

inline int ceil_div(long long a, long long b) { return int((a + b - 1) / b); }

}  // namespace tincr
