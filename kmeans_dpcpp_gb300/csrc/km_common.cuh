// Shared definitions for the GB300 Lloyd k-means engine (device + host side).
//
// Every kernel in this library follows the semantics of the SYCL kernels in
// src/*.hpp of kmeans_dpcpp; the per-kernel files cite the exact lines.
#pragma once

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cmath>
#include <limits>
#include <string>
#include <cuda_runtime.h>
#if __has_include(<nvtx3/nvToolsExt.h>)
#include <nvtx3/nvToolsExt.h>
#define KMC_HAVE_NVTX 1
#endif

#include "../../include/kmeans_gb300.h"

namespace kmc {

// A named NVTX range for the duration of a scope: profilers (ncu, Nsight
// Systems) show the library's phases -- fit creation (operand conversion,
// autotuning), the Lloyd loop, the final pass, serving steps.  NVTX is
// header-only and costs nothing unless a tool is attached.
struct Range {
    explicit Range(const char *name) {
#ifdef KMC_HAVE_NVTX
        nvtxRangePushA(name);
#else
        (void)name;
#endif
    }
    ~Range() {
#ifdef KMC_HAVE_NVTX
        nvtxRangePop();
#endif
    }
    Range(const Range &) = delete;
    Range &operator=(const Range &) = delete;
};

// ---------------------------------------------------------------------------
// Error reporting.  The C-ABI never throws; every entry point returns a status
// code and leaves a human-readable message in a thread-local buffer.
// ---------------------------------------------------------------------------
void set_error(const char *fmt, ...);
const char *get_error();

#define KMC_CUDA_TRY(...)                                                       \
    do {                                                                        \
        cudaError_t _e = (__VA_ARGS__);                                                \
        if (_e != cudaSuccess) {                                                \
            ::kmc::set_error("CUDA error %s (%d) at %s:%d: %s",                 \
                             cudaGetErrorName(_e), (int)_e, __FILE__, __LINE__, \
                             cudaGetErrorString(_e));                           \
            return (_e == cudaErrorMemoryAllocation) ? KMC_ERR_OUT_OF_MEMORY    \
                                                     : KMC_ERR_CUDA;            \
        }                                                                       \
    } while (0)

#define KMC_TRY(...)                      \
    do {                                  \
        int _s = (__VA_ARGS__);           \
        if (_s != KMC_OK) return _s;      \
    } while (0)

#define KMC_CHECK_ARG(cond, ...)                    \
    do {                                            \
        if (!(cond)) {                              \
            ::kmc::set_error(__VA_ARGS__);          \
            return KMC_ERR_INVALID_ARGUMENT;        \
        }                                           \
    } while (0)

inline int check_launch(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("kernel launch failed (%s): %s", what, cudaGetErrorString(e));
        return KMC_ERR_CUDA;
    }
    return KMC_OK;
}

// quotient_ceil of src/quotients_utils.hpp:5-6
template <typename T>
__host__ __device__ constexpr T ceil_div(T a, T b) { return (a + b - 1) / b; }

template <typename T>
__host__ __device__ inline T pos_inf() { return std::numeric_limits<T>::infinity(); }

// Number of SMs of the current device (cached per device).
int num_sms();
// L2 size in bytes of the current device.
int64_t l2_bytes();
// Returns the unused memory of the library's pools to the system.
int trim_pools();

// The library's own stream-ordered memory pool on the current device.  It
// keeps freed memory mapped (release threshold = unlimited), so a fit that
// follows another reuses the pages instead of mapping gigabytes again;
// kmc_trim_cached_memory() hands the unused part back.
cudaMemPool_t scratch_pool();

// Allocations left before an injected out-of-memory failure (< 0: none);
// set by kmc_debug_fail_allocation.
extern std::atomic<long long> g_fail_alloc_after;

// True when the injected failure fires for this allocation (once).
inline bool injected_alloc_failure() {
    long long v = g_fail_alloc_after.load();
    while (v >= 0) {
        if (g_fail_alloc_after.compare_exchange_weak(v, v - 1)) return v == 0;
    }
    return false;
}

// Stream-ordered scratch allocation (the library's pool, on the caller's stream).
struct Scratch {
    void *ptr = nullptr;
    cudaStream_t stream = nullptr;
    Scratch() = default;
    Scratch(const Scratch &) = delete;
    Scratch &operator=(const Scratch &) = delete;
    int alloc(size_t bytes, cudaStream_t s) {
        if (ptr) cudaFreeAsync(ptr, stream);  // re-allocation replaces the old block
        ptr = nullptr;
        stream = s;
        if (bytes == 0) bytes = 16;
        if (injected_alloc_failure()) {
            set_error("stream-ordered allocation of %zu bytes failed: injected out-of-memory "
                      "failure (kmc_debug_fail_allocation)", bytes);
            return KMC_ERR_OUT_OF_MEMORY;
        }
        cudaMemPool_t pool = scratch_pool();
        cudaError_t e = pool != nullptr ? cudaMallocFromPoolAsync(&ptr, bytes, pool, s)
                                        : cudaMallocAsync(&ptr, bytes, s);
        if (e != cudaSuccess) {
            ptr = nullptr;
            set_error("stream-ordered allocation of %zu bytes failed: %s", bytes,
                      cudaGetErrorString(e));
            return KMC_ERR_OUT_OF_MEMORY;
        }
        return KMC_OK;
    }
    // Stream-ordered free now (the object can be re-used).
    void release() {
        if (ptr) cudaFreeAsync(ptr, stream);
        ptr = nullptr;
    }
    ~Scratch() { release(); }
    template <typename U> U *as() const { return static_cast<U *>(ptr); }
};

// Round a byte count up to a multiple of 256 (suballocation alignment).
inline size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

}  // namespace kmc
