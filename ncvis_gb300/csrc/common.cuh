// Shared definitions for the NCVis GB300 engine: status codes, error
// propagation, kernel-launch accounting, small device helpers.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>

namespace ncvis_gpu {

// Status codes returned through the C ABI (mirrored in include/ncvis_gb300.h).
enum Status : int {
    kOk = 0,
    kInvalidArgument = 1,
    kCudaError = 2,
    kUnsupported = 3,
    kDeviceTimeout = 4,
    kInternal = 5,
};

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &msg) : std::runtime_error(msg), code(c) {}
};

inline void check_cuda(cudaError_t e, const char *what, const char *file, int line) {
    if (e != cudaSuccess) {
        char buf[512];
        snprintf(buf, sizeof(buf), "CUDA error %s (%d) in %s at %s:%d", cudaGetErrorString(e),
                 (int)e, what, file, line);
        throw Error(kCudaError, buf);
    }
}

#define NCVIS_CUDA(call) ::ncvis_gpu::check_cuda((call), #call, __FILE__, __LINE__)

// A stream-ordered device allocation freed when it goes out of scope, on
// every exit path (errors included).
struct StreamBuffer {
    void *p = nullptr;
    cudaStream_t s;
    StreamBuffer(size_t bytes, cudaStream_t st) : s(st) {
        NCVIS_CUDA(cudaMallocAsync(&p, bytes > 0 ? bytes : 1, s));
    }
    StreamBuffer(const StreamBuffer &) = delete;
    StreamBuffer &operator=(const StreamBuffer &) = delete;
    ~StreamBuffer() {
        if (p) cudaFreeAsync(p, s);
    }
};

// Two CUDA events (start, stop), destroyed when they go out of scope.
struct EventPair {
    cudaEvent_t a = nullptr, b = nullptr;
    EventPair() {
        NCVIS_CUDA(cudaEventCreate(&a));
        const cudaError_t e = cudaEventCreate(&b);
        if (e != cudaSuccess) {
            cudaEventDestroy(a);
            a = nullptr;
            NCVIS_CUDA(e);
        }
    }
    EventPair(const EventPair &) = delete;
    EventPair &operator=(const EventPair &) = delete;
    ~EventPair() {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
    float ms() const {
        float t = 0.f;
        NCVIS_CUDA(cudaEventElapsedTime(&t, a, b));
        return t;
    }
};

// NVTX ranges over the host-side enqueue of each pipeline stage, named
// "ncvis.<stage>" (the reference's DEBUG stage timers, src/ncvis.cpp:370-437,
// name the same stages).  A profiler filters kernels by them, e.g.
// `ncu --nvtx --nvtx-include "ncvis.optimize/"`.  NVTX is header-only: without
// a tool attached every call returns at once.  next() closes the open range
// and opens the next one; the destructor closes the last (on error paths too).
struct StageRanges {
    bool open = false;
    StageRanges() = default;
    StageRanges(const StageRanges &) = delete;
    StageRanges &operator=(const StageRanges &) = delete;
    void next(const char *name) {
        if (open) nvtxRangePop();
        nvtxRangePushA(name);
        open = true;
    }
    void close() {
        if (open) nvtxRangePop();
        open = false;
    }
    ~StageRanges() { close(); }
};

inline void require(bool ok, const std::string &msg, int code = kInvalidArgument) {
    if (!ok) throw Error(code, msg);
}

// Every kernel this library launches goes through NCVIS_LAUNCH, which counts
// it; ncvis_kernel_launch_count() exposes the total so that a benchmark can
// state how many engine kernels ran in a timed region.
std::atomic<uint64_t> &launch_counter();

#define NCVIS_LAUNCH(kernel, grid, block, smem, stream, ...)                        \
    do {                                                                             \
        kernel<<<(grid), (block), (smem), (stream)>>>(__VA_ARGS__);                  \
        ::ncvis_gpu::launch_counter().fetch_add(1, std::memory_order_relaxed);       \
        NCVIS_CUDA(cudaGetLastError());                                              \
    } while (0)

// Makes `msg` the text ncvis_get_last_error() returns on this thread.
void record_error(const char *msg);

// SMs of the current device (asked each time: a process may drive several).
inline int num_sms() {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    return v > 0 ? v : 1;
}

inline unsigned ceil_div(size_t a, size_t b) { return (unsigned)((a + b - 1) / b); }

#ifdef __CUDACC__
// Index of the segment holding `t` in an ascending prefix array p[0..B]
// (p[0] <= t < p[B]).
__device__ __forceinline__ int segment_of(const int64_t *__restrict__ p, int B, int64_t t) {
    int lo = 0, hi = B - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (p[mid] <= t)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}
#endif

}  // namespace ncvis_gpu
