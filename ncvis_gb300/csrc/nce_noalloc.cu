// ncvis_nce_loss_device_noalloc: the NCE loss of ncvis_nce_loss_device
// computed without allocating device memory.
//
// Some callers cannot allocate device memory at the moment they need the
// loss: a serving process whose memory pool already owns every free byte of
// HBM (a new cudaMalloc would fail), a latency-critical loop that cannot
// afford the device-wide synchronisation cudaMalloc/cudaFree may imply, or a
// host framework whose policy forbids allocations outside its own pool.  For
// them, the per-block FP64 partial sums and the argument-check flag that
// ncvis_nce_loss_device keeps in freshly allocated memory live here in one
// file-scope device array of fixed size (kScratchBytes = 65,568 bytes),
// present on every GPU that loads the library until the process exits.  A
// call therefore accepts at most kNoAllocMaxEdges = 2^20 edges.
//
// Host code cannot pass the array's name to a kernel (on the host it names a
// host-side stand-in, not device memory).  Set-up, once per device (and again
// if that device's context was destroyed and created anew): with the device
// current, cudaGetSymbolAddress gives the array's device address, which is
// kept with the context's unique id; later calls in the same context reuse
// it.  The first call on a device does this set-up, which also loads the
// library's device code there; make it at start-up, while memory is free,
// and before any stream capture.  Every call waits for its stream (it reads
// the argument-check flag back to the host).  All calls share the array and
// each leaves its contents behind: the check flag is cleared at the start of
// every call (the partials are overwritten), and calls whose GPU work
// overlaps in time race on the array.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "../../include/ncvis_gb300.h"
#include "common.cuh"
#include "stages.cuh"

namespace ncvis_gpu {

namespace {

constexpr int64_t kNoAllocMaxEdges = int64_t(1) << 20;
// Two doubles of partials per block of the loss kernel (kNceThreads threads),
// plus two, as nce_workspace_bytes; then a 16-byte slot holding the check flag.
constexpr size_t kPartialDoubles = 2 * (kNoAllocMaxEdges / kNceThreads + 1);
constexpr size_t kScratchDoubles = kPartialDoubles + 2;
constexpr size_t kScratchBytes = sizeof(double) * kScratchDoubles;
static_assert(kNoAllocMaxEdges % kNceThreads == 0, "the edge limit fills whole loss blocks");
static_assert(kScratchBytes == 65568, "the documented size of the scratch array");

__device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

using CtxGetCurrentFn = CUresult (*)(CUcontext *);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long *);

template <class Fn>
Fn driver_entry(const char *name) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    NCVIS_CUDA(cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q));
    require(q == cudaDriverEntryPointSuccess && p != nullptr,
            std::string("nce_loss_noalloc: driver entry point ") + name + " is unavailable",
            kCudaError);
    return (Fn)p;
}

// Unique id of the current context (0 when the thread has none yet).
unsigned long long current_context_id() {
    static const CtxGetCurrentFn get_current = driver_entry<CtxGetCurrentFn>("cuCtxGetCurrent");
    static const CtxGetIdFn get_id = driver_entry<CtxGetIdFn>("cuCtxGetId");
    CUcontext ctx = nullptr;
    require(get_current(&ctx) == CUDA_SUCCESS, "nce_loss_noalloc: cuCtxGetCurrent failed",
            kCudaError);
    if (!ctx) return 0;
    unsigned long long id = 0;
    require(get_id(ctx, &id) == CUDA_SUCCESS, "nce_loss_noalloc: cuCtxGetId failed", kCudaError);
    return id;
}

constexpr int kMaxDevices = 128;
std::mutex g_mu;
struct Setup {
    unsigned long long ctx_id = 0;
    double *addr = nullptr;
};
Setup g_setup[kMaxDevices];

// Device address of g_noalloc_scratch on the current device, looked up at
// set-up (the device's first call, or its first call in a new context).
double *scratch_on_current_device() {
    int dev = 0;
    NCVIS_CUDA(cudaGetDevice(&dev));
    require(dev >= 0 && dev < kMaxDevices, "nce_loss_noalloc: device index out of range");
    std::lock_guard<std::mutex> lock(g_mu);
    const unsigned long long id = current_context_id();
    Setup &e = g_setup[dev];
    if (id == 0 || e.ctx_id != id || !e.addr) {
        void *p = nullptr;
        NCVIS_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        require(p != nullptr, "nce_loss_noalloc: no device address for the scratch array",
                kCudaError);
        e.addr = (double *)p;
        e.ctx_id = current_context_id();  // the lookup made the context current if it was not
    }
    return e.addr;
}

// flag = 1 if any src/dst entry lies outside [0, N).
__global__ void check_edges(const int32_t *__restrict__ src, const int32_t *__restrict__ dst,
                            int64_t E, int64_t N, int *__restrict__ flag) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t a = src[e], b = dst[e];
        if (a < 0 || a >= N || b < 0 || b >= N) atomicOr(flag, 1);
    }
}

}  // namespace

}  // namespace ncvis_gpu

using namespace ncvis_gpu;

extern "C" int ncvis_nce_loss_device_noalloc(size_t N, size_t d, size_t E, const int32_t *d_src,
                                             const int32_t *d_dst, const float *dY,
                                             const float *dQ, size_t n_noise, float a, float b,
                                             uint64_t seed, uint32_t tag, uint64_t edge_offset,
                                             double *d_loss, void *stream) {
    try {
        require(d_src && d_dst && dY && dQ && d_loss, "nce_loss_noalloc: null pointer");
        require(N >= 2 && N < (size_t(1) << 31) && d >= 1 && d <= 32 && n_noise >= 1 &&
                    n_noise <= 1024,
                "nce_loss_noalloc: need 2 <= N < 2^31, 1 <= d <= 32, 1 <= n_noise <= 1024");
        require((int64_t)E <= kNoAllocMaxEdges,
                "nce_loss_noalloc: at most 2^20 edges per call (E = " + std::to_string(E) + ")");
        // The loss kernels' partials must stay below the flag slot.
        require(nce_workspace_bytes((int64_t)E) <= sizeof(double) * kPartialDoubles,
                "nce_loss_noalloc: the loss workspace exceeds the scratch array", kInternal);
        cudaStream_t s = (cudaStream_t)stream;
        double *scratch = scratch_on_current_device();
        int *flag = (int *)(scratch + kPartialDoubles);
        NCVIS_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), s));
        if (E > 0) {
            const unsigned grid = (unsigned)std::min<int64_t>(((int64_t)E + 255) / 256,
                                                              16 * num_sms());
            NCVIS_LAUNCH(check_edges, grid, 256, 0, s, d_src, d_dst, (int64_t)E, (int64_t)N, flag);
        }
        int bad = 0;
        NCVIS_CUDA(cudaMemcpyAsync(&bad, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
        NCVIS_CUDA(cudaStreamSynchronize(s));
        require(bad == 0, "nce_loss_noalloc: an edge endpoint is outside [0, N)");
        run_nce(0, (int64_t)N, (int)d, (int64_t)E, d_src, d_dst, dY, dQ, (int)n_noise, a, b, seed,
                tag, edge_offset, nullptr, nullptr, d_loss, scratch, s);
        return NCVIS_OK;
    } catch (const Error &e) {
        record_error(e.what());
        return e.code;
    } catch (const std::exception &e) {
        record_error(e.what());
        return NCVIS_INTERNAL;
    }
}
