// Device-wide exclusive prefix sum (int32 counts -> int64 offsets), used for
// CSR offsets.  Three passes: per-tile totals, a single-block scan of the
// tile totals, and a per-tile rescan that adds the tile's offset.
#include <algorithm>

#include "common.cuh"
#include "stages.cuh"

namespace ncvis_gpu {

namespace {

constexpr int kThreads = 512;
constexpr int kPerThread = 8;
constexpr int kTile = kThreads * kPerThread;

__device__ __forceinline__ int64_t block_exclusive_scan(int64_t v, int64_t *warp_tot,
                                                        int64_t *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int64_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int64_t w = (lane < (int)(blockDim.x >> 5)) ? warp_tot[lane] : 0;
        int64_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int64_t t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += t;
        }
        if (lane < (int)(blockDim.x >> 5)) warp_tot[lane] = wi - w;
        if (lane == 31) *total = wi;
    }
    __syncthreads();
    int64_t res = warp_tot[warp] + incl - v;
    __syncthreads();
    return res;
}

__global__ void __launch_bounds__(kThreads) tile_totals(const int32_t *__restrict__ in, int64_t n,
                                                        int64_t *__restrict__ totals) {
    __shared__ int64_t warp_tot[32];
    __shared__ int64_t total;
    const int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kPerThread;
    int64_t s = 0;
#pragma unroll
    for (int j = 0; j < kPerThread; ++j)
        if (base + j < n) s += in[base + j];
    block_exclusive_scan(s, warp_tot, &total);
    if (threadIdx.x == 0) totals[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kThreads) scan_totals(int64_t *__restrict__ totals, int64_t tiles,
                                                        int64_t *__restrict__ grand) {
    __shared__ int64_t warp_tot[32];
    __shared__ int64_t total;
    int64_t carry = 0;
    for (int64_t b = 0; b < tiles; b += kThreads) {
        const int64_t i = b + threadIdx.x;
        int64_t v = (i < tiles) ? totals[i] : 0;
        int64_t ex = block_exclusive_scan(v, warp_tot, &total);
        if (i < tiles) totals[i] = carry + ex;
        carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) *grand = carry;
}

__global__ void __launch_bounds__(kThreads) tile_rescan(const int32_t *__restrict__ in, int64_t n,
                                                        const int64_t *__restrict__ offsets,
                                                        const int64_t *__restrict__ grand,
                                                        int64_t *__restrict__ out) {
    __shared__ int64_t warp_tot[32];
    __shared__ int64_t total;
    const int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kPerThread;
    int32_t v[kPerThread];
    int64_t s = 0;
#pragma unroll
    for (int j = 0; j < kPerThread; ++j) {
        v[j] = (base + j < n) ? in[base + j] : 0;
        s += v[j];
    }
    int64_t run = offsets[blockIdx.x] + block_exclusive_scan(s, warp_tot, &total);
#pragma unroll
    for (int j = 0; j < kPerThread; ++j) {
        if (base + j < n) out[base + j] = run;
        run += v[j];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = *grand;
}

}  // namespace

size_t scan_workspace_bytes(int64_t n) { return sizeof(int64_t) * ((n + kTile - 1) / kTile + 2); }

void launch_exclusive_scan_i32_to_i64(const int32_t *in, int64_t *out, int64_t n, void *ws,
                                      cudaStream_t s) {
    const int64_t tiles = (n + kTile - 1) / kTile;
    int64_t *totals = (int64_t *)ws;
    int64_t *grand = totals + tiles + 1;
    if (tiles > 0) NCVIS_LAUNCH(tile_totals, (unsigned)tiles, kThreads, 0, s, in, n, totals);
    NCVIS_LAUNCH(scan_totals, 1, kThreads, 0, s, totals, tiles, grand);
    NCVIS_LAUNCH(tile_rescan, (unsigned)std::max<int64_t>(tiles, 1), kThreads, 0, s, in, n, totals,
                 grand, out);
}

}  // namespace ncvis_gpu
