// ncvis_measure_update_rate: the rate at which this GPU serves the SGD
// kernel's memory pattern, measured live — the ceiling its pair-update rate
// is compared against.
//
// Every SGD sample reads one random row of Y (ld.cg) and applies one random
// row update (red.global.add), rows of d floats in an array of `rows` rows
// that stays resident in L2.  Such traffic is bounded by the L2's rate for
// random small requests, far below what the byte counts would allow at HBM
// or L2 bandwidth, so the HBM roofline says little about the kernel.  This
// measures, on the SGD kernel's own launch shape (two resident 256-thread
// blocks per SM, four rows in flight per thread), the rate of
//   * random row gathers alone, and
//   * random row gathers each followed by a reduction into the same row.
// Row indices come from an integer hash; every access stays in bounds.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "../../include/ncvis_gb300.h"
#include "common.cuh"

namespace ncvis_gpu {

namespace {

constexpr int kThreads = 256;
constexpr int kInFlight = 4;

__device__ __forceinline__ uint32_t mix32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352dU;
    x ^= x >> 15;
    x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}

template <int D, bool kUpdate>
__global__ void __launch_bounds__(kThreads) random_rows(float *__restrict__ Y, uint32_t rows,
                                                        int iters, float *__restrict__ sink) {
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t st = mix32(tid * 9781u + 17u);
    float acc = 0.f;
    for (int it = 0; it < iters; ++it) {
        uint32_t r[kInFlight];
        float v[kInFlight];
#pragma unroll
        for (int g = 0; g < kInFlight; ++g) {
            st = mix32(st + (uint32_t)g);
            r[g] = (uint32_t)(((uint64_t)st * rows) >> 32);  // < rows
        }
#pragma unroll
        for (int g = 0; g < kInFlight; ++g) {
            if constexpr (D == 2) {
                v[g] = __ldcg(reinterpret_cast<const float2 *>(Y + (size_t)r[g] * 2)).x;
            } else if constexpr (D == 4) {
                v[g] = __ldcg(reinterpret_cast<const float4 *>(Y + (size_t)r[g] * 4)).x;
            } else {
                v[g] = __ldcg(Y + r[g]);
            }
        }
#pragma unroll
        for (int g = 0; g < kInFlight; ++g) {
            acc += v[g];
            if constexpr (kUpdate) {
                float *p = Y + (size_t)r[g] * D;
                if constexpr (D == 2) {
                    asm volatile("red.global.add.v2.f32 [%0], {%1, %2};" ::"l"(p), "f"(0.f), "f"(0.f)
                                 : "memory");
                } else if constexpr (D == 4) {
                    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(0.f),
                                 "f"(0.f), "f"(0.f), "f"(0.f)
                                 : "memory");
                } else {
                    asm volatile("red.global.add.f32 [%0], %1;" ::"l"(p), "f"(0.f) : "memory");
                }
            }
        }
    }
    if (acc == 1.2345e-30f) sink[tid] = acc;  // keeps the loads; never true for the zero array
}

template <int D, bool kUpdate>
double time_rate(float *Y, uint32_t rows, float *sink, cudaStream_t s) {
    const int blocks = 2 * num_sms();
    const int64_t threads = (int64_t)blocks * kThreads;
    const int iters = (int)std::max<int64_t>(1, (int64_t(1) << 26) / (threads * kInFlight));
    EventPair t;
    NCVIS_LAUNCH((random_rows<D, kUpdate>), blocks, kThreads, 0, s, Y, rows, 2, sink);
    NCVIS_CUDA(cudaEventRecord(t.a, s));
    NCVIS_LAUNCH((random_rows<D, kUpdate>), blocks, kThreads, 0, s, Y, rows, iters, sink);
    NCVIS_CUDA(cudaEventRecord(t.b, s));
    NCVIS_CUDA(cudaEventSynchronize(t.b));
    const float ms = t.ms();
    return (double)threads * kInFlight * iters / (ms * 1e-3);
}

template <int D>
void measure(uint32_t rows, double *gathers, double *updates, cudaStream_t s) {
    float *Y = nullptr, *sink = nullptr;
    const size_t threads = (size_t)2 * num_sms() * kThreads;
    NCVIS_CUDA(cudaMalloc(&Y, (size_t)rows * D * sizeof(float)));
    cudaError_t e = cudaMalloc(&sink, threads * sizeof(float));
    if (e != cudaSuccess) {
        cudaFree(Y);
        NCVIS_CUDA(e);
    }
    try {
        NCVIS_CUDA(cudaMemsetAsync(Y, 0, (size_t)rows * D * sizeof(float), s));
        *gathers = time_rate<D, false>(Y, rows, sink, s);
        *updates = time_rate<D, true>(Y, rows, sink, s);
    } catch (...) {
        cudaFree(Y);
        cudaFree(sink);
        throw;
    }
    NCVIS_CUDA(cudaFree(Y));
    NCVIS_CUDA(cudaFree(sink));
}

}  // namespace

}  // namespace ncvis_gpu

extern "C" int ncvis_measure_update_rate(size_t rows, size_t d, double *gathers_per_s,
                                         double *updates_per_s, void *stream) {
    using namespace ncvis_gpu;
    try {
        require(rows >= 1 && rows < (size_t(1) << 31), "update rate: rows must be in [1, 2^31)");
        require(d == 1 || d == 2 || d == 4, "update rate: d must be 1, 2 or 4", kUnsupported);
        require(gathers_per_s != nullptr && updates_per_s != nullptr,
                "update rate: null output pointer");
        cudaStream_t s = (cudaStream_t)stream;
        if (d == 1) measure<1>((uint32_t)rows, gathers_per_s, updates_per_s, s);
        if (d == 2) measure<2>((uint32_t)rows, gathers_per_s, updates_per_s, s);
        if (d == 4) measure<4>((uint32_t)rows, gathers_per_s, updates_per_s, s);
        return NCVIS_OK;
    } catch (const Error &e) {
        record_error(e.what());
        return e.code;
    } catch (const std::exception &e) {
        record_error(e.what());
        return NCVIS_INTERNAL;
    }
}
