// K6: NCVis::init_embedding (src/ncvis.cpp:184-273) over the CSR graph.
//
//   Y ~ U(0,1), element t from draw t of the one-thread pcg64(seed) stream
//       (src/ncvis.cpp:195-200); each thread jumps to its own offset;
//   repeat n_init_epochs times (src/ncvis.cpp:203-261):
//       Y_new[i] = sum over row i, in CSR order, of alpha * Y_old[j]
//                  (one thread per row, FP32, multiply then add as the
//                  reference's build does: no fused multiply-add);
//       mean, population std per dimension (FP64 block partial sums, cast to
//       FP32 and divided by N in FP32 as the reference does);
//       Y_new = (Y_new - mean) / sigma;
//   ping-pong buffers, result left in Y (src/ncvis.cpp:262-267).
#include <algorithm>

#include "common.cuh"
#include "rng.cuh"
#include "stages.cuh"

namespace ncvis_gpu {

namespace {

constexpr int kThreads = 256;
constexpr int kMaxDim = 32;  // dimensions held in registers by the row kernels

__global__ void uniform_init(float *__restrict__ Y, int64_t n, uint64_t seed, int per_thread) {
    const int64_t t0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * per_thread;
    if (t0 >= n) return;
    Pcg64 g(seed);
    g.advance((uint64_t)t0);
    const int64_t t1 = min(n, t0 + per_thread);
    for (int64_t t = t0; t < t1; ++t) Y[t] = unit_float(g.next());
}

// Block partial sums (FP64) of per-dimension values, written to part[blk][d].
__device__ __forceinline__ void block_partial(double *vals, int d, double *part) {
    __shared__ double red[kThreads / 32][kMaxDim];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int c = 0; c < d; ++c) {
        double v = vals[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][c] = v;
    }
    __syncthreads();
    if (threadIdx.x < d) {
        double s = 0;
        for (int w = 0; w < kThreads / 32; ++w) s += red[w][threadIdx.x];
        part[(size_t)blockIdx.x * d + threadIdx.x] = s;
    }
}

__global__ void __launch_bounds__(kThreads) spmm_rows(int64_t N, int d,
                                                      const int64_t *__restrict__ row_ptr,
                                                      const int32_t *__restrict__ cols,
                                                      float alpha, const float *__restrict__ Yold,
                                                      float *__restrict__ Ynew,
                                                      double *__restrict__ part) {
    const int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x;
    double sums[kMaxDim];
    for (int c = 0; c < d; ++c) sums[c] = 0;
    if (i < N) {
        float acc[kMaxDim];
        for (int c = 0; c < d; ++c) acc[c] = 0.f;
        const int64_t p1 = row_ptr[i + 1];
        for (int64_t p = row_ptr[i]; p < p1; ++p) {
            const float *y = Yold + (int64_t)cols[p] * d;
            for (int c = 0; c < d; ++c) acc[c] = __fadd_rn(acc[c], __fmul_rn(alpha, y[c]));
        }
        for (int c = 0; c < d; ++c) {
            Ynew[i * d + c] = acc[c];
            sums[c] = acc[c];
        }
    }
    block_partial(sums, d, part);
}

__global__ void __launch_bounds__(kThreads) centred_squares(int64_t N, int d,
                                                            const float *__restrict__ Y,
                                                            const float *__restrict__ mean,
                                                            double *__restrict__ part) {
    const int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x;
    double sums[kMaxDim];
    for (int c = 0; c < d; ++c) {
        sums[c] = 0;
        if (i < N) {
            float dev = __fsub_rn(Y[i * d + c], mean[c]);
            sums[c] = __fmul_rn(dev, dev);
        }
    }
    block_partial(sums, d, part);
}

// stat[c] = reduce(part[:, c]); mode 0: mean = sum / N; mode 1: sigma = sqrt(sum / N).
__global__ void finish_stat(const double *__restrict__ part, int blocks, int d, int64_t N, int mode,
                            float *__restrict__ stat) {
    __shared__ double red[32];
    for (int c = 0; c < d; ++c) {
        double s = 0;
        for (int b = threadIdx.x; b < blocks; b += blockDim.x) s += part[(size_t)b * d + c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
            const float v = __fdiv_rn((float)t, (float)N);
            stat[c] = (mode == 0) ? v : sqrtf(v);
        }
        __syncthreads();
    }
}

__global__ void standardize(int64_t n, int d, float *__restrict__ Y, const float *__restrict__ mean,
                            const float *__restrict__ sigma) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(t % d);
        Y[t] = __fdiv_rn(__fsub_rn(Y[t], mean[c]), sigma[c]);
    }
}

inline size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

}  // namespace

size_t init_workspace_bytes(int64_t N, int d) {
    const int64_t blocks = (N + kThreads - 1) / kThreads;
    return align256(sizeof(float) * N * d) + align256(sizeof(double) * blocks * d) +
           2 * align256(sizeof(float) * d);
}

void run_init_embedding(int64_t N, int d, const int64_t *row_ptr, const int32_t *cols,
                        uint64_t seed, int n_init_epochs, float alpha, float *Y, void *workspace,
                        cudaStream_t s) {
    require(d >= 1 && d <= kMaxDim, "init_embedding: d must be in [1, 32]");
    const int64_t blocks = (N + kThreads - 1) / kThreads;
    char *p = (char *)workspace;
    float *other = (float *)p;   p += align256(sizeof(float) * N * d);
    double *part = (double *)p;  p += align256(sizeof(double) * blocks * d);
    float *mean = (float *)p;    p += align256(sizeof(float) * d);
    float *sigma = (float *)p;

    const int64_t n = N * d;
    const int per_thread = 64;
    NCVIS_LAUNCH(uniform_init, ceil_div(ceil_div(n, per_thread), kThreads), kThreads, 0, s, Y, n,
                 seed, per_thread);
    float *bufs[2] = {Y, other};
    const unsigned elem_grid = (unsigned)std::min<int64_t>((n + kThreads - 1) / kThreads,
                                                           8 * num_sms());
    for (int ep = 0; ep < n_init_epochs; ++ep) {
        const float *y_old = bufs[ep % 2];
        float *y_new = bufs[(ep + 1) % 2];
        NCVIS_LAUNCH(spmm_rows, (unsigned)blocks, kThreads, 0, s, N, d, row_ptr, cols, alpha, y_old,
                     y_new, part);
        NCVIS_LAUNCH(finish_stat, 1, 1024, 0, s, part, (int)blocks, d, N, 0, mean);
        NCVIS_LAUNCH(centred_squares, (unsigned)blocks, kThreads, 0, s, N, d, y_new, mean, part);
        NCVIS_LAUNCH(finish_stat, 1, 1024, 0, s, part, (int)blocks, d, N, 1, sigma);
        NCVIS_LAUNCH(standardize, elem_grid, kThreads, 0, s, n, d, y_new, mean, sigma);
    }
    if (n_init_epochs % 2)
        NCVIS_CUDA(cudaMemcpyAsync(Y, other, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
}

}  // namespace ncvis_gpu
