// K6: NCVis::init_embedding (src/ncvis.cpp:184-273) over the CSR graph.
//
//   Y ~ U(0,1), element t from draw t of the one-thread pcg64(seed) stream
//       (src/ncvis.cpp:195-200); each thread jumps to its own offset;
//   repeat n_init_epochs times (src/ncvis.cpp:203-261):
//       Y_new[i] = sum over row i, in CSR order, of alpha * Y_old[j]
//                  (one thread per row, FP32, multiply then add as the
//                  reference's build does: no fused multiply-add);
//       mean, population std per dimension (FP64 block partial sums, cast to
//       FP32 and divided by N in FP32 as the reference does; or, on request,
//       the reference's one-thread FP32 sums in row order, whose rounding
//       drifts ~1e-4 relative from the exact statistics at a million rows);
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

// Row i's alpha-weighted neighbour sum for d <= 4: the column indices and
// rows of eight edges are loaded together before they are added in CSR order
// (the same sums as one edge at a time, one memory round trip per eight edges
// instead of two per edge).
template <int D>
__device__ __forceinline__ void row_average(const int64_t *__restrict__ row_ptr,
                                            const int32_t *__restrict__ cols, float alpha,
                                            const float *__restrict__ Yold, int64_t i,
                                            float (&acc)[D]) {
#pragma unroll
    for (int c = 0; c < D; ++c) acc[c] = 0.f;
    const int64_t p0 = row_ptr[i], p1 = row_ptr[i + 1];
    for (int64_t p = p0; p < p1; p += 8) {
        int32_t cc[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) cc[k] = (p + k < p1) ? __ldg(cols + p + k) : -1;
        float yv[8][D];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            if (cc[k] >= 0) {
                if constexpr (D == 2) {
                    const float2 t = __ldg(reinterpret_cast<const float2 *>(Yold) + cc[k]);
                    yv[k][0] = t.x;
                    yv[k][1] = t.y;
                } else {
#pragma unroll
                    for (int c = 0; c < D; ++c) yv[k][c] = __ldg(Yold + (int64_t)cc[k] * D + c);
                }
            }
        }
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (cc[k] >= 0) {
#pragma unroll
                for (int c = 0; c < D; ++c) acc[c] = __fadd_rn(acc[c], __fmul_rn(alpha, yv[k][c]));
            }
    }
}

// spmm_rows for d <= 4 (row_average per row).
template <int D>
__global__ void __launch_bounds__(kThreads) spmm_rows_d(int64_t N, const int64_t *__restrict__ row_ptr,
                                                        const int32_t *__restrict__ cols,
                                                        float alpha, const float *__restrict__ Yold,
                                                        float *__restrict__ Ynew,
                                                        double *__restrict__ part) {
    const int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x;
    double sums[kMaxDim];
#pragma unroll
    for (int c = 0; c < D; ++c) sums[c] = 0;
    if (i < N) {
        float acc[D];
        row_average<D>(row_ptr, cols, alpha, Yold, i, acc);
#pragma unroll
        for (int c = 0; c < D; ++c) {
            Ynew[i * D + c] = acc[c];
            sums[c] = acc[c];
        }
    }
    block_partial(sums, D, part);
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

// The reference's one-thread statistics (src/ncvis.cpp:226-254 on one
// thread): per dimension an FP32 sum over the rows in order, mode 0 of the
// values (stat = sum / N), mode 1 of (y - mean)^2 (stat = sqrt(sum / N)).
// One block: all threads stage chunks of rows into shared memory with
// asynchronous copies, the next chunk in flight while lane c < d adds up
// dimension c of the current one; the adds form one dependent chain per
// dimension (N FP32 adds, ~2 ms per pass at a million rows).
constexpr int kSeqFloats = 8192;  // floats per staged chunk (32 KB; whole rows)

__device__ __forceinline__ void cp_async4(float *dst, const float *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(
                     (uint32_t)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}

__global__ void __launch_bounds__(kThreads) sequential_stat(const float *__restrict__ Y, int64_t N,
                                                            int d, int mode,
                                                            const float *__restrict__ mean,
                                                            float *__restrict__ stat) {
    extern __shared__ float chunk[];  // [2][rows_per * d]
    const int64_t rows_per = kSeqFloats / d;
    const int64_t per = rows_per * d;
    const int64_t n = N * d;
    const int64_t chunks = (n + per - 1) / per;
    auto issue = [&](int64_t k) {
        float *dst = chunk + (k & 1) * per;
        const int64_t base = k * per;
        const int64_t len = min(per, n - base);
        for (int64_t t = threadIdx.x; t < len; t += blockDim.x) cp_async4(dst + t, Y + base + t);
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    const int c = threadIdx.x;
    const float m = (mode == 1 && c < d) ? mean[c] : 0.f;
    float s = 0.f;
    issue(0);
    for (int64_t k = 0; k < chunks; ++k) {
        if (k + 1 < chunks) {
            issue(k + 1);
            asm volatile("cp.async.wait_group 1;" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;" ::: "memory");
        }
        __syncthreads();
        if (c < d) {
            const float *v = chunk + (k & 1) * per;
            const int64_t rows = min(rows_per, N - k * rows_per);
#pragma unroll 8
            for (int64_t r = 0; r < rows; ++r) {
                float t = v[r * d + c];
                if (mode == 1) {
                    t = __fsub_rn(t, m);
                    t = __fmul_rn(t, t);
                }
                s = __fadd_rn(s, t);
            }
        }
        __syncthreads();
    }
    if (c < d) {
        const float v = __fdiv_rn(s, (float)N);
        stat[c] = (mode == 0) ? v : __fsqrt_rn(v);
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

// ---- batched problems: problem p owns rows [off[p], off[p+1]), its own
// seed, and row tiles [tp[p], tp[p+1]) of kThreads rows each.

__global__ void uniform_init_batched(float *__restrict__ Y, int64_t total, int d,
                                     const int64_t *__restrict__ off, int B,
                                     const uint64_t *__restrict__ seeds) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    const int p = segment_of(off, B, t / d);
    Pcg64 g(seeds[p]);
    g.advance((uint64_t)(t - off[p] * d));
    Y[t] = unit_float(g.next());
}

__device__ __forceinline__ int64_t tile_rows(const int64_t *tp, const int64_t *off, int B, int &p,
                                             int64_t &row_end) {
    p = segment_of(tp, B, blockIdx.x);
    row_end = off[p + 1];
    return off[p] + ((int64_t)blockIdx.x - tp[p]) * kThreads + threadIdx.x;
}

__global__ void __launch_bounds__(kThreads) spmm_rows_batched(
    const int64_t *__restrict__ tp, const int64_t *__restrict__ off, int B, int d,
    const int64_t *__restrict__ row_ptr, const int32_t *__restrict__ cols, float alpha,
    const float *__restrict__ Yold, float *__restrict__ Ynew, double *__restrict__ part) {
    int p;
    int64_t row_end;
    const int64_t i = tile_rows(tp, off, B, p, row_end);
    double sums[kMaxDim];
    for (int c = 0; c < d; ++c) sums[c] = 0;
    if (i < row_end) {
        float acc[kMaxDim];
        for (int c = 0; c < d; ++c) acc[c] = 0.f;
        const int64_t p1 = row_ptr[i + 1];
        for (int64_t q = row_ptr[i]; q < p1; ++q) {
            const float *y = Yold + (int64_t)cols[q] * d;
            for (int c = 0; c < d; ++c) acc[c] = __fadd_rn(acc[c], __fmul_rn(alpha, y[c]));
        }
        for (int c = 0; c < d; ++c) {
            Ynew[i * d + c] = acc[c];
            sums[c] = acc[c];
        }
    }
    block_partial(sums, d, part);
}

template <int D>
__global__ void __launch_bounds__(kThreads) spmm_rows_batched_d(
    const int64_t *__restrict__ tp, const int64_t *__restrict__ off, int B,
    const int64_t *__restrict__ row_ptr, const int32_t *__restrict__ cols, float alpha,
    const float *__restrict__ Yold, float *__restrict__ Ynew, double *__restrict__ part) {
    int p;
    int64_t row_end;
    const int64_t i = tile_rows(tp, off, B, p, row_end);
    double sums[kMaxDim];
#pragma unroll
    for (int c = 0; c < D; ++c) sums[c] = 0;
    if (i < row_end) {
        float acc[D];
        row_average<D>(row_ptr, cols, alpha, Yold, i, acc);
#pragma unroll
        for (int c = 0; c < D; ++c) {
            Ynew[i * D + c] = acc[c];
            sums[c] = acc[c];
        }
    }
    block_partial(sums, D, part);
}

__global__ void __launch_bounds__(kThreads) centred_squares_batched(
    const int64_t *__restrict__ tp, const int64_t *__restrict__ off, int B, int d,
    const float *__restrict__ Y, const float *__restrict__ mean, double *__restrict__ part) {
    int p;
    int64_t row_end;
    const int64_t i = tile_rows(tp, off, B, p, row_end);
    double sums[kMaxDim];
    for (int c = 0; c < d; ++c) {
        sums[c] = 0;
        if (i < row_end) {
            const float dev = __fsub_rn(Y[i * d + c], mean[p * d + c]);
            sums[c] = __fmul_rn(dev, dev);
        }
    }
    block_partial(sums, d, part);
}

// One block per problem: stat[p*d + c] from the partials of p's tiles.
__global__ void finish_stat_batched(const double *__restrict__ part, const int64_t *__restrict__ tp,
                                    const int64_t *__restrict__ off, int d, int mode,
                                    float *__restrict__ stat) {
    __shared__ double red[32];
    const int p = blockIdx.x;
    const int64_t n = off[p + 1] - off[p];
    for (int c = 0; c < d; ++c) {
        double s = 0;
        for (int64_t b = tp[p] + threadIdx.x; b < tp[p + 1]; b += blockDim.x) s += part[b * d + c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
            const float v = __fdiv_rn((float)t, (float)n);
            stat[p * d + c] = (mode == 0) ? v : sqrtf(v);
        }
        __syncthreads();
    }
}

__global__ void standardize_batched(int64_t total, int d, const int64_t *__restrict__ off, int B,
                                    float *__restrict__ Y, const float *__restrict__ mean,
                                    const float *__restrict__ sigma) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t row = t / d;
        const int c = (int)(t - row * d);
        const int p = segment_of(off, B, row);
        Y[t] = __fdiv_rn(__fsub_rn(Y[t], mean[p * d + c]), sigma[p * d + c]);
    }
}

inline size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

}  // namespace

int init_tile_rows() { return kThreads; }

size_t init_batched_workspace_bytes(int64_t total_rows, int64_t n_tiles, int B, int d) {
    return align256(sizeof(float) * total_rows * d) + align256(sizeof(double) * n_tiles * d) +
           2 * align256(sizeof(float) * B * d);
}

void run_init_embedding_batched(int64_t total_rows, int d, const int64_t *off, const int64_t *tp,
                                int B, int64_t n_tiles, const uint64_t *seeds,
                                const int64_t *row_ptr, const int32_t *cols, int n_init_epochs,
                                float alpha, float *Y, void *workspace, cudaStream_t s) {
    require(d >= 1 && d <= kMaxDim, "init_embedding: d must be in [1, 32]");
    char *p = (char *)workspace;
    float *other = (float *)p;   p += align256(sizeof(float) * total_rows * d);
    double *part = (double *)p;  p += align256(sizeof(double) * n_tiles * d);
    float *mean = (float *)p;    p += align256(sizeof(float) * B * d);
    float *sigma = (float *)p;
    const int64_t n = total_rows * d;
    NCVIS_LAUNCH(uniform_init_batched, ceil_div(n, kThreads), kThreads, 0, s, Y, n, d, off, B, seeds);
    float *bufs[2] = {Y, other};
    const unsigned elem_grid = (unsigned)std::min<int64_t>((n + kThreads - 1) / kThreads,
                                                           8 * num_sms());
    for (int ep = 0; ep < n_init_epochs; ++ep) {
        const float *y_old = bufs[ep % 2];
        float *y_new = bufs[(ep + 1) % 2];
        switch (d) {
            case 1:
                NCVIS_LAUNCH(spmm_rows_batched_d<1>, (unsigned)n_tiles, kThreads, 0, s, tp, off, B,
                             row_ptr, cols, alpha, y_old, y_new, part);
                break;
            case 2:
                NCVIS_LAUNCH(spmm_rows_batched_d<2>, (unsigned)n_tiles, kThreads, 0, s, tp, off, B,
                             row_ptr, cols, alpha, y_old, y_new, part);
                break;
            case 3:
                NCVIS_LAUNCH(spmm_rows_batched_d<3>, (unsigned)n_tiles, kThreads, 0, s, tp, off, B,
                             row_ptr, cols, alpha, y_old, y_new, part);
                break;
            case 4:
                NCVIS_LAUNCH(spmm_rows_batched_d<4>, (unsigned)n_tiles, kThreads, 0, s, tp, off, B,
                             row_ptr, cols, alpha, y_old, y_new, part);
                break;
            default:
                NCVIS_LAUNCH(spmm_rows_batched, (unsigned)n_tiles, kThreads, 0, s, tp, off, B, d,
                             row_ptr, cols, alpha, y_old, y_new, part);
        }
        NCVIS_LAUNCH(finish_stat_batched, B, 256, 0, s, part, tp, off, d, 0, mean);
        NCVIS_LAUNCH(centred_squares_batched, (unsigned)n_tiles, kThreads, 0, s, tp, off, B, d,
                     y_new, mean, part);
        NCVIS_LAUNCH(finish_stat_batched, B, 256, 0, s, part, tp, off, d, 1, sigma);
        NCVIS_LAUNCH(standardize_batched, elem_grid, kThreads, 0, s, n, d, off, B, y_new, mean,
                     sigma);
    }
    if (n_init_epochs % 2)
        NCVIS_CUDA(cudaMemcpyAsync(Y, other, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
}

size_t init_workspace_bytes(int64_t N, int d) {
    const int64_t blocks = (N + kThreads - 1) / kThreads;
    return align256(sizeof(float) * N * d) + align256(sizeof(double) * blocks * d) +
           2 * align256(sizeof(float) * d);
}

void run_init_embedding(int64_t N, int d, const int64_t *row_ptr, const int32_t *cols,
                        uint64_t seed, int n_init_epochs, float alpha, float *Y, void *workspace,
                        cudaStream_t s, bool sequential_stats) {
    require(d >= 1 && d <= kMaxDim, "init_embedding: d must be in [1, 32]");
    const size_t seq_smem = sizeof(float) * 2 * (size_t)(kSeqFloats / d) * d;
    if (sequential_stats)
        NCVIS_CUDA(cudaFuncSetAttribute(sequential_stat,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)seq_smem));
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
        switch (d) {
            case 1:
                NCVIS_LAUNCH(spmm_rows_d<1>, (unsigned)blocks, kThreads, 0, s, N, row_ptr, cols,
                             alpha, y_old, y_new, part);
                break;
            case 2:
                NCVIS_LAUNCH(spmm_rows_d<2>, (unsigned)blocks, kThreads, 0, s, N, row_ptr, cols,
                             alpha, y_old, y_new, part);
                break;
            case 3:
                NCVIS_LAUNCH(spmm_rows_d<3>, (unsigned)blocks, kThreads, 0, s, N, row_ptr, cols,
                             alpha, y_old, y_new, part);
                break;
            case 4:
                NCVIS_LAUNCH(spmm_rows_d<4>, (unsigned)blocks, kThreads, 0, s, N, row_ptr, cols,
                             alpha, y_old, y_new, part);
                break;
            default:
                NCVIS_LAUNCH(spmm_rows, (unsigned)blocks, kThreads, 0, s, N, d, row_ptr, cols,
                             alpha, y_old, y_new, part);
        }
        if (sequential_stats) {
            NCVIS_LAUNCH(sequential_stat, 1, kThreads, seq_smem, s, y_new, N, d, 0, nullptr,
                         mean);
            NCVIS_LAUNCH(sequential_stat, 1, kThreads, seq_smem, s, y_new, N, d, 1, mean, sigma);
        } else {
            NCVIS_LAUNCH(finish_stat, 1, 1024, 0, s, part, (int)blocks, d, N, 0, mean);
            NCVIS_LAUNCH(centred_squares, (unsigned)blocks, kThreads, 0, s, N, d, y_new, mean,
                         part);
            NCVIS_LAUNCH(finish_stat, 1, 1024, 0, s, part, (int)blocks, d, N, 1, sigma);
        }
        NCVIS_LAUNCH(standardize, elem_grid, kThreads, 0, s, n, d, y_new, mean, sigma);
    }
    if (n_init_epochs % 2)
        NCVIS_CUDA(cudaMemcpyAsync(Y, other, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
}

}  // namespace ncvis_gpu
