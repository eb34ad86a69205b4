// Trustworthiness (Venna & Kaski 2001, the definition scikit-learn's
// manifold.trustworthiness implements) of an embedding Y of X at full size on
// the GPU:
//
//   T(k) = 1 - 2 / (N k (2N - 3k - 1)) * sum_i sum_{j in kNN_Y(i)} max(0, r(i, j) - k),
//
// r(i, j) the 1-based rank of j among the other points by their distance to
// i in X.  kNN_Y comes from the engine's exact FP32 kNN of Y (squared L2).
// For every i and each of its k embedding neighbours j the rank is counted
// directly: r(i, j) = #{m : d_X(i, m) < d_X(i, j)}, where m = i itself is
// counted (d_X(i, i) ~ 0) and stands for the 1 of the 1-based rank.  The
// counts take one pass over all N^2 pairs: a tiled FP32 distance GEMM (64
// queries x 128 candidates per tile, 4 x 8 per thread) whose epilogue
// compares each distance with its query's k thresholds.  Thresholds and
// tiles form distances with the same function and the same sequential FMA
// order over the coordinates, so d_X(i, j) meets its own threshold exactly
// and is not counted.  Distances are the engine's (squared L2, or
// 1 - <x, y> after the inner-product spaces' preprocessing), whose order is
// the order of the Euclidean distances for the cosine and correlation spaces.
#include <cuda_runtime.h>

#include <cfloat>
#include <string>

#include "../../include/ncvis_gb300.h"
#include "common.cuh"
#include "stages.cuh"

namespace ncvis_gpu {

namespace {

constexpr int BM = 64;   // queries per block
constexpr int BN = 128;  // candidates per tile
constexpr int BK = 16;   // reduction slice
constexpr int NT = 256;  // threads per block
constexpr int KQ = 16;   // threshold slots per query (k <= 16)

// Offsets of the scratch buffers in one allocation, 256-byte aligned.
struct Scratch {
    size_t total = 0;
    size_t take(size_t bytes) {
        const size_t off = total;
        total += (bytes + 255) / 256 * 256;
        return off;
    }
};

// Distance from its GEMM terms, with every rounding spelled out.
__device__ __forceinline__ float gemm_distance(float qn, float cn, float dot, bool l2) {
    return l2 ? __fsub_rn(__fadd_rn(qn, cn), __fmul_rn(2.f, dot)) : __fsub_rn(1.f, dot);
}

// thr[i][q] = d_X(i, nbr[i][q]) for q < k; empty slots -FLT_MAX (count nothing).
__global__ void thresholds(const float *__restrict__ Xp, const float *__restrict__ sqn, int64_t N,
                           int D, bool l2, const int32_t *__restrict__ nbr, int k,
                           float *__restrict__ thr) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N * KQ) return;
    const int64_t i = t / KQ;
    const int q = (int)(t % KQ);
    float out = -FLT_MAX;
    if (q < k) {
        const int32_t j = nbr[i * k + q];
        if (j >= 0 && j < N) {
            float dot = 0.f;
            for (int c = 0; c < D; ++c) dot = fmaf(Xp[i * D + c], Xp[(int64_t)j * D + c], dot);
            out = gemm_distance(sqn[i], sqn[j], dot, l2);
        }
    }
    thr[t] = out;
}

// counts[i][q] += #{m in this block's candidate range : d_X(i, m) < thr[i][q]}.
__global__ void __launch_bounds__(NT) count_closer(const float *__restrict__ Xp,
                                                   const float *__restrict__ sqn, int64_t N, int D,
                                                   bool l2, const float *__restrict__ thr,
                                                   int splits, int32_t *__restrict__ counts) {
    __shared__ __align__(16) float As[BK * BM];
    __shared__ float Bs[BK * BN];
    __shared__ float ths[KQ * BM];
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    const int64_t q0 = (int64_t)blockIdx.x * BM;
    const int64_t c_begin = N * blockIdx.y / splits;
    const int64_t c_end = N * (blockIdx.y + 1) / splits;
    for (int t = tid; t < KQ * BM; t += NT) {
        const int q = t / KQ, slot = t % KQ;
        ths[slot * BM + q] = (q0 + q < N) ? thr[(q0 + q) * KQ + slot] : -FLT_MAX;
    }
    float qn[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int64_t q = q0 + ty * 4 + i;
        qn[i] = (q < N) ? sqn[q] : 0.f;
    }
    int cnt[4][KQ];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int s = 0; s < KQ; ++s) cnt[i][s] = 0;
    __syncthreads();

    for (int64_t c0 = c_begin; c0 < c_end; c0 += BN) {
        float acc[4][8];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
        for (int k0 = 0; k0 < D; k0 += BK) {
            {  // queries: 64 rows x 16 columns, 4 per thread
                const int q = tid >> 2, kk = (tid & 3) * 4;
                const int64_t gq = q0 + q;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int kc = k0 + kk + j;
                    As[(kk + j) * BM + q] = (gq < N && kc < D) ? Xp[gq * D + kc] : 0.f;
                }
            }
            {  // candidates: 128 rows x 16 columns, 8 per thread
                const int c = tid >> 1, kk = (tid & 1) * 8;
                const int64_t gc = c0 + c;
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const int kc = k0 + kk + j;
                    Bs[(kk + j) * BN + c] = (gc < c_end && kc < D) ? Xp[gc * D + kc] : 0.f;
                }
            }
            __syncthreads();
#pragma unroll
            for (int kk = 0; kk < BK; ++kk) {
                const float4 a = *reinterpret_cast<const float4 *>(&As[kk * BM + ty * 4]);
                float b[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) b[j] = Bs[kk * BN + tx + 16 * j];
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    acc[0][j] = fmaf(a.x, b[j], acc[0][j]);
                    acc[1][j] = fmaf(a.y, b[j], acc[1][j]);
                    acc[2][j] = fmaf(a.z, b[j], acc[2][j]);
                    acc[3][j] = fmaf(a.w, b[j], acc[3][j]);
                }
            }
            __syncthreads();
        }
        // Distances of this tile (candidates past the range count nothing).
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int64_t gc = c0 + tx + 16 * j;
            const float cn = (gc < c_end) ? sqn[gc] : 0.f;
#pragma unroll
            for (int i = 0; i < 4; ++i)
                acc[i][j] = (gc < c_end) ? gemm_distance(qn[i], cn, acc[i][j], l2) : FLT_MAX;
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
#pragma unroll
            for (int s = 0; s < KQ; ++s) {
                const float th = ths[s * BM + ty * 4 + i];
                int n = 0;
#pragma unroll
                for (int j = 0; j < 8; ++j) n += acc[i][j] < th ? 1 : 0;
                cnt[i][s] += n;
            }
        }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int64_t q = q0 + ty * 4 + i;
        if (q >= N) continue;
#pragma unroll
        for (int s = 0; s < KQ; ++s)
            if (cnt[i][s]) atomicAdd(&counts[q * KQ + s], cnt[i][s]);
    }
}

// sum over queries and their k slots of max(0, count - k), in FP64.
__global__ void penalty_sum(const int32_t *__restrict__ counts, int64_t N, int k,
                            double *__restrict__ out) {
    __shared__ double red[NT / 32];
    double v = 0.0;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < N * KQ;
         t += (int64_t)gridDim.x * blockDim.x) {
        if ((int)(t % KQ) < k) v += (double)max(0, counts[t] - k);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < NT / 32; ++w) s += red[w];
        atomicAdd(out, s);
    }
}

}  // namespace

}  // namespace ncvis_gpu

extern "C" int ncvis_trustworthiness_device(const float *dX, size_t N, size_t D, int distance,
                                            const float *dY, size_t d, size_t k, double *out,
                                            void *stream) {
    using namespace ncvis_gpu;
    char *base = nullptr;
    cudaStream_t s = (cudaStream_t)stream;
    try {
        require(dX && dY && out, "trustworthiness: null pointer");
        require(k >= 1 && k <= (size_t)KQ, "trustworthiness: k must be in [1, 16]");
        require(N >= 2 * k + 2 && N < (size_t(1) << 31) && N * KQ < (size_t(1) << 31),
                "trustworthiness: need 2k + 2 <= N < 2^27");
        require(D >= 1 && d >= 1, "trustworthiness: D and d must be positive");
        require(distance >= 0 && distance <= 3,
                "[ncvis::NCVis::buildKNN] Unrecognized distance type.");
        Scratch L;
        const size_t o_Xp = L.take(sizeof(float) * N * D);
        const size_t o_sqn = L.take(sizeof(float) * N);
        const size_t o_flag = L.take(sizeof(int) * 2);
        const size_t o_nbr = L.take(sizeof(int32_t) * N * k);
        const size_t o_nd = L.take(sizeof(float) * N * k);
        const size_t o_thr = L.take(sizeof(float) * N * KQ);
        const size_t o_cnt = L.take(sizeof(int32_t) * N * KQ);
        const size_t o_sum = L.take(sizeof(double));
        NCVIS_CUDA(cudaMallocAsync((void **)&base, L.total, s));
        int32_t *nbr = (int32_t *)(base + o_nbr);
        // kNN of the embedding (exact FP32, squared L2), rows without the point itself.
        int rc = ncvis_knn_device(dY, N, d, NCVIS_SQUARED_L2, k, NCVIS_KNN_FP32, 0, nbr,
                                  (float *)(base + o_nd), stream);
        if (rc != NCVIS_OK) throw Error(rc, ncvis_get_last_error());
        NCVIS_CUDA(cudaMemsetAsync(base + o_flag, 0, sizeof(int) * 2, s));
        launch_preprocess(dX, (int64_t)N, (int)D, distance, (float *)(base + o_Xp),
                          (float *)(base + o_sqn), nullptr, 0, (int *)(base + o_flag), s);
        int bad = 0;
        NCVIS_CUDA(cudaMemcpyAsync(&bad, base + o_flag, sizeof(int), cudaMemcpyDeviceToHost, s));
        NCVIS_CUDA(cudaStreamSynchronize(s));
        require(bad == 0, "trustworthiness: X contains non-finite values");
        const bool l2 = (distance == kSquaredL2);
        const float *Xp = (const float *)(base + o_Xp);
        const float *sqn = (const float *)(base + o_sqn);
        float *thr = (float *)(base + o_thr);
        int32_t *cnt = (int32_t *)(base + o_cnt);
        NCVIS_LAUNCH(thresholds, (unsigned)ceil_div((int64_t)N * KQ, 256), 256, 0, s, Xp, sqn,
                     (int64_t)N, (int)D, l2, nbr, (int)k, thr);
        NCVIS_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * N * KQ, s));
        const int64_t q_tiles = ceil_div((int64_t)N, BM);
        const int splits = (int)std::max<int64_t>(
            1, std::min<int64_t>(64, ceil_div(2 * (int64_t)num_sms(), q_tiles)));
        NCVIS_LAUNCH(count_closer, dim3((unsigned)q_tiles, (unsigned)splits), NT, 0, s, Xp, sqn,
                     (int64_t)N, (int)D, l2, thr, splits, cnt);
        double *dsum = (double *)(base + o_sum);
        NCVIS_CUDA(cudaMemsetAsync(dsum, 0, sizeof(double), s));
        NCVIS_LAUNCH(penalty_sum, 2 * num_sms(), NT, 0, s, cnt, (int64_t)N, (int)k, dsum);
        double P = 0.0;
        NCVIS_CUDA(cudaMemcpyAsync(&P, dsum, sizeof(double), cudaMemcpyDeviceToHost, s));
        NCVIS_CUDA(cudaStreamSynchronize(s));
        NCVIS_CUDA(cudaFreeAsync(base, s));
        base = nullptr;
        const double n = (double)N, kk = (double)k;
        *out = 1.0 - P * (2.0 / (n * kk * (2.0 * n - 3.0 * kk - 1.0)));
        return NCVIS_OK;
    } catch (const Error &e) {
        if (base) cudaFreeAsync(base, s);
        record_error(e.what());
        return e.code;
    } catch (const std::exception &e) {
        if (base) cudaFreeAsync(base, s);
        record_error(e.what());
        return NCVIS_INTERNAL;
    }
}
