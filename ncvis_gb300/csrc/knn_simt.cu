// K3 + K4: exact kNN in FP32, the plain drop-in replacement for the
// reference's HNSW build and query (src/ncvis.cpp:72-153).
//
// K3 (knn_select_f32): a tiled FP32 FFMA distance GEMM.  A block owns 64
// query points and sweeps one candidate range in tiles of 128; each thread
// accumulates a 4 x 8 patch of dot products.  Distances use the GEMM forms
// |q|^2 + |c|^2 - 2<q,c> (squared L2) and 1 - <q,c> (inner-product spaces).
// Every query keeps a sorted list of its R best (distance, index) pairs in
// shared memory; a tile's distances pass a per-query threshold filter into a
// per-query buffer and are merged into the list between tiles.  Large
// problems use one candidate range; small ones split the range so that the
// grid fills the GPU, and K4 merges the splits.
//
// K4 (rerank): one warp per point recomputes the exact FP32 distance of each
// candidate the way the hnswlib spaces define it (sum of squared
// differences, or 1 - dot; coordinates summed per lane, then across the
// warp), ranks the candidates by (distance, index), drops rank 0 and writes
// ranks k..1, i.e. the k farthest of the k+1 nearest in descending order, as
// findKNN stores them.
#include <algorithm>
#include <cfloat>

#include "common.cuh"
#include "stages.cuh"

namespace ncvis_gpu {

namespace {

constexpr int BM = 64;   // queries per block
constexpr int BN = 128;  // candidates per tile
constexpr int BK = 16;   // reduction slice
constexpr int NT = 256;  // threads per block
constexpr int AS = BM + 4;  // shared-memory row strides (float4-aligned, fewer bank conflicts)
constexpr int BS = BN + 4;

__device__ __forceinline__ bool pair_less(float da, int ia, float db, int ib) {
    return da < db || (da == db && ia < ib);
}

struct SelectSmem {
    float *As;     // [BK][AS]
    float *Bs;     // [BK][BS]
    float *lst_d;  // [R][BM]
    int *lst_i;    // [R][BM]
    float *buf_d;  // [BN][BM]
    int *buf_i;    // [BN][BM]
    int *lst_n;    // [BM]
    int *buf_n;    // [BM]
    float *thr;    // [BM]
};

__host__ __device__ inline size_t select_smem_bytes(int R) {
    return sizeof(float) * (BK * AS + BK * BS) + (sizeof(float) + sizeof(int)) * (size_t)R * BM +
           (sizeof(float) + sizeof(int)) * (size_t)BN * BM + sizeof(int) * 2 * BM +
           sizeof(float) * BM;
}

__device__ inline SelectSmem carve(char *base, int R) {
    SelectSmem s;
    s.As = (float *)base;
    s.Bs = s.As + BK * AS;
    s.lst_d = s.Bs + BK * BS;
    s.lst_i = (int *)(s.lst_d + R * BM);
    s.buf_d = (float *)(s.lst_i + R * BM);
    s.buf_i = (int *)(s.buf_d + BN * BM);
    s.lst_n = s.buf_i + BN * BM;
    s.buf_n = s.lst_n + BM;
    s.thr = (float *)(s.buf_n + BM);
    return s;
}

// With seg.B > 0 the points form seg.B independent problems, problem p owning
// rows [offsets[p], offsets[p+1]) and query tiles [tile_prefix[p],
// tile_prefix[p+1]); a query only sees candidates of its own problem.
__global__ void __launch_bounds__(NT) knn_select_f32(const float *__restrict__ Xp,
                                                     const float *__restrict__ sqnorm, int64_t N,
                                                     int D, int dist, int R, int splits,
                                                     int32_t *__restrict__ cand_i,
                                                     float *__restrict__ cand_d, Segments seg) {
    extern __shared__ __align__(16) char smem_raw[];
    SelectSmem sm = carve(smem_raw, R);
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    int64_t q0 = (int64_t)blockIdx.x * BM, lo = 0, hi = N;
    if (seg.B > 0) {
        const int p = segment_of(seg.tile_prefix, seg.B, blockIdx.x);
        lo = seg.offsets[p];
        hi = seg.offsets[p + 1];
        q0 = lo + ((int64_t)blockIdx.x - seg.tile_prefix[p]) * BM;
    }
    const int64_t n_seg = hi - lo;
    const int split = blockIdx.y;
    const int64_t c_begin = lo + n_seg * split / splits;
    const int64_t c_end = lo + n_seg * (split + 1) / splits;
    N = hi;  // queries of this tile stop at the end of their problem
    const bool l2 = (dist == kSquaredL2);

    if (tid < BM) {
        sm.lst_n[tid] = 0;
        sm.buf_n[tid] = 0;
        sm.thr[tid] = FLT_MAX;
    }
    float qn[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        int64_t q = q0 + ty * 4 + i;
        qn[i] = (q < N) ? sqnorm[q] : 0.f;
    }
    __syncthreads();

    // Global -> register staging of one K slice: thread t holds the 4 values
    // (k0 + 4 (t & 3) ..) of query row t / 4 and of candidate rows t / 4 and
    // t / 4 + 64 (float4 loads when D is a multiple of 4).
    const bool vec = (D & 3) == 0;
    const int lr = tid >> 2, lk = (tid & 3) * 4;
    auto load4 = [&](int64_t row, int64_t row_end, int kc, float4 &v) {
        if (row < row_end && vec && kc < D) {
            v = __ldg(reinterpret_cast<const float4 *>(Xp + row * D + kc));
        } else {
            v.x = (row < row_end && kc < D) ? Xp[row * D + kc] : 0.f;
            v.y = (row < row_end && kc + 1 < D) ? Xp[row * D + kc + 1] : 0.f;
            v.z = (row < row_end && kc + 2 < D) ? Xp[row * D + kc + 2] : 0.f;
            v.w = (row < row_end && kc + 3 < D) ? Xp[row * D + kc + 3] : 0.f;
        }
    };
    auto store4 = [&](float *M, int stride, int row, const float4 &v) {
        M[(lk + 0) * stride + row] = v.x;
        M[(lk + 1) * stride + row] = v.y;
        M[(lk + 2) * stride + row] = v.z;
        M[(lk + 3) * stride + row] = v.w;
    };

    for (int64_t c0 = c_begin; c0 < c_end; c0 += BN) {
        float acc[4][8];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;

        float4 ra, rb0, rb1;
        load4(q0 + lr, N, lk, ra);
        load4(c0 + lr, c_end, lk, rb0);
        load4(c0 + 64 + lr, c_end, lk, rb1);
        for (int k0 = 0; k0 < D; k0 += BK) {
            store4(sm.As, AS, lr, ra);
            store4(sm.Bs, BS, lr, rb0);
            store4(sm.Bs, BS, lr + 64, rb1);
            __syncthreads();
            if (k0 + BK < D) {  // next slice in flight while this one is used
                load4(q0 + lr, N, k0 + BK + lk, ra);
                load4(c0 + lr, c_end, k0 + BK + lk, rb0);
                load4(c0 + 64 + lr, c_end, k0 + BK + lk, rb1);
            }
#pragma unroll
            for (int kk = 0; kk < BK; ++kk) {
                const float4 a = *reinterpret_cast<const float4 *>(&sm.As[kk * AS + ty * 4]);
                const float4 b0 = *reinterpret_cast<const float4 *>(&sm.Bs[kk * BS + tx * 4]);
                const float4 b1 = *reinterpret_cast<const float4 *>(&sm.Bs[kk * BS + 64 + tx * 4]);
                const float b[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
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

        // Threshold filter into the per-query buffers.
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int64_t gc = c0 + (j < 4 ? tx * 4 + j : 64 + tx * 4 + (j - 4));
            if (gc >= c_end) continue;
            const float cn = l2 ? sqnorm[gc] : 0.f;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int q = ty * 4 + i;
                if (q0 + q >= N) continue;
                const float dv = l2 ? (qn[i] + cn) - 2.f * acc[i][j] : 1.f - acc[i][j];
                if (dv <= sm.thr[q]) {
                    const int slot = atomicAdd(&sm.buf_n[q], 1);
                    sm.buf_d[slot * BM + q] = dv;
                    sm.buf_i[slot * BM + q] = (int)gc;
                }
            }
        }
        __syncthreads();

        // Merge each query's buffer into its sorted list.
        if (tid < BM) {
            const int q = tid;
            int n = sm.lst_n[q];
            const int nb = sm.buf_n[q];
            for (int t = 0; t < nb; ++t) {
                const float dv = sm.buf_d[t * BM + q];
                const int iv = sm.buf_i[t * BM + q];
                if (n == R) {
                    if (!pair_less(dv, iv, sm.lst_d[(R - 1) * BM + q], sm.lst_i[(R - 1) * BM + q]))
                        continue;
                    --n;
                }
                int p = n;
                while (p > 0 && pair_less(dv, iv, sm.lst_d[(p - 1) * BM + q],
                                          sm.lst_i[(p - 1) * BM + q])) {
                    sm.lst_d[p * BM + q] = sm.lst_d[(p - 1) * BM + q];
                    sm.lst_i[p * BM + q] = sm.lst_i[(p - 1) * BM + q];
                    --p;
                }
                sm.lst_d[p * BM + q] = dv;
                sm.lst_i[p * BM + q] = iv;
                ++n;
            }
            sm.lst_n[q] = n;
            sm.buf_n[q] = 0;
            sm.thr[q] = (n == R) ? sm.lst_d[(R - 1) * BM + q] : FLT_MAX;
        }
        __syncthreads();
    }

    // Write this split's list; empty slots are marked with index -1.
    const int C = R * splits;
    for (int t = tid; t < BM * R; t += NT) {
        const int q = t % BM, p = t / BM;
        const int64_t gq = q0 + q;
        if (gq >= N) continue;
        const bool have = p < sm.lst_n[q];
        cand_i[gq * C + (int64_t)split * R + p] = have ? sm.lst_i[p * BM + q] : -1;
        cand_d[gq * C + (int64_t)split * R + p] = have ? sm.lst_d[p * BM + q] : FLT_MAX;
    }
}

// One warp per point.  The query row is spread over the lanes (coordinate
// t in lane t % 32); each candidate row is read coalesced and its exact FP32
// distance reduced across the warp (the same lane split for (i, j) and
// (j, i), so d(i, j) == d(j, i)).  Candidates are then ranked; C <= 1024.
template <int T>  // ceil(D / 32) coordinates per lane, T <= 4; T == 0: any D
__global__ void __launch_bounds__(128) rerank_rows(const float *__restrict__ Xp, int64_t N, int D,
                                                   int dist, const int32_t *__restrict__ cand_i,
                                                   int C, int k, int32_t *__restrict__ inds,
                                                   float *__restrict__ dists,
                                                   const int32_t *__restrict__ order) {
    extern __shared__ __align__(16) char smem_raw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp;
    float *sd = (float *)smem_raw + (size_t)warp * C * 2;
    int *si = (int *)(sd + C);
    if (w >= N) return;
    // Rows in `order` (a permutation of [0, N)) when given: neighbouring points
    // then run together and share their candidates' rows in L2.
    const int64_t row = order ? (int64_t)order[w] : w;
    const float *q = Xp + row * D;
    const bool l2 = (dist == kSquaredL2);
    float qv[T > 0 ? T : 1];
    if (T > 0) {
#pragma unroll
        for (int t = 0; t < T; ++t) {
            const int c = lane + 32 * t;
            qv[t] = c < D ? q[c] : 0.f;
        }
    }
    // Candidates in flight per warp: 8 (64 registers) took the rerank of
    // 1,024,000 rows x 32 candidates from 3.84 to 2.68 ms against 4; 16 (128
    // registers, half the resident warps) 4.02 ms.
    constexpr int U = 8;
    for (int c0 = 0; c0 < C; c0 += U) {
        int idx[U];
        float part[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            idx[u] = (c0 + u < C) ? cand_i[row * C + c0 + u] : -1;  // warp-uniform
            part[u] = 0.f;
        }
        if (T > 0) {
#pragma unroll
            for (int t = 0; t < T; ++t) {
                const int col = lane + 32 * t;
                float yv[U];
#pragma unroll
                for (int u = 0; u < U; ++u)
                    yv[u] = (idx[u] >= 0 && col < D) ? Xp[(int64_t)idx[u] * D + col] : 0.f;
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    if (col < D) {
                        if (l2) {
                            const float diff = __fsub_rn(qv[t], yv[u]);
                            part[u] = __fadd_rn(part[u], __fmul_rn(diff, diff));
                        } else {
                            part[u] = __fadd_rn(part[u], __fmul_rn(qv[t], yv[u]));
                        }
                    }
                }
            }
        } else {
#pragma unroll
            for (int u = 0; u < U; ++u) {
                if (idx[u] < 0) continue;
                const float *y = Xp + (int64_t)idx[u] * D;
                for (int col = lane; col < D; col += 32) {
                    const float yv = y[col];
                    if (l2) {
                        const float diff = __fsub_rn(q[col], yv);
                        part[u] = __fadd_rn(part[u], __fmul_rn(diff, diff));
                    } else {
                        part[u] = __fadd_rn(part[u], __fmul_rn(q[col], yv));
                    }
                }
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                part[u] = __fadd_rn(part[u], __shfl_xor_sync(0xffffffffu, part[u], o));
            if (lane == 0 && c0 + u < C) {
                sd[c0 + u] = idx[u] >= 0 ? (l2 ? part[u] : __fsub_rn(1.f, part[u])) : FLT_MAX;
                si[c0 + u] = idx[u];
            }
        }
    }
    __syncwarp();
    for (int c = lane; c < C; c += 32) {
        const int idx = si[c];
        if (idx < 0) continue;
        const float dv = sd[c];
        int rank = 0;
        for (int t = 0; t < C; ++t) {
            const int it = si[t];
            rank += (it >= 0 && pair_less(sd[t], it, dv, idx)) ? 1 : 0;
        }
        if (rank >= 1 && rank <= k) {
            inds[row * k + (k - rank)] = idx;
            dists[row * k + (k - rank)] = dv;
        }
    }
}

}  // namespace

int knn_f32_query_tile() { return BM; }

KnnPlan plan_knn_f32(int64_t N, int k, int rerank_factor) {
    KnnPlan p;
    if (rerank_factor <= 0) rerank_factor = 2;
    int64_t R = std::max<int64_t>((int64_t)rerank_factor * k, (int64_t)k + 1);
    R = std::min<int64_t>(R, N);
    R = std::min<int64_t>(R, 256);
    p.R = (int)R;
    // Split the candidate range until the grid covers the GPU twice.
    const int64_t tiles = (N + BM - 1) / BM;
    int splits = 1;
    while (tiles * splits < 2 * num_sms() && splits * 2 * p.R <= 1024 &&
           N / (splits * 2) >= BN)
        splits *= 2;
    p.splits = splits;
    return p;
}

void launch_knn_select_f32(const float *Xp, const float *sqnorm, int64_t N, int D, int dist,
                           const KnnPlan &plan, int32_t *cand_i, float *cand_d, cudaStream_t s,
                           const Segments &seg) {
    const size_t smem = select_smem_bytes(plan.R);
    // Set on every launch: the attribute is per device, and a cached flag
    // would race between host threads running different engines.
    NCVIS_CUDA(cudaFuncSetAttribute(knn_select_f32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
    const int64_t tiles = seg.B > 0 ? seg.n_tiles : (int64_t)ceil_div(N, BM);
    dim3 grid((unsigned)tiles, plan.splits);
    NCVIS_LAUNCH(knn_select_f32, grid, NT, smem, s, Xp, sqnorm, N, D, dist, plan.R, plan.splits,
                 cand_i, cand_d, seg);
}

void launch_rerank(const float *Xp, int64_t N, int D, int dist, const int32_t *cand_i, int C,
                   int k, int32_t *inds, float *dists, cudaStream_t s, const int32_t *order) {
    require(C <= 1024, "rerank: too many candidates per point");
    const int warps = 4;
    const size_t smem = (size_t)warps * C * 8;
    const unsigned grid = ceil_div(N, warps);
    // The shared-memory attribute is set on every launch (per device; no
    // cached flag shared between host threads).
    auto go = [&](auto kernel) {
        NCVIS_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        NCVIS_LAUNCH(kernel, grid, warps * 32, smem, s, Xp, N, D, dist, cand_i, C, k, inds, dists,
                     order);
    };
    switch ((D + 31) / 32) {
        case 1: go(rerank_rows<1>); break;
        case 2: go(rerank_rows<2>); break;
        case 3: go(rerank_rows<3>); break;
        case 4: go(rerank_rows<4>); break;
        default: go(rerank_rows<0>);
    }
}

}  // namespace ncvis_gpu
