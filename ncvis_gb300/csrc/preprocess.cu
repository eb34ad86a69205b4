// K1: per-point preprocessing of NCVis::preprocess (src/ncvis.cpp:32-70).
// correlation: subtract the row mean; cosine and correlation: divide by the
// row's Euclidean norm when it is non-zero; squared_L2 and inner_product:
// copy.  One warp per row; the squared norm of the result (for the
// |x|^2 + |y|^2 - 2<x,y> form of squared L2) and the zero-padded BF16
// copies for the tensor-core kNN are produced in the same pass.
#include "common.cuh"
#include "stages.cuh"

namespace ncvis_gpu {

namespace {

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(256) preprocess_rows(const float *__restrict__ X, int64_t N,
                                                       int D, int dist, float *__restrict__ Xp,
                                                       float *__restrict__ sqnorm,
                                                       __nv_bfloat16 *__restrict__ Xb,
                                                       __nv_bfloat16 *__restrict__ Xc, int ldb,
                                                       int *__restrict__ bad_flag) {
    const int lane = threadIdx.x & 31;
    const int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (row >= N) return;
    const float *x = X + row * D;
    float *out = Xp + row * D;

    float mean = 0.f;
    bool finite = true;
    if (dist == kCorrelation) {
        float s = 0.f;
        for (int t = lane; t < D; t += 32) s += x[t];
        mean = warp_sum(s) / (float)D;
    }
    float sq = 0.f;
    for (int t = lane; t < D; t += 32) {
        float v = x[t];
        finite &= isfinite(v);
        v = v - mean;
        sq += v * v;
    }
    sq = warp_sum(sq);
    float scale_div = 1.f;
    const bool normalise = (dist == kCorrelation || dist == kCosine) && sq != 0.f;
    if (normalise) scale_div = sqrtf(sq);
    float sq_out = 0.f;
    for (int t = lane; t < D; t += 32) {
        float v = x[t] - mean;
        if (normalise) v = v / scale_div;
        out[t] = v;
        sq_out += v * v;
        if (Xb) Xb[row * ldb + t] = __float2bfloat16_rn(v);
        if (Xc) Xc[row * ldb + t] = __float2bfloat16_rn(v);
    }
    // With Xc (squared L2 on the tensor cores) columns D and D + 1 hold 1, 1 in
    // the query copy and -|x|^2 / 2 split into a BF16 high and low part in the
    // candidate copy, so that a row pair's product is <q, c> - |c|^2 / 2.
    const int extra = Xc ? 2 : 0;
    if (Xb)
        for (int t = D + extra + lane; t < ldb; t += 32) Xb[row * ldb + t] = __float2bfloat16_rn(0.f);
    if (Xc)
        for (int t = D + extra + lane; t < ldb; t += 32) Xc[row * ldb + t] = __float2bfloat16_rn(0.f);
    sq_out = warp_sum(sq_out);
    if (lane == 0) {
        sqnorm[row] = sq_out;
        if (Xc) {
            const float h = -0.5f * sq_out;
            const __nv_bfloat16 hi = __float2bfloat16_rn(h);
            const __nv_bfloat16 lo = __float2bfloat16_rn(h - __bfloat162float(hi));
            Xb[row * ldb + D] = __float2bfloat16_rn(1.f);
            Xb[row * ldb + D + 1] = __float2bfloat16_rn(1.f);
            Xc[row * ldb + D] = hi;
            Xc[row * ldb + D + 1] = lo;
        }
    }
    if (!__all_sync(0xffffffffu, finite) && lane == 0) atomicOr(bad_flag, 1);
}

}  // namespace

void launch_preprocess(const float *X, int64_t N, int D, int dist, float *Xp, float *sqnorm,
                       __nv_bfloat16 *Xb, int ldb, int *bad_flag, cudaStream_t s,
                       __nv_bfloat16 *Xc) {
    const int warps_per_block = 8;
    NCVIS_LAUNCH(preprocess_rows, ceil_div(N, warps_per_block), 32 * warps_per_block, 0, s, X, N,
                 D, dist, Xp, sqnorm, Xb, Xc, ldb, bad_flag);
}

}  // namespace ncvis_gpu
