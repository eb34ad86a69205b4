// K7: NCVis::optimize (src/ncvis.cpp:275-352), noise-contrastive SGD on the
// embedding Y and the learnable log-normaliser Q.
//
// Per epoch e: step = alpha (1 - (e/n_epochs)^2); every positive edge (i, j)
// is followed by nu_e noise samples o ~ U{0..N-1} \ {i}; for each sample
//   d2 = |y_i - y_o|^2,  Ph = 1 / (1 + a d2^b),
//   w  = 1/(1 + Ph/(nu e^Q)) (positive) | -1/(1 + nu e^Q / Ph) (noise),
//   Q -= alpha_Q w,   w <- 2 w Ph a b d2^(b-1)   (w = 1 when nu == 0),
//   dx = clip((y_o - y_i) w step, +-4),  y_i += dx,  y_o -= dx.
//
// Hogwild mode (sgd_epoch): the reference runs this lock-free on OpenMP
// threads, each with a private copy of Q over a contiguous chunk of the edge
// list, and averages the copies at the end of the epoch.  Here each GPU
// thread is such a chain: a contiguous chunk of edges, a private Q copy, and
// Philox4x32-10 noise keyed by (seed) and counted by (edge, epoch, sample
// pair, retry); the chains' copies are averaged in FP64 by reduce_q.  Y is
// read through L2 (ld.cg) so that chains on other SMs see each other's
// updates as the reference's threads do; y_o -= dx is an L2 reduction
// (red.add), y_i is kept in registers over a run of equal sources and
// written back when the source changes: stored if no one else changed the
// row meanwhile, else as the chain's own change added to it (put_row).
//
// Replay mode (sgd_replay): one thread executes the one-thread reference
// sample by sample, with the reference build's arithmetic grouping (noise
// weight -1/(nu e^Q (1 + a d2^b) + 1), final weight (w d2^(b-1)) ((a b)(Ph+Ph)),
// w*step formed once) in round-to-nearest without contraction, powers and
// exponentials evaluated in double and rounded once, and the noise indices
// read from a recorded stream.
#include <algorithm>
#include <cfloat>
#include <cmath>

#include "common.cuh"
#include "rng.cuh"
#include "stages.cuh"

namespace ncvis_gpu {

namespace {

constexpr int kThreads = 256;

template <int D>
struct Vec {
    float v[D];
};

template <int D>
__device__ __forceinline__ Vec<D> load_row(const float *Y, int64_t i) {
    Vec<D> r;
    if constexpr (D == 2) {
        float2 t = __ldcg(reinterpret_cast<const float2 *>(Y + i * 2));
        r.v[0] = t.x;
        r.v[1] = t.y;
    } else {
#pragma unroll
        for (int c = 0; c < D; ++c) r.v[c] = __ldcg(Y + i * D + c);
    }
    return r;
}

template <int D>
__device__ __forceinline__ void store_row(float *Y, int64_t i, const Vec<D> &r) {
    if constexpr (D == 2) {
        __stcg(reinterpret_cast<float2 *>(Y + i * 2), make_float2(r.v[0], r.v[1]));
    } else {
#pragma unroll
        for (int c = 0; c < D; ++c) __stcg(Y + i * D + c, r.v[c]);
    }
}

// y[row] -= dx as an L2 reduction: no read-modify-write round trip through
// the SM, and concurrent updates of the row by other chains all land (plain
// stores of 8-byte rows from many SMs contend for the same 32-byte sectors
// and run at about half the rate).  With no concurrent writer the result is
// the store of y - dx bit for bit.
template <int D>
__device__ __forceinline__ void sub_row(float *Y, int64_t i, const Vec<D> &dx) {
    float *p = Y + i * D;
    if constexpr (D == 2) {
        asm volatile("red.global.add.v2.f32 [%0], {%1, %2};" ::"l"(p), "f"(-dx.v[0]), "f"(-dx.v[1])
                     : "memory");
    } else if constexpr (D == 4) {
        asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(-dx.v[0]),
                     "f"(-dx.v[1]), "f"(-dx.v[2]), "f"(-dx.v[3])
                     : "memory");
    } else {
#pragma unroll
        for (int c = 0; c < D; ++c)
            asm volatile("red.global.add.f32 [%0], %1;" ::"l"(p + c), "f"(-dx.v[c]) : "memory");
    }
}

// Writes back a source row the chain held in registers (yi; it read yi0 when
// it took the row): a plain store when Y still holds yi0, else only the
// chain's change yi - yi0 is added, as an L2 reduction, so that the updates
// other chains (or the block's window write-back) made to the row while it
// was held are kept.  The reference's threads write every sample to Y at
// once (src/ncvis.cpp:335-338), so theirs are lost only to true races; a
// plain store of the held row would drop every update others made to it
// during a run of its edges.  One chain with no window change to the row
// stores yi bit for bit.
template <int D>
__device__ __forceinline__ void put_row(float *Y, int64_t i, const Vec<D> &yi, const Vec<D> &yi0) {
    const Vec<D> now = load_row<D>(Y, i);
    bool same = true;
#pragma unroll
    for (int c = 0; c < D; ++c) same &= __float_as_uint(now.v[c]) == __float_as_uint(yi0.v[c]);
    if (same) {
        store_row<D>(Y, i, yi);
    } else {
        Vec<D> back;  // yi0 - yi: sub_row adds yi - yi0
#pragma unroll
        for (int c = 0; c < D; ++c) back.v[c] = yi0.v[c] - yi.v[c];
        sub_row<D>(Y, i, back);
    }
}

struct EpochConst {
    float step, nu_f, a, b, ab, alpha_Q, pow_b1_at_zero;
    int nu;
    float b1, ab2;  // b - 1 and 2ab
};

// 2^x by the SFU's approximation (ex2.approx.ftz.f32, PTX ISA).
__device__ __forceinline__ float ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// The update weight of one sample (w * step), Q copy updated in place.
// With Ph = 1/denom, denom = 1 + a d2^b, nm = nu e^Q and t = 1 + nm denom:
//   noise:    w = -1/t,      final weight -(2ab) d2^(b-1) / (t denom)
//   positive: w = 1 - 1/t,   final weight (2ab) d2^(b-1) w / denom
// (the reference's 1/(1 + Ph/nm) and -1/(1 + nm/Ph), src/ncvis.cpp:309-321),
// so one reciprocal, r = 1/(t denom), serves both Q's update and the weight;
// d2^b and d2^(b-1) come from one log2.
__device__ __forceinline__ float nce_weight(float d2, bool positive, const EpochConst &k,
                                            float &Qc) {
    // Every product is rounded on its own (no contraction the compiler may
    // choose per call site), so each kernel that calls this computes the
    // same bits for the same inputs.
    if (k.nu == 0) return k.step;
    float p, p1;
    if (d2 > 0.f) {
        const float lg = __log2f(d2);
        p = ex2_approx(__fmul_rn(k.b, lg));
        p1 = ex2_approx(__fmul_rn(k.b1, lg));
    } else {
        p = 0.f;
        p1 = k.pow_b1_at_zero;
    }
    const float denom = fmaf(k.a, p, 1.f);
    const float t = fmaf(__fmul_rn(k.nu_f, __expf(Qc)), denom, 1.f);
    const float r = __fdividef(1.f, __fmul_rn(t, denom));
    float w;
    if (positive) {
        w = fmaf(-r, denom, 1.f);  // 1 - 1/t
        Qc = fmaf(-w, k.alpha_Q, Qc);
        w = __fmul_rn(__fmul_rn(w, p1), __fmul_rn(k.ab2, __fmul_rn(r, t)));  // r t = 1/denom
    } else {
        Qc = fmaf(__fmul_rn(r, denom), k.alpha_Q, Qc);  // r denom = 1/t
        w = -__fmul_rn(__fmul_rn(p1, k.ab2), r);
    }
    return __fmul_rn(w, k.step);
}

template <int D>
__device__ __forceinline__ float sq_dist(const Vec<D> &x, const Vec<D> &y) {
    float d2 = 0.f;
#pragma unroll
    for (int c = 0; c < D; ++c) {
        const float t = x.v[c] - y.v[c];
        d2 = fmaf(t, t, d2);
    }
    return d2;
}

__device__ __forceinline__ float clip4(float v) { return fminf(fmaxf(v, -4.f), 4.f); }

// Samples of a group whose row was loaded before an earlier sample of the
// same group stored it are reloaded, so a chain always sees its own updates.
template <int D, int G>
__device__ __forceinline__ void run_group(float *Y, Vec<D> &yi, const uint32_t (&o)[G], int count,
                                          bool first_is_positive, const EpochConst &k, float &Qc) {
    Vec<D> yo[G];
#pragma unroll
    for (int t = 0; t < G; ++t)
        if (t < count) yo[t] = load_row<D>(Y, o[t]);
#pragma unroll
    for (int t = 0; t < G; ++t) {
        if (t >= count) break;
        bool dup = false;
#pragma unroll
        for (int u = 0; u < t; ++u) dup |= (o[u] == o[t]);
        if (dup) yo[t] = load_row<D>(Y, o[t]);
        const float ws = nce_weight(sq_dist<D>(yi, yo[t]), first_is_positive && t == 0, k, Qc);
        Vec<D> dx;
#pragma unroll
        for (int c = 0; c < D; ++c) {
            dx.v[c] = clip4((yo[t].v[c] - yi.v[c]) * ws);
            yi.v[c] += dx.v[c];
        }
        sub_row<D>(Y, o[t], dx);
    }
}

// One edge of a chain: the positive sample and its noise samples, with y_i
// held in registers by the caller.
template <int D>
__device__ __forceinline__ void run_edge(float *Y, Vec<D> &yi, uint32_t i, uint32_t j, int64_t e,
                                         uint32_t N, uint32_t lo, const EpochConst &k, float &Qc,
                                         uint32_t key0, uint32_t key1, uint32_t tag) {
    // Rows gathered per round trip: eight for D <= 3; four for D = 4, where
    // eight 4-float rows in flight spill registers.
    constexpr int kGroup = D <= 3 ? 8 : 4;
    int s = 0;  // next noise sample
    if (j != i) {
        // The positive sample and the first kGroup - 2 noise samples share one
        // group (one round trip per edge while nu <= kGroup - 2).
        uint32_t o[kGroup - 1];
        o[0] = j;
        const int first = min(k.nu, kGroup - 2);
#pragma unroll
        for (int p = 0; p < kGroup / 2 - 1; ++p) {
            o[1 + 2 * p] = o[2 + 2 * p] = 0u;
            if (2 * p < first) {
                noise_pair(key0, key1, (uint64_t)e, tag, (uint32_t)p, i - lo, N, o[1 + 2 * p],
                           o[2 + 2 * p]);
                o[1 + 2 * p] += lo;
                o[2 + 2 * p] += lo;
            }
        }
        run_group<D, kGroup - 1>(Y, yi, o, 1 + first, true, k, Qc);
        s = first;
    } else {
        // A self edge: y_i += dx then y_i -= dx on one row (src/ncvis.cpp:337-338).
        const float ws = nce_weight(0.f, true, k, Qc);
#pragma unroll
        for (int c = 0; c < D; ++c) {
            const float dx = clip4(0.f * ws);
            yi.v[c] = (yi.v[c] + dx) - dx;
        }
    }
    // Remaining noise samples in groups of kGroup (kGroup / 2 Philox blocks).
    for (; s < k.nu; s += kGroup) {
        uint32_t o[kGroup];
#pragma unroll
        for (int p = 0; p < kGroup / 2; ++p) {
            noise_pair(key0, key1, (uint64_t)e, tag, (uint32_t)(s >> 1) + p, i - lo, N, o[2 * p],
                       o[2 * p + 1]);
            o[2 * p] += lo;
            o[2 * p + 1] += lo;
        }
        run_group<D, kGroup>(Y, yi, o, min(kGroup, k.nu - s), false, k, Qc);
    }
}

// A chain's edges [e0, e1) (e0 a multiple of 4): edge indices come in aligned
// groups of four, the next group loaded while the current one runs; y_i stays
// in registers while consecutive edges share their source row and is written
// back (put_row) when the row changes.
template <int D>
__device__ __forceinline__ void run_chain(float *Y, const int32_t *__restrict__ src,
                                          const int32_t *__restrict__ dst, int64_t e0, int64_t e1,
                                          uint32_t N, uint32_t lo, const EpochConst &k, float &Qc,
                                          uint32_t key0, uint32_t key1, uint32_t tag) {
    if (e0 >= e1) return;
    auto load4 = [&](int64_t e, int4 &s4, int4 &d4) {
        if (e + 4 <= e1) {
            s4 = __ldg(reinterpret_cast<const int4 *>(src + e));
            d4 = __ldg(reinterpret_cast<const int4 *>(dst + e));
        } else {
            s4.x = src[e];
            d4.x = dst[e];
            s4.y = e + 1 < e1 ? src[e + 1] : 0;
            d4.y = e + 1 < e1 ? dst[e + 1] : 0;
            s4.z = e + 2 < e1 ? src[e + 2] : 0;
            d4.z = e + 2 < e1 ? dst[e + 2] : 0;
            s4.w = e + 3 < e1 ? src[e + 3] : 0;
            d4.w = e + 3 < e1 ? dst[e + 3] : 0;
        }
    };
    int4 s4, d4;
    load4(e0, s4, d4);
    uint32_t cur = (uint32_t)s4.x;
    Vec<D> yi = load_row<D>(Y, cur);
    Vec<D> yi0 = yi;
    for (int64_t e = e0; e < e1; e += 4) {
        int4 ns4 = s4, nd4 = d4;
        if (e + 4 < e1) load4(e + 4, ns4, nd4);
        const int32_t sv[4] = {s4.x, s4.y, s4.z, s4.w};
        const int32_t dv[4] = {d4.x, d4.y, d4.z, d4.w};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            if (e + q >= e1) break;
            const uint32_t i = (uint32_t)sv[q];
            if (i != cur) {
                put_row<D>(Y, cur, yi, yi0);
                cur = i;
                yi = load_row<D>(Y, cur);
                yi0 = yi;
            }
            run_edge<D>(Y, yi, i, (uint32_t)dv[q], e + q, N, lo, k, Qc, key0, key1, tag);
        }
        s4 = ns4;
        d4 = nd4;
    }
    put_row<D>(Y, cur, yi, yi0);
}

template <int D>
__global__ void __launch_bounds__(kThreads) sgd_epoch(float *__restrict__ Y,
                                                      const int32_t *__restrict__ src,
                                                      const int32_t *__restrict__ dst, int64_t E,
                                                      uint32_t N, const float *__restrict__ Q_in,
                                                      double *__restrict__ q_part, EpochConst k,
                                                      int epoch, uint32_t key0, uint32_t key1,
                                                      int64_t chunk, int64_t n_chains) {
    const int64_t chain = (int64_t)blockIdx.x * kThreads + threadIdx.x;
    const int64_t e0 = chain < n_chains ? min(E, chain * chunk) : E;
    const int64_t e1 = min(E, e0 + chunk);
    float Qc = *Q_in;
    run_chain<D>(Y, src, dst, e0, e1, N, 0u, k, Qc, key0, key1, (uint32_t)epoch);
    // Chain copies of Q, summed in FP64 per block.
    __shared__ double red[kThreads / 32];
    double v = chain < n_chains ? (double)Qc : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < kThreads / 32; ++w) t += red[w];
        q_part[blockIdx.x] = t;
    }
}

// Runtime-d variant (d > 4).
__global__ void __launch_bounds__(kThreads) sgd_epoch_generic(
    float *__restrict__ Y, int d, const int32_t *__restrict__ src, const int32_t *__restrict__ dst,
    int64_t E, uint32_t N, const float *__restrict__ Q_in, double *__restrict__ q_part, EpochConst k,
    int epoch, uint32_t key0, uint32_t key1, int64_t chunk, int64_t n_chains) {
    const int64_t chain = (int64_t)blockIdx.x * kThreads + threadIdx.x;
    const int64_t e0 = chain < n_chains ? chain * chunk : E;
    const int64_t e1 = min(E, e0 + chunk);
    float Qc = *Q_in;
    for (int64_t e = e0; e < e1; ++e) {
        const int64_t i = src[e];
        for (int s = 0; s <= k.nu; ++s) {
            const int64_t o = (s == 0) ? (int64_t)dst[e]
                                       : (int64_t)noise_index(key0, key1, (uint64_t)e,
                                                              (uint32_t)epoch, (uint32_t)(s - 1),
                                                              (uint32_t)i, N);
            float d2 = 0.f;
            for (int c = 0; c < d; ++c) {
                const float t = __ldcg(Y + i * d + c) - __ldcg(Y + o * d + c);
                d2 = fmaf(t, t, d2);
            }
            const float ws = nce_weight(d2, s == 0, k, Qc);
            for (int c = 0; c < d; ++c) {
                const float dx = clip4((__ldcg(Y + o * d + c) - __ldcg(Y + i * d + c)) * ws);
                __stcg(Y + i * d + c, __ldcg(Y + i * d + c) + dx);
                __stcg(Y + o * d + c, __ldcg(Y + o * d + c) - dx);
            }
        }
    }
    __shared__ double red[kThreads / 32];
    double v = chain < n_chains ? (double)Qc : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < kThreads / 32; ++w) t += red[w];
        q_part[blockIdx.x] = t;
    }
}

// Batched problems: problem p owns rows [off[p], off[p+1]), edges
// [eoff[p], eoff[p+1]) and chains [cp[p], cp[p+1]); its noise samples are
// uniform over its own rows; chain copies of its Q go to chain_q.
template <int D>
__global__ void __launch_bounds__(kThreads) sgd_epoch_batched(
    float *__restrict__ Y, const int32_t *__restrict__ src, const int32_t *__restrict__ dst,
    const int64_t *__restrict__ off, const int64_t *__restrict__ eoff,
    const int64_t *__restrict__ cp, int B, int64_t n_chains, const float *__restrict__ Qs,
    float *__restrict__ chain_q, EpochConst k, int epoch, uint32_t key0, uint32_t key1) {
    const int64_t chain = (int64_t)blockIdx.x * kThreads + threadIdx.x;
    if (chain >= n_chains) return;
    const int p = segment_of(cp, B, chain);
    const int64_t lc = chain - cp[p], nc = cp[p + 1] - cp[p];
    const int64_t Ep = eoff[p + 1] - eoff[p];
    const int64_t chunk = ((Ep + nc - 1) / nc + 3) & ~(int64_t)3;
    // Aligned to 4 relative to the global edge array: shift by the problem's misalignment.
    const int64_t base = eoff[p];
    int64_t e0 = base + min(Ep, lc * chunk);
    int64_t e1 = base + min(Ep, (lc + 1) * chunk);
    const uint32_t lo = (uint32_t)off[p];
    const uint32_t Np = (uint32_t)(off[p + 1] - off[p]);
    float Qc = Qs[p];
    if (e0 < e1) {
        // Leading edges up to the next multiple of 4 run one by one.
        const int64_t a = min(e1, (e0 + 3) & ~(int64_t)3);
        for (int64_t e = e0; e < a; ++e) {
            Vec<D> yi = load_row<D>(Y, (uint32_t)src[e]);
            const Vec<D> yi0 = yi;
            run_edge<D>(Y, yi, (uint32_t)src[e], (uint32_t)dst[e], e, Np, lo, k, Qc, key0, key1,
                        (uint32_t)epoch);
            put_row<D>(Y, (uint32_t)src[e], yi, yi0);
        }
        run_chain<D>(Y, src, dst, a, e1, Np, lo, k, Qc, key0, key1, (uint32_t)epoch);
    }
    chain_q[chain] = Qc;
}

// Qs[p] = mean of problem p's chain copies (FP64), one block per problem.
__global__ void reduce_q_batched(const float *__restrict__ chain_q, const int64_t *__restrict__ cp,
                                 float *__restrict__ Qs) {
    __shared__ double red[32];
    const int p = blockIdx.x;
    double s = 0;
    for (int64_t c = cp[p] + threadIdx.x; c < cp[p + 1]; c += blockDim.x) s += chain_q[c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        Qs[p] = (float)(t / (double)(cp[p + 1] - cp[p]));
    }
}

// Q = (sum of the chains' copies) / chains, as the reference's epoch-end
// average over threads (src/ncvis.cpp:342-349).
__global__ void reduce_q(const double *__restrict__ q_part, int blocks, int64_t chains,
                         float *__restrict__ Q) {
    __shared__ double red[32];
    double s = 0;
    for (int b = threadIdx.x; b < blocks; b += blockDim.x) s += q_part[b];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        *Q = (float)(t / (double)chains);
    }
}

// ---------------------------------------------------------------- staged noise
//
// Noise samples served from a shared-memory window of Y instead of from the
// whole array.  A block's chains run their edges in rounds; for each round
// the block draws W / kSegRows segment starts uniformly from [0, N), copies
// the window rows (kSegRows consecutive rows from each start, wrapping at N) into
// shared memory with coalesced loads, and every noise sample of the round is
// a uniform pick among the window's rows.  Each pick is therefore uniform
// over [0, N) (the segment start is uniform and the pick within the window
// is uniform).  A pick equal to the edge's source i (probability 1/N) is
// redrawn within the same window, where the reference redraws over all rows
// (src/ncvis.cpp:299-301): rows sharing a segment with i get at most 1/N of
// extra probability per sample.  Otherwise what changes is only that the
// samples of one round of one block share a window.  y_o -= dx is applied to the
// window copy; at the end of the round the window's change (current minus
// loaded) is added to Y with coalesced L2 reductions, so updates made to the
// same rows meanwhile by other blocks are kept.  The positive sample and y_i
// are handled as in sgd_epoch.

constexpr int kWinThreads = 512;
constexpr uint32_t kSegRows = 256;  // rows per window segment

__device__ __forceinline__ uint32_t window_row(const uint32_t *seg, uint32_t u, uint32_t N) {
    const uint32_t r = seg[u / kSegRows] + (u % kSegRows);
    return r >= N ? r - N : r;
}

// Segment t of round r of block b in epoch `tag`: uniform in [0, N).
__device__ __forceinline__ uint32_t segment_start(uint32_t k0, uint32_t k1, uint32_t b, uint32_t r,
                                                  uint32_t tag, uint32_t t, uint32_t N) {
    const Philox4x32 x = philox4x32_10(b, r, tag, t | 0x20000000u, k0 ^ 0x3c6ef372u, k1);
    return bounded_index(x.v[0], x.v[1], N);
}

// A block's window: W rows of the problem of N rows starting at row `base`
// of Y, either 256-row segments at the starts in `seg` (wrapping at N) or,
// `whole`, the problem's rows in order (W == N).
struct WindowSpec {
    const uint32_t *seg;
    uint32_t W, N, base;
    bool whole;
};

__device__ __forceinline__ uint32_t spec_row(const WindowSpec &w, uint32_t u) {
    return w.base + (w.whole ? u : window_row(w.seg, u, w.N));
}

// A noise sample whose window row is the edge source i is redrawn from
// blocks (e_lo, e_hi ^ retry<<16, tag, s/2 | 3<<30) under key (k0 ^ retry, k1),
// up to 64 times; then the next window row is taken.
__device__ __forceinline__ uint32_t window_redraw(uint32_t k0, uint32_t k1, uint64_t e, uint32_t tag,
                                                  uint32_t s, uint32_t u, uint32_t i,
                                                  const WindowSpec &ws) {
    const uint32_t W = ws.W;
    for (uint32_t retry = 1; spec_row(ws, u) == i; ++retry) {
        if (retry > 64) {
            u = (u + 1 == W) ? 0 : u + 1;
            break;
        }
        const Philox4x32 rr = philox4x32_10((uint32_t)e, (uint32_t)(e >> 32) ^ (retry << 16), tag,
                                            (s >> 1) | 0xC0000000u, k0 ^ retry, k1);
        u = bounded_index(rr.v[2 * (s & 1)], rr.v[2 * (s & 1) + 1], W);
    }
    return u;
}

// Window picks of noise samples 8q .. 8q+7 of edge e: the eight 16-bit
// halves of one Philox block (e_lo, e_hi, tag, q | 2^30), each masked to the
// window size (a power of two <= 2^16, so every pick is exactly uniform).
__device__ __forceinline__ Philox4x32 window_block(uint32_t k0, uint32_t k1, uint64_t e,
                                                   uint32_t tag, uint32_t q) {
    return philox4x32_10((uint32_t)e, (uint32_t)(e >> 32), tag, q | 0x40000000u, k0, k1);
}

__device__ __forceinline__ uint32_t window_pick(const Philox4x32 &r, int t, uint32_t W) {
    return (r.v[t >> 1] >> ((t & 1) * 16)) & (W - 1);
}

template <int D>
__device__ __forceinline__ Vec<D> load_win(const float *w, uint32_t u) {
    Vec<D> r;
    if constexpr (D == 2) {
        const float2 t = reinterpret_cast<const float2 *>(w)[u];
        r.v[0] = t.x;
        r.v[1] = t.y;
    } else if constexpr (D == 4) {
        const float4 t = reinterpret_cast<const float4 *>(w)[u];
        r.v[0] = t.x;
        r.v[1] = t.y;
        r.v[2] = t.z;
        r.v[3] = t.w;
    } else {
#pragma unroll
        for (int c = 0; c < D; ++c) r.v[c] = w[u * D + c];
    }
    return r;
}

template <int D>
__device__ __forceinline__ void store_win(float *w, uint32_t u, const Vec<D> &r) {
    if constexpr (D == 2) {
        reinterpret_cast<float2 *>(w)[u] = make_float2(r.v[0], r.v[1]);
    } else if constexpr (D == 4) {
        reinterpret_cast<float4 *>(w)[u] = make_float4(r.v[0], r.v[1], r.v[2], r.v[3]);
    } else {
#pragma unroll
        for (int c = 0; c < D; ++c) w[u * D + c] = r.v[c];
    }
}

// One noise sample against window row u: y_o read from the window and
// y_o - dx stored back, a lock-free read-modify-write like the reference's
// (shared-memory atomics measured ~10% slower for the optimizer at 1,024,000
// points; concurrent updates of one window row are rare).
template <int D>
__device__ __forceinline__ void window_sample(float *win, uint32_t u, Vec<D> &yi,
                                              const EpochConst &k, float &Qc) {
    const Vec<D> yo = load_win<D>(win, u);
    const float ws = nce_weight(sq_dist<D>(yi, yo), false, k, Qc);
    Vec<D> dx, yn;
#pragma unroll
    for (int c = 0; c < D; ++c) {
        dx.v[c] = clip4((yo.v[c] - yi.v[c]) * ws);
        yi.v[c] += dx.v[c];
        yn.v[c] = yo.v[c] - dx.v[c];
    }
    store_win<D>(win, u, yn);
}

// The positive sample of edge (i, j) on the held source row yi, with the
// target row yj (a self edge adds and removes the same step, as the
// reference's y_i += dx; y_i -= dx on one row, src/ncvis.cpp:337-338).
template <int D>
__device__ __forceinline__ void edge_positive(float *Y, uint32_t i, uint32_t j, const Vec<D> &yj,
                                              const EpochConst &k, float &Qc, Vec<D> &yi) {
    if (j != i) {
        const float w = nce_weight(sq_dist<D>(yi, yj), true, k, Qc);
        Vec<D> dx;
#pragma unroll
        for (int c = 0; c < D; ++c) {
            dx.v[c] = clip4((yj.v[c] - yi.v[c]) * w);
            yi.v[c] += dx.v[c];
        }
        sub_row<D>(Y, j, dx);
    } else {
        const float w = nce_weight(0.f, true, k, Qc);
#pragma unroll
        for (int c = 0; c < D; ++c) {
            const float dx = clip4(0.f * w);
            yi.v[c] = (yi.v[c] + dx) - dx;
        }
    }
}

// The nu noise samples of edge e (source i) from the round's window.
// kMulShift: every pick is a 32-bit Philox word scaled to the window by
// multiply-shift (four per block; exactly uniform for any window size W, as
// the window of a whole small problem needs; for a power of two it takes the
// word's top bits); otherwise eight 16-bit halves of a block masked to the
// power-of-two window.
template <int D, bool kMulShift>
__device__ __forceinline__ void edge_noise(int64_t e, uint32_t i, const EpochConst &k, float &Qc,
                                           uint32_t key0, uint32_t key1, uint32_t tag, float *win,
                                           const WindowSpec &ws, Vec<D> &yi) {
    if constexpr (kMulShift) {
        for (int s0 = 0; s0 < k.nu; s0 += 4) {
            const Philox4x32 r = philox4x32_10((uint32_t)e, (uint32_t)(e >> 32), tag,
                                               (uint32_t)(s0 >> 2) | 0x50000000u, key0, key1);
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                if (s0 + t >= k.nu) break;
                const uint32_t pick = (uint32_t)(((uint64_t)r.v[t] * ws.W) >> 32);
                const uint32_t u =
                    window_redraw(key0, key1, (uint64_t)e, tag, (uint32_t)(s0 + t), pick, i, ws);
                window_sample<D>(win, u, yi, k, Qc);
            }
        }
    } else {
        for (int s0 = 0; s0 < k.nu; s0 += 8) {
            const Philox4x32 r = window_block(key0, key1, (uint64_t)e, tag, (uint32_t)(s0 >> 3));
#pragma unroll
            for (int t = 0; t < 8; ++t) {
                if (s0 + t >= k.nu) break;
                const uint32_t u = window_redraw(key0, key1, (uint64_t)e, tag, (uint32_t)(s0 + t),
                                                 window_pick(r, t, ws.W), i, ws);
                window_sample<D>(win, u, yi, k, Qc);
            }
        }
    }
}

// Switches the held source row to i (writing the previous one back).
template <int D>
__device__ __forceinline__ void hold_source(float *Y, uint32_t i, bool &have, uint32_t &ci,
                                            Vec<D> &yi, Vec<D> &yi0) {
    if (!have || i != ci) {
        if (have) put_row<D>(Y, ci, yi, yi0);
        ci = i;
        yi = load_row<D>(Y, ci);
        yi0 = yi;
        have = true;
    }
}

// Edges [a, b) of a chain against the round's window; the chain's current
// source row (ci, yi, read as yi0; valid when `have`) carries over rounds and
// is written back by put_row.  Two schedules of the positive gathers, both
// exact for one chain: a gathered row that this chain may have written
// between the gather and its use is read again, so the chain always sees its
// own updates.
//
// Pipelined (window_edges_pipelined): while edge e runs, the positive rows of
// edges e+1 .. e+P are in flight and the indices of edge e+P+1 are being
// read; rows written in between are the source held at the gather and the
// sources and targets of the edges run in between.
template <int D, bool kMulShift, int P>
__device__ __forceinline__ void window_edges_pipelined(
    float *Y, const int32_t *__restrict__ src, const int32_t *__restrict__ dst, int64_t a,
    int64_t b, const EpochConst &k, float &Qc, uint32_t key0, uint32_t key1, uint32_t tag,
    float *win, const WindowSpec &ws, bool &have, uint32_t &ci, Vec<D> &yi, Vec<D> &yi0) {
    static_assert(P >= 1 && P <= 3, "pipeline depth");
    if (a >= b) return;
    // Slot q holds edge e+q: indices for q <= P, the gathered row and its
    // stale flag for q < P (edges at or past b are -1).
    int32_t ps[P + 1], pd[P + 1];
    Vec<D> pyj[P];
    bool pst[P];
    const int32_t held0 = have ? (int32_t)ci : -1;
#pragma unroll
    for (int q = 0; q <= P; ++q) {
        ps[q] = a + q < b ? src[a + q] : -1;
        pd[q] = a + q < b ? dst[a + q] : -1;
    }
#pragma unroll
    for (int q = 0; q < P; ++q) {
        pyj[q] = Vec<D>{};
        if (pd[q] >= 0 && pd[q] != ps[q]) pyj[q] = load_row<D>(Y, pd[q]);
        pst[q] = pd[q] == held0;
    }
    for (int64_t e = a; e < b; ++e) {
        const int32_t held = have ? (int32_t)ci : -1;
        Vec<D> nyj = {};
        if (pd[P] >= 0 && pd[P] != ps[P]) nyj = load_row<D>(Y, pd[P]);
        const int32_t ns = e + P + 1 < b ? src[e + P + 1] : -1;
        const int32_t nd = e + P + 1 < b ? dst[e + P + 1] : -1;

        const uint32_t i = (uint32_t)ps[0], j = (uint32_t)pd[0];
        hold_source<D>(Y, i, have, ci, yi, yi0);
        edge_positive<D>(Y, i, j, (j != i && pst[0]) ? load_row<D>(Y, j) : pyj[0], k, Qc, yi);
        edge_noise<D, kMulShift>(e, i, k, Qc, key0, key1, tag, win, ws, yi);
        // Rows in flight that edge e may have written: its source (stored at
        // a later switch), its target, and for the row gathered at this edge
        // the source held before it.
#pragma unroll
        for (int q = 1; q < P; ++q) pst[q] |= (pd[q] == ps[0]) | (pd[q] == pd[0]);
        const bool nst = (pd[P] == held) | (pd[P] == ps[0]) | (pd[P] == pd[0]);
#pragma unroll
        for (int q = 0; q < P - 1; ++q) pyj[q] = pyj[q + 1], pst[q] = pst[q + 1];
        pyj[P - 1] = nyj, pst[P - 1] = nst;
#pragma unroll
        for (int q = 0; q < P; ++q) ps[q] = ps[q + 1], pd[q] = pd[q + 1];
        ps[P] = ns, pd[P] = nd;
    }
}

// Grouped (window_edges_grouped): the indices of four edges in one vector load
// each and their positive rows gathered together before the group runs; rows
// written in between are the source held at the gather and the group's
// earlier sources and targets.  (a is a multiple of 4.)
template <int D, bool kMulShift>
__device__ __forceinline__ void window_edges_grouped(
    float *Y, const int32_t *__restrict__ src, const int32_t *__restrict__ dst, int64_t a,
    int64_t b, const EpochConst &k, float &Qc, uint32_t key0, uint32_t key1, uint32_t tag,
    float *win, const WindowSpec &ws, bool &have, uint32_t &ci, Vec<D> &yi, Vec<D> &yi0) {
    for (int64_t e = a; e < b; e += 4) {
        int32_t sv[4], dv[4];
        if (e + 4 <= b && (e & 3) == 0) {
            const int4 s4 = __ldg(reinterpret_cast<const int4 *>(src + e));
            const int4 d4 = __ldg(reinterpret_cast<const int4 *>(dst + e));
            sv[0] = s4.x, sv[1] = s4.y, sv[2] = s4.z, sv[3] = s4.w;
            dv[0] = d4.x, dv[1] = d4.y, dv[2] = d4.z, dv[3] = d4.w;
        } else {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                sv[q] = e + q < b ? src[e + q] : -1;
                dv[q] = e + q < b ? dst[e + q] : -1;
            }
        }
        Vec<D> yj[4] = {};
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (dv[q] >= 0 && dv[q] != sv[q]) yj[q] = load_row<D>(Y, dv[q]);
        const int32_t ci0 = have ? (int32_t)ci : -1;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            if (e + q >= b) break;
            const uint32_t i = (uint32_t)sv[q], j = (uint32_t)dv[q];
            hold_source<D>(Y, i, have, ci, yi, yi0);
            bool stale = dv[q] == ci0;
#pragma unroll
            for (int x = 0; x < q; ++x) stale |= (dv[q] == sv[x]) | (dv[q] == dv[x]);
            edge_positive<D>(Y, i, j, (j != i && stale) ? load_row<D>(Y, j) : yj[q], k, Qc, yi);
            edge_noise<D, kMulShift>(e + q, i, k, Qc, key0, key1, tag, win, ws, yi);
        }
    }
}

// Schedule by the epoch's noise count: with one noise sample per edge an edge
// is too short for a one-edge pipeline to cover a gather, and the grouped
// form is faster (1,024,000 points, ms per epoch at nu = 1 / 2 / 4 / 8 / 16:
// grouped 0.497 / 0.580 / 0.734 / 1.03 / 1.67, pipelined one edge ahead 0.540
// / 0.568 / 0.653 / 0.860 / 1.39; two and three edges ahead were slower).
// Each kernel instance carries one of them (kGrouped); the single-problem
// optimizer takes the grouped one in the epochs with nu = 1.
template <int D, bool kMulShift, bool kGrouped>
__device__ __forceinline__ void window_edges(float *Y, const int32_t *__restrict__ src,
                                             const int32_t *__restrict__ dst, int64_t a, int64_t b,
                                             const EpochConst &k, float &Qc, uint32_t key0,
                                             uint32_t key1, uint32_t tag, float *win,
                                             const WindowSpec &ws, bool &have, uint32_t &ci,
                                             Vec<D> &yi, Vec<D> &yi0) {
    if constexpr (kGrouped)
        window_edges_grouped<D, kMulShift>(Y, src, dst, a, b, k, Qc, key0, key1, tag, win, ws,
                                           have, ci, yi, yi0);
    else
        window_edges_pipelined<D, kMulShift, 1>(Y, src, dst, a, b, k, Qc, key0, key1, tag, win,
                                                ws, have, ci, yi, yi0);
}

template <int D, bool kGrouped>
__global__ void __launch_bounds__(kWinThreads, 2) sgd_epoch_window(
    float *__restrict__ Y, const int32_t *__restrict__ src, const int32_t *__restrict__ dst,
    int64_t E, uint32_t N, const float *__restrict__ Q_in, double *__restrict__ q_part,
    EpochConst k, int epoch, uint32_t key0, uint32_t key1, int64_t chunk, int64_t n_chains,
    uint32_t W, int round_edges) {
    extern __shared__ __align__(16) float win_smem[];
    float *win = win_smem;                                    // current window rows [W][D]
    float *loaded = win_smem + (size_t)W * D;                 // the rows as loaded [W][D]
    uint32_t *seg = reinterpret_cast<uint32_t *>(loaded + (size_t)W * D);  // [W / kSegRows]
    const int64_t chain = (int64_t)blockIdx.x * kWinThreads + threadIdx.x;
    const int64_t e0 = chain < n_chains ? min(E, chain * chunk) : E;
    const int64_t e1 = min(E, e0 + chunk);
    const int rounds = (int)((chunk + round_edges - 1) / round_edges);
    const uint32_t nseg = W / kSegRows;
    float Qc = *Q_in;
    bool have = false;
    uint32_t ci = 0;
    Vec<D> yi, yi0;
#pragma unroll
    for (int c = 0; c < D; ++c) yi.v[c] = yi0.v[c] = 0.f;
    for (int r = 0; r < rounds; ++r) {
        for (uint32_t t = threadIdx.x; t < nseg; t += kWinThreads)
            seg[t] = segment_start(key0, key1, blockIdx.x, (uint32_t)r, (uint32_t)epoch, t, N);
        __syncthreads();
        for (uint32_t u = threadIdx.x; u < W; u += kWinThreads) {
            const Vec<D> v = load_row<D>(Y, window_row(seg, u, N));
            store_win<D>(win, u, v);
            store_win<D>(loaded, u, v);
        }
        __syncthreads();
        const int64_t a = min(e1, e0 + (int64_t)r * round_edges);
        const int64_t b = min(e1, a + round_edges);
        const WindowSpec ws{seg, W, N, 0u, false};
        window_edges<D, false, kGrouped>(Y, src, dst, a, b, k, Qc, key0, key1, (uint32_t)epoch,
                                         win, ws, have, ci, yi, yi0);
        __syncthreads();
        for (uint32_t u = threadIdx.x; u < W; u += kWinThreads) {
            const Vec<D> now = load_win<D>(win, u), was = load_win<D>(loaded, u);
            Vec<D> minus;  // loaded - current: sub_row adds current - loaded
            bool moved = false;
#pragma unroll
            for (int c = 0; c < D; ++c) {
                minus.v[c] = was.v[c] - now.v[c];
                moved |= (minus.v[c] != 0.f);
            }
            if (moved) sub_row<D>(Y, window_row(seg, u, N), minus);
        }
        __syncthreads();
    }
    if (have) put_row<D>(Y, ci, yi, yi0);
    __shared__ double red[kWinThreads / 32];
    double v = chain < n_chains ? (double)Qc : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < kWinThreads / 32; ++w) t += red[w];
        q_part[blockIdx.x] = t;
    }
}

// Batched problems with staged noise: every block's chains belong to one
// problem (problem p owns blocks [bp[p], bp[p+1]) and chains [cp[p], cp[p+1]),
// the last block of a problem partly idle); the window is the problem's rows
// when they fit or 256-row segments at uniform starts within the problem
// otherwise; either way each pick is a multiply-shift of a 32-bit Philox word
// over the window, exactly uniform.  Blocks of T chains (T in 64, 128,
// 256: the engine's autotuner picks T with the edges per chain).
constexpr uint32_t kBatWindow = 1024;  // rows; two copies of d <= 4 floats fit 32 KB

template <int D, int T>
__global__ void __launch_bounds__(T) sgd_epoch_window_batched(
    float *__restrict__ Y, const int32_t *__restrict__ src, const int32_t *__restrict__ dst,
    const int64_t *__restrict__ off, const int64_t *__restrict__ eoff,
    const int64_t *__restrict__ cp, const int64_t *__restrict__ bp, int B,
    const float *__restrict__ Qs, float *__restrict__ chain_q, EpochConst k, int epoch,
    uint32_t key0, uint32_t key1, int round_edges) {
    __shared__ __align__(16) float win[kBatWindow * D];
    __shared__ __align__(16) float loaded[kBatWindow * D];
    __shared__ uint32_t seg[kBatWindow / kSegRows];
    const int p = segment_of(bp, B, (int64_t)blockIdx.x);
    const int64_t lc = ((int64_t)blockIdx.x - bp[p]) * T + threadIdx.x;
    const int64_t nc = cp[p + 1] - cp[p];
    const int64_t Ep = eoff[p + 1] - eoff[p];
    const int64_t chunk = ((Ep + nc - 1) / nc + 3) & ~(int64_t)3;
    const bool active = lc < nc;
    const int64_t e0 = eoff[p] + (active ? min(Ep, lc * chunk) : Ep);
    const int64_t e1 = eoff[p] + (active ? min(Ep, (lc + 1) * chunk) : Ep);
    const uint32_t base = (uint32_t)off[p];
    const uint32_t Np = (uint32_t)(off[p + 1] - off[p]);
    const bool whole = Np <= kBatWindow;
    const uint32_t W = whole ? Np : kBatWindow;
    const int rounds = (int)((chunk + round_edges - 1) / round_edges);
    const WindowSpec ws{seg, W, Np, base, whole};
    float Qc = Qs[p];
    bool have = false;
    uint32_t ci = 0;
    Vec<D> yi, yi0;
#pragma unroll
    for (int c = 0; c < D; ++c) yi.v[c] = yi0.v[c] = 0.f;
    for (int r = 0; r < rounds; ++r) {
        if (!whole)
            for (uint32_t t = threadIdx.x; t < W / kSegRows; t += T)
                seg[t] = segment_start(key0, key1, blockIdx.x, (uint32_t)r, (uint32_t)epoch, t, Np);
        __syncthreads();
        for (uint32_t u = threadIdx.x; u < W; u += T) {
            const Vec<D> v = load_row<D>(Y, spec_row(ws, u));
            store_win<D>(win, u, v);
            store_win<D>(loaded, u, v);
        }
        __syncthreads();
        const int64_t a = min(e1, e0 + (int64_t)r * round_edges);
        const int64_t b = min(e1, a + round_edges);
        // One pick scheme for both window forms, so the kernel carries one copy
        // of the edge loop (with two, its blocks of both forms on one SM
        // thrashed the instruction cache).
        // The pipelined schedule in every epoch (the grouped one measured the
        // same at one noise sample per edge on the 256-problem workload).
        window_edges<D, true, false>(Y, src, dst, a, b, k, Qc, key0, key1, (uint32_t)epoch, win,
                                     ws, have, ci, yi, yi0);
        __syncthreads();
        for (uint32_t u = threadIdx.x; u < W; u += T) {
            const Vec<D> now = load_win<D>(win, u), was = load_win<D>(loaded, u);
            Vec<D> minus;
            bool moved = false;
#pragma unroll
            for (int c = 0; c < D; ++c) {
                minus.v[c] = was.v[c] - now.v[c];
                moved |= (minus.v[c] != 0.f);
            }
            if (moved) sub_row<D>(Y, spec_row(ws, u), minus);
        }
        __syncthreads();
    }
    if (have) put_row<D>(Y, ci, yi, yi0);
    if (active) chain_q[cp[p] + lc] = Qc;
}

// ---------------------------------------------------------------- replay

// The reference build's d_sqr: left to right for d <= 3; for d >= 4 four
// running lane sums over the first 4*floor(d/4) coordinates, folded as
// (l0 + l2) + (l1 + l3), the remainder added pairwise into the folded lanes.
__device__ float replay_sq_dist(const float *x, const float *y, int d) {
    float lane[4] = {0.f, 0.f, 0.f, 0.f};
    const int body = (d >= 4) ? (d / 4) * 4 : 0;
    for (int t = 0; t < body; t += 4)
        for (int l = 0; l < 4; ++l) {
            const float u = __fsub_rn(x[t + l], y[t + l]);
            lane[l] = __fadd_rn(lane[l], __fmul_rn(u, u));
        }
    float f0 = __fadd_rn(lane[0], lane[2]);
    float f1 = __fadd_rn(lane[1], lane[3]);
    int t = body;
    const int rem = d - body;
    if (rem >= 2) {
        const float u0 = __fsub_rn(x[t], y[t]), u1 = __fsub_rn(x[t + 1], y[t + 1]);
        f0 = __fadd_rn(__fmul_rn(u0, u0), f0);
        f1 = __fadd_rn(__fmul_rn(u1, u1), f1);
        t += 2;
    }
    float acc = __fadd_rn(f0, f1);
    if (t < d) {
        const float u = __fsub_rn(x[t], y[t]);
        acc = __fadd_rn(acc, __fmul_rn(u, u));
    }
    return acc;
}

__device__ __forceinline__ void replay_sample(float *Y, int d, int64_t i, int64_t o, bool positive,
                                              uint64_t nu, float a, float b, float alpha_Q,
                                              float step, float &Qc) {
    const float d2 = replay_sq_dist(Y + i * d, Y + o * d, d);
    float w = 1.f;
    if (nu != 0) {
        const float p = (float)pow((double)d2, (double)b);
        const float denom = __fadd_rn(__fmul_rn(a, p), 1.f);
        const float ph = __fdiv_rn(1.f, denom);
        const float ab2ph = __fmul_rn(__fmul_rn(a, b), __fadd_rn(ph, ph));
        const float nm = __fmul_rn((float)nu, (float)exp((double)Qc));
        w = positive ? __fdiv_rn(1.f, __fadd_rn(__fdiv_rn(ph, nm), 1.f))
                     : __fdiv_rn(-1.f, __fadd_rn(__fmul_rn(nm, denom), 1.f));
        Qc = __fsub_rn(Qc, __fmul_rn(w, alpha_Q));
        const float p1 = (float)pow((double)d2, (double)__fsub_rn(b, 1.f));
        w = __fmul_rn(__fmul_rn(w, p1), ab2ph);
    }
    const float ws = __fmul_rn(w, step);
    for (int c = 0; c < d; ++c) {
        float dx = __fmul_rn(__fsub_rn(Y[o * d + c], Y[i * d + c]), ws);
        dx = fminf(fmaxf(dx, -4.f), 4.f);
        Y[i * d + c] = __fadd_rn(Y[i * d + c], dx);
        Y[o * d + c] = __fsub_rn(Y[o * d + c], dx);
    }
}

// Indices outside [0, N) stop the replay and set *err (no write happens).
__global__ void sgd_replay(float *Y, int64_t N, int d, const int32_t *__restrict__ src,
                           const int32_t *__restrict__ dst, int64_t e0, int64_t e1,
                           const int32_t *__restrict__ stream, int64_t pos, float *Q, int epoch,
                           int n_epochs, uint64_t nu, float a, float b, float alpha, float alpha_Q,
                           int *err) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const float frac = __fdiv_rn((float)epoch, (float)n_epochs);
    const float step = __fmul_rn(alpha, __fsub_rn(1.f, __fmul_rn(frac, frac)));
    float Qc = *Q;
    for (int64_t e = e0; e < e1; ++e) {
        const int64_t i = src[e], j = dst[e];
        if (i < 0 || i >= N || j < 0 || j >= N) {
            *err = 1;
            return;
        }
        replay_sample(Y, d, i, j, true, nu, a, b, alpha_Q, step, Qc);
        for (uint64_t s = 0; s < nu; ++s) {
            const int64_t o = stream[pos++];
            if (o < 0 || o >= N) {
                *err = 1;
                return;
            }
            replay_sample(Y, d, i, o, false, nu, a, b, alpha_Q, step, Qc);
        }
    }
    *Q = Qc;
}

EpochConst epoch_const(const SgdArgs &g, int epoch, int nu) {
    EpochConst k;
    const float frac = (float)epoch / (float)g.n_epochs;
    k.step = g.alpha * (1.f - frac * frac);
    k.nu = nu;
    k.nu_f = (float)nu;
    k.a = g.a;
    k.b = g.b;
    k.ab = g.a * g.b;
    k.alpha_Q = g.alpha_Q;
    k.pow_b1_at_zero = std::pow(0.f, g.b - 1.f);
    k.b1 = g.b - 1.f;
    k.ab2 = 2.f * g.a * g.b;
    return k;
}

}  // namespace

namespace {

// Threads of the d-specialised epoch kernel that fit on the GPU at once.
int64_t resident_chains(int d) {
    int blocks = 0;
    cudaError_t err;
    switch (d) {
        case 1: err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, sgd_epoch<1>, kThreads, 0); break;
        case 2: err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, sgd_epoch<2>, kThreads, 0); break;
        case 3: err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, sgd_epoch<3>, kThreads, 0); break;
        case 4: err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, sgd_epoch<4>, kThreads, 0); break;
        default:
            err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, sgd_epoch_generic, kThreads, 0);
    }
    if (err != cudaSuccess || blocks < 1) blocks = 1;
    return (int64_t)blocks * kThreads * num_sms();
}

}  // namespace

int sgd_default_chains(int64_t E, int64_t N, int d) {
    // Every chain resident at once, each with at least 16 edges so that its
    // copy of Q follows many samples before the epoch average, and at most one
    // chain per 2 points.  y_o updates are L2 reductions, so concurrent chains
    // do not overwrite each other's noise updates; at 10,000 points 1,250,
    // 5,000 and 10,000 chains gave trustworthiness 0.9577, 0.9574 and 0.9569
    // (fit 42, 17 and 11 ms).
    int64_t chains = std::min<int64_t>(resident_chains(d), std::max<int64_t>(E / 16, 1));
    chains = std::min<int64_t>(chains, std::max<int64_t>(N / 2, 1));
    return (int)std::max<int64_t>(chains, 1);
}

size_t sgd_workspace_bytes(int chains) {
    const int64_t most = std::max<int64_t>(chains, (int64_t)num_sms() * 2048);
    return sizeof(double) * ((most + kThreads - 1) / kThreads + 1);
}

void run_sgd_hogwild(const SgdArgs &g, int epoch_begin, int epoch_end, const size_t *n_noise,
                     int chains, void *workspace, cudaStream_t s) {
    require(g.N >= 2 && g.N < (int64_t(1) << 31), "optimize: N must be in [2, 2^31)");
    if (chains <= 0) chains = sgd_default_chains(g.E, g.N, g.d);
    const int blocks = (int)ceil_div(chains, kThreads);
    const int64_t total_chains = chains;
    const int64_t chunk = ((g.E + total_chains - 1) / total_chains + 3) & ~(int64_t)3;
    double *q_part = (double *)workspace;
    uint32_t key0, key1;
    noise_key(g.seed, key0, key1);
    for (int ep = epoch_begin; ep < epoch_end; ++ep) {
        const int nu = (int)n_noise[ep];
        EpochConst k = epoch_const(g, ep, nu);
        switch (g.d) {
            case 1:
                NCVIS_LAUNCH(sgd_epoch<1>, blocks, kThreads, 0, s, g.Y, g.src, g.dst, g.E,
                             (uint32_t)g.N, g.Q, q_part, k, ep, key0, key1, chunk, total_chains);
                break;
            case 2:
                NCVIS_LAUNCH(sgd_epoch<2>, blocks, kThreads, 0, s, g.Y, g.src, g.dst, g.E,
                             (uint32_t)g.N, g.Q, q_part, k, ep, key0, key1, chunk, total_chains);
                break;
            case 3:
                NCVIS_LAUNCH(sgd_epoch<3>, blocks, kThreads, 0, s, g.Y, g.src, g.dst, g.E,
                             (uint32_t)g.N, g.Q, q_part, k, ep, key0, key1, chunk, total_chains);
                break;
            case 4:
                NCVIS_LAUNCH(sgd_epoch<4>, blocks, kThreads, 0, s, g.Y, g.src, g.dst, g.E,
                             (uint32_t)g.N, g.Q, q_part, k, ep, key0, key1, chunk, total_chains);
                break;
            default:
                NCVIS_LAUNCH(sgd_epoch_generic, blocks, kThreads, 0, s, g.Y, g.d, g.src, g.dst,
                             g.E, (uint32_t)g.N, g.Q, q_part, k, ep, key0, key1, chunk, total_chains);
        }
        NCVIS_LAUNCH(reduce_q, 1, 1024, 0, s, q_part, blocks, total_chains, g.Q);
    }
}

// Window rows of the staged-noise kernel: the largest power of two, at most
// 4096, whose two copies of D floats per row fit in 64 KiB.
uint32_t sgd_window_rows(int d) {
    uint32_t w = 4096;
    while (w > kSegRows && (size_t)w * d * 8 > 65536) w >>= 1;
    return w;
}

// Dynamic shared memory of sgd_epoch_window: the window and its loaded copy,
// the segment starts.
size_t window_smem_bytes(int d) {
    const uint32_t W = sgd_window_rows(d);
    return (size_t)W * d * 8 + (W / kSegRows) * 4;
}

bool sgd_window_applies(int64_t N, int d) {
    return d >= 1 && d <= 4 && N >= 16 * (int64_t)sgd_window_rows(d);
}

namespace {

template <int D>
void launch_window_epoch(unsigned blocks, size_t smem, cudaStream_t s, const SgdArgs &g,
                         double *q_part, const EpochConst &k, int ep, uint32_t key0, uint32_t key1,
                         int64_t chunk, int64_t chains, uint32_t W, int round_edges) {
    auto launch = [&](auto kernel) {
        NCVIS_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem));
        NCVIS_LAUNCH(kernel, blocks, kWinThreads, smem, s, g.Y, g.src, g.dst, g.E, (uint32_t)g.N,
                     g.Q, q_part, k, ep, key0, key1, chunk, chains, W, round_edges);
    };
    if (k.nu == 1)
        launch(sgd_epoch_window<D, true>);
    else
        launch(sgd_epoch_window<D, false>);
}

int64_t window_resident_chains(int d) {
    const size_t smem = window_smem_bytes(d);
    int blocks = 0;
    cudaError_t err;
    auto occ = [&](auto kernel) {
        cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kernel, kWinThreads, smem);
    };
    switch (d) {
        case 1: err = occ(sgd_epoch_window<1, false>); break;
        case 2: err = occ(sgd_epoch_window<2, false>); break;
        case 3: err = occ(sgd_epoch_window<3, false>); break;
        default: err = occ(sgd_epoch_window<4, false>);
    }
    if (err != cudaSuccess || blocks < 1) blocks = 1;
    return (int64_t)blocks * kWinThreads * num_sms();
}

}  // namespace

int sgd_window_default_chains(int64_t E, int64_t N, int d) {
    // As sgd_default_chains: every chain resident, at least 16 edges each, at
    // most one chain per 2 points.
    int64_t chains = std::min<int64_t>(window_resident_chains(d), std::max<int64_t>(E / 16, 1));
    chains = std::min<int64_t>(chains, std::max<int64_t>(N / 2, 1));
    return (int)std::max<int64_t>(chains, 1);
}

void run_sgd_window(const SgdArgs &g, int epoch_begin, int epoch_end, const size_t *n_noise,
                    int chains, int round_edges, void *workspace, cudaStream_t s) {
    require(g.N >= 2 && g.N < (int64_t(1) << 31), "optimize: N must be in [2, 2^31)");
    require(sgd_window_applies(g.N, g.d),
            "optimize: staged noise needs 1 <= d <= 4 and N >= 16 window rows");
    if (chains <= 0) chains = sgd_window_default_chains(g.E, g.N, g.d);
    if (round_edges <= 0) round_edges = 16;
    round_edges = (round_edges + 3) & ~3;
    const uint32_t W = sgd_window_rows(g.d);
    const size_t smem = window_smem_bytes(g.d);
    const unsigned blocks = ceil_div(chains, kWinThreads);
    const int64_t total_chains = chains;
    const int64_t chunk = ((g.E + total_chains - 1) / total_chains + 3) & ~(int64_t)3;
    double *q_part = (double *)workspace;
    uint32_t key0, key1;
    noise_key(g.seed, key0, key1);
    for (int ep = epoch_begin; ep < epoch_end; ++ep) {
        EpochConst k = epoch_const(g, ep, (int)n_noise[ep]);
        switch (g.d) {
            case 1:
                launch_window_epoch<1>(blocks, smem, s, g, q_part, k, ep, key0, key1,
                                                   chunk, total_chains, W, round_edges);
                break;
            case 2:
                launch_window_epoch<2>(blocks, smem, s, g, q_part, k, ep, key0, key1,
                                                   chunk, total_chains, W, round_edges);
                break;
            case 3:
                launch_window_epoch<3>(blocks, smem, s, g, q_part, k, ep, key0, key1,
                                                   chunk, total_chains, W, round_edges);
                break;
            default:
                launch_window_epoch<4>(blocks, smem, s, g, q_part, k, ep, key0, key1,
                                                   chunk, total_chains, W, round_edges);
        }
        NCVIS_LAUNCH(reduce_q, 1, 1024, 0, s, q_part, (int)blocks, total_chains, g.Q);
    }
}

bool sgd_window_batched_threads_ok(int threads) {
    return threads == 64 || threads == 128 || threads == 256;
}

template <int D, int T>
void launch_window_batched(const SgdBatch &g, const int64_t *bp, int64_t n_blocks,
                           const EpochConst &k, int ep, uint32_t key0, uint32_t key1,
                           int round_edges, cudaStream_t s) {
    NCVIS_LAUNCH((sgd_epoch_window_batched<D, T>), (unsigned)n_blocks, T, 0, s, g.Y, g.src, g.dst,
                 g.off, g.eoff, g.cp, bp, g.B, g.Qs, g.chain_q, k, ep, key0, key1, round_edges);
}

template <int D>
void launch_window_batched_t(const SgdBatch &g, const int64_t *bp, int64_t n_blocks, int threads,
                             const EpochConst &k, int ep, uint32_t key0, uint32_t key1,
                             int round_edges, cudaStream_t s) {
    switch (threads) {
        case 64: launch_window_batched<D, 64>(g, bp, n_blocks, k, ep, key0, key1, round_edges, s); break;
        case 128: launch_window_batched<D, 128>(g, bp, n_blocks, k, ep, key0, key1, round_edges, s); break;
        default: launch_window_batched<D, 256>(g, bp, n_blocks, k, ep, key0, key1, round_edges, s);
    }
}

void run_sgd_window_batched(const SgdBatch &g, const int64_t *bp, int64_t n_blocks, int threads,
                            const size_t *n_noise, cudaStream_t s) {
    require(g.d >= 1 && g.d <= 4, "batched optimize: d must be in [1, 4]");
    require(sgd_window_batched_threads_ok(threads),
            "batched optimize: chains per block must be 64, 128 or 256");
    uint32_t key0, key1;
    noise_key(g.seed, key0, key1);
    const int round_edges = 16;
    for (int ep = 0; ep < g.n_epochs; ++ep) {
        SgdArgs one{0, g.d, 0, nullptr, nullptr, nullptr, nullptr, g.seed, g.n_epochs,
                    g.a, g.b, g.alpha, g.alpha_Q};
        EpochConst k = epoch_const(one, ep, (int)n_noise[ep]);
        switch (g.d) {
            case 1: launch_window_batched_t<1>(g, bp, n_blocks, threads, k, ep, key0, key1, round_edges, s); break;
            case 2: launch_window_batched_t<2>(g, bp, n_blocks, threads, k, ep, key0, key1, round_edges, s); break;
            case 3: launch_window_batched_t<3>(g, bp, n_blocks, threads, k, ep, key0, key1, round_edges, s); break;
            default: launch_window_batched_t<4>(g, bp, n_blocks, threads, k, ep, key0, key1, round_edges, s);
        }
        NCVIS_LAUNCH(reduce_q_batched, g.B, 256, 0, s, g.chain_q, g.cp, g.Qs);
    }
}

void run_sgd_hogwild_batched(const SgdBatch &g, const size_t *n_noise, cudaStream_t s) {
    require(g.d >= 1 && g.d <= 4, "batched optimize: d must be in [1, 4]");
    uint32_t key0, key1;
    noise_key(g.seed, key0, key1);
    const unsigned blocks = ceil_div(g.n_chains, kThreads);
    for (int ep = 0; ep < g.n_epochs; ++ep) {
        SgdArgs one{0, g.d, 0, nullptr, nullptr, nullptr, nullptr, g.seed, g.n_epochs,
                    g.a, g.b, g.alpha, g.alpha_Q};
        EpochConst k = epoch_const(one, ep, (int)n_noise[ep]);
        switch (g.d) {
            case 1:
                NCVIS_LAUNCH(sgd_epoch_batched<1>, blocks, kThreads, 0, s, g.Y, g.src, g.dst, g.off,
                             g.eoff, g.cp, g.B, g.n_chains, g.Qs, g.chain_q, k, ep, key0, key1);
                break;
            case 2:
                NCVIS_LAUNCH(sgd_epoch_batched<2>, blocks, kThreads, 0, s, g.Y, g.src, g.dst, g.off,
                             g.eoff, g.cp, g.B, g.n_chains, g.Qs, g.chain_q, k, ep, key0, key1);
                break;
            case 3:
                NCVIS_LAUNCH(sgd_epoch_batched<3>, blocks, kThreads, 0, s, g.Y, g.src, g.dst, g.off,
                             g.eoff, g.cp, g.B, g.n_chains, g.Qs, g.chain_q, k, ep, key0, key1);
                break;
            default:
                NCVIS_LAUNCH(sgd_epoch_batched<4>, blocks, kThreads, 0, s, g.Y, g.src, g.dst, g.off,
                             g.eoff, g.cp, g.B, g.n_chains, g.Qs, g.chain_q, k, ep, key0, key1);
        }
        NCVIS_LAUNCH(reduce_q_batched, g.B, 256, 0, s, g.chain_q, g.cp, g.Qs);
    }
}

int64_t sgd_batched_resident_chains(int d) {
    int blocks = 0;
    cudaError_t err;
    switch (d) {
        case 1: err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, sgd_epoch_batched<1>, kThreads, 0); break;
        case 2: err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, sgd_epoch_batched<2>, kThreads, 0); break;
        case 3: err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, sgd_epoch_batched<3>, kThreads, 0); break;
        default: err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, sgd_epoch_batched<4>, kThreads, 0);
    }
    if (err != cudaSuccess || blocks < 1) blocks = 1;
    return (int64_t)blocks * kThreads * num_sms();
}

void launch_sgd_replay(const SgdArgs &g, int epoch, size_t nu, int64_t edge_begin,
                       int64_t edge_end, const int32_t *stream, int64_t stream_offset, int *err,
                       cudaStream_t s) {
    NCVIS_LAUNCH(sgd_replay, 1, 32, 0, s, g.Y, g.N, g.d, g.src, g.dst, edge_begin, edge_end,
                 stream, stream_offset, g.Q, epoch, g.n_epochs, (uint64_t)nu, g.a, g.b, g.alpha,
                 g.alpha_Q, err);
}

}  // namespace ncvis_gpu
