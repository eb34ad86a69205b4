// K8: the noise-contrastive loss that NCVis::optimize (src/ncvis.cpp:275-352)
// descends, as a differentiable function of Y and Q.
//
// With Ph(d2) = 1 / (1 + a d2^b) and nu noise samples per positive edge, the
// loss of a batch of edges (i, j) is
//   L = sum_edges [ softplus(log nu + Q - log Ph(|y_i - y_j|^2))
//                 + sum_{s < nu} softplus(log Ph(|y_i - y_o_s|^2) - Q - log nu) ],
// o_s the edge's noise samples (noise_index in rng.cuh, keyed by the seed and
// counted by the global edge index, so forward and backward see the same
// samples without storing them).  Its gradient is the reference's update:
//   dL/dQ      = w,  w = 1/(1 + Ph/(nu e^Q)) (positive) | -1/(1 + nu e^Q/Ph) (noise)
//   dL/dy_i    = g (y_i - y_o),  g = 2 w a b Ph d2^(b-1);   dL/dy_o = -dL/dy_i
// i.e. the reference moves y_i by clip(-step dL/dy_i) and Q by -alpha_Q dL/dQ
// (before its clip and its sequential Q copy).  Per-sample terms are FP32;
// the loss and dL/dQ are reduced in FP64 (per-block partials, then one block).
#include <algorithm>
#include <cfloat>
#include <cmath>

#include "common.cuh"
#include "rng.cuh"
#include "stages.cuh"

namespace ncvis_gpu {

namespace {

constexpr int kThreads = kNceThreads;

struct NceConst {
    float a, b, log_nu, Q, pow_b1_at_zero;
    int nu;
    uint32_t k0, k1, tag;
};

// Terms of one sample: loss, dL/dQ (w) and g (dL/dy_i = g (y_i - y_o)).
// d2^(b-1) is d2^b / d2; softplus and the sigmoid share exp(-|u|).
__device__ __forceinline__ void sample_terms(float d2, bool positive, const NceConst &c,
                                             float &loss, float &w, float &g) {
    const float p = d2 > 0.f ? powf(d2, c.b) : 0.f;
    const float p1 = d2 > 0.f ? p / d2 : c.pow_b1_at_zero;
    const float ap = c.a * p;
    const float log_ph = -log1pf(ap);
    const float ph = 1.f / (1.f + ap);
    const float u = positive ? c.log_nu + c.Q - log_ph : log_ph - c.Q - c.log_nu;
    const float t = __expf(-fabsf(u));
    loss = fmaxf(u, 0.f) + log1pf(t);
    const float sg = u >= 0.f ? 1.f / (1.f + t) : t / (1.f + t);
    w = positive ? sg : -sg;
    g = 2.f * w * c.a * c.b * ph * p1;
}

__device__ __forceinline__ void block_sum2(double v0, double v1, double *part) {
    __shared__ double red[2][kThreads / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v0 += __shfl_xor_sync(0xffffffffu, v0, o);
        v1 += __shfl_xor_sync(0xffffffffu, v1, o);
    }
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = v0;
        red[1][threadIdx.x >> 5] = v1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s0 = 0, s1 = 0;
        for (int w = 0; w < kThreads / 32; ++w) s0 += red[0][w], s1 += red[1][w];
        part[2 * blockIdx.x] = s0;
        part[2 * blockIdx.x + 1] = s1;
    }
}

// One thread per edge.  mode 0: loss partials; mode 1: gradient (dY scaled by
// *scale, accumulated atomically) and dL/dQ partials.
__global__ void __launch_bounds__(kThreads) nce_edges(int mode, int64_t E, int d, uint32_t N,
                                                      const int32_t *__restrict__ src,
                                                      const int32_t *__restrict__ dst,
                                                      const float *__restrict__ Y,
                                                      const float *__restrict__ Qp,
                                                      uint64_t edge_offset, NceConst c,
                                                      const float *__restrict__ scale,
                                                      float *__restrict__ dY,
                                                      double *__restrict__ part) {
    const int64_t e = (int64_t)blockIdx.x * kThreads + threadIdx.x;
    c.Q = *Qp;
    double acc_loss = 0.0, acc_dq = 0.0;
    if (e < E) {
        const int64_t i = src[e];
        const float sc = (mode == 1) ? *scale : 0.f;
        for (int s = 0; s <= c.nu; ++s) {
            const int64_t o = (s == 0) ? (int64_t)dst[e]
                                       : (int64_t)noise_index(c.k0, c.k1, edge_offset + e, c.tag,
                                                              (uint32_t)(s - 1), (uint32_t)i, N);
            float d2 = 0.f;
            for (int q = 0; q < d; ++q) {
                const float t = Y[i * d + q] - Y[o * d + q];
                d2 = fmaf(t, t, d2);
            }
            float loss, w, g;
            sample_terms(d2, s == 0, c, loss, w, g);
            acc_loss += loss;
            acc_dq += w;
            if (mode == 1 && o != i) {
                const float gs = g * sc;
                for (int q = 0; q < d; ++q) {
                    const float diff = Y[i * d + q] - Y[o * d + q];
                    atomicAdd(&dY[i * d + q], gs * diff);
                    atomicAdd(&dY[o * d + q], -gs * diff);
                }
            }
        }
    }
    block_sum2(acc_loss, acc_dq, part);
}

template <int D>
struct Row {
    float v[D];
};

template <int D>
__device__ __forceinline__ Row<D> load_row(const float *__restrict__ Y, int64_t i) {
    Row<D> r;
    const float *p = Y + i * D;
    if constexpr (D % 4 == 0) {
#pragma unroll
        for (int q = 0; q < D; q += 4) {
            const float4 t = __ldg(reinterpret_cast<const float4 *>(p + q));
            r.v[q] = t.x, r.v[q + 1] = t.y, r.v[q + 2] = t.z, r.v[q + 3] = t.w;
        }
    } else if constexpr (D == 2) {
        const float2 t = __ldg(reinterpret_cast<const float2 *>(p));
        r.v[0] = t.x, r.v[1] = t.y;
    } else {
#pragma unroll
        for (int q = 0; q < D; ++q) r.v[q] = __ldg(p + q);
    }
    return r;
}

// dY[i] += g as L2 vector reductions.
template <int D>
__device__ __forceinline__ void add_row(float *dY, int64_t i, const Row<D> &g) {
    float *p = dY + i * D;
    if constexpr (D % 4 == 0) {
#pragma unroll
        for (int q = 0; q < D; q += 4)
            asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p + q),
                         "f"(g.v[q]), "f"(g.v[q + 1]), "f"(g.v[q + 2]), "f"(g.v[q + 3])
                         : "memory");
    } else if constexpr (D == 2) {
        asm volatile("red.global.add.v2.f32 [%0], {%1, %2};" ::"l"(p), "f"(g.v[0]), "f"(g.v[1])
                     : "memory");
    } else {
#pragma unroll
        for (int q = 0; q < D; ++q) atomicAdd(p + q, g.v[q]);
    }
}

// nce_edges for d = D with rows of 4 D bytes aligned to their vector width:
// y_i read once per edge and its gradient summed in registers, noise drawn
// two samples per Philox block (the same indices as noise_index) and the rows
// of several samples loaded per round trip, the y_o gradients applied as L2
// reductions, per-thread sums in FP32 (1 + nu terms, in sample order) and the
// block sums in FP64.
template <int D>
__global__ void __launch_bounds__(kThreads) nce_edges_t(int mode, int64_t E, uint32_t N,
                                                        const int32_t *__restrict__ src,
                                                        const int32_t *__restrict__ dst,
                                                        const float *__restrict__ Y,
                                                        const float *__restrict__ Qp,
                                                        uint64_t edge_offset, NceConst c,
                                                        const float *__restrict__ scale,
                                                        float *__restrict__ dY,
                                                        double *__restrict__ part) {
    const int64_t e = (int64_t)blockIdx.x * kThreads + threadIdx.x;
    c.Q = *Qp;
    float acc_loss = 0.f, acc_dq = 0.f;
    if (e < E) {
        const int64_t i = src[e];
        const Row<D> yi = load_row<D>(Y, i);
        const float sc = (mode == 1) ? *scale : 0.f;
        Row<D> gi;
#pragma unroll
        for (int q = 0; q < D; ++q) gi.v[q] = 0.f;
        // Rows loaded a group at a time (Y does not change during the loss):
        // the positive row together with the first group of noise rows, then
        // kG noise rows per round trip, noise samples 2p, 2p+1 from Philox
        // block p (noise_pair, the indices noise_index gives).
        constexpr int kG = D <= 4 ? 8 : (D <= 8 ? 4 : 2);
        const uint64_t eg = edge_offset + (uint64_t)e;
        uint32_t o[kG];
        Row<D> yo[kG];
        auto fetch = [&](int n0) {
#pragma unroll
            for (int t = 0; t < kG; t += 2)
                if (n0 + t < c.nu)
                    noise_pair(c.k0, c.k1, eg, c.tag, (uint32_t)(n0 + t) >> 1, (uint32_t)i, N, o[t],
                               o[t + 1]);
#pragma unroll
            for (int t = 0; t < kG; ++t)
                if (n0 + t < c.nu) yo[t] = load_row<D>(Y, o[t]);
        };
        auto sample = [&](uint32_t ot, const Row<D> &yr, bool positive) {
            Row<D> diff;
            float d2 = 0.f;
#pragma unroll
            for (int q = 0; q < D; ++q) {
                diff.v[q] = yi.v[q] - yr.v[q];
                d2 = fmaf(diff.v[q], diff.v[q], d2);
            }
            float loss, w, g;
            sample_terms(d2, positive, c, loss, w, g);
            acc_loss += loss;
            acc_dq += w;
            if (mode == 1 && (int64_t)ot != i) {
                const float gs = g * sc;
                Row<D> go;
#pragma unroll
                for (int q = 0; q < D; ++q) {
                    gi.v[q] = fmaf(gs, diff.v[q], gi.v[q]);
                    go.v[q] = -gs * diff.v[q];
                }
                add_row<D>(dY, ot, go);
            }
        };
        const uint32_t oj = (uint32_t)dst[e];
        const Row<D> yj = load_row<D>(Y, oj);
        if (c.nu > 0) fetch(0);
        sample(oj, yj, true);
        for (int n0 = 0; n0 < c.nu; n0 += kG) {
#pragma unroll
            for (int t = 0; t < kG; ++t) {
                if (n0 + t >= c.nu) break;
                sample(o[t], yo[t], false);
            }
            if (n0 + kG < c.nu) fetch(n0 + kG);
        }
        if (mode == 1) add_row<D>(dY, i, gi);
    }
    block_sum2((double)acc_loss, (double)acc_dq, part);
}

// out[0] = sum of part[2b + which] over blocks (FP64), optionally scaled.
__global__ void finish_sum(const double *__restrict__ part, int blocks, int which,
                           const float *__restrict__ scale, double *__restrict__ out) {
    __shared__ double red[32];
    double s = 0;
    for (int b = threadIdx.x; b < blocks; b += blockDim.x) s += part[2 * b + which];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        out[0] = scale ? t * (double)*scale : t;
    }
}

__global__ void noise_table(int64_t E, uint32_t N, const int32_t *__restrict__ src, int nu,
                            uint32_t k0, uint32_t k1, uint32_t tag, uint64_t edge_offset,
                            int32_t *__restrict__ out) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= E * nu) return;
    const int64_t e = t / nu;
    const int s = (int)(t % nu);
    out[t] = (int32_t)noise_index(k0, k1, edge_offset + e, tag, (uint32_t)s, (uint32_t)src[e], N);
}

}  // namespace

void launch_noise_table(int64_t N, int64_t E, const int32_t *src, int nu, uint64_t seed,
                        uint32_t tag, uint64_t edge_offset, int32_t *out, cudaStream_t s) {
    if (E == 0 || nu == 0) return;
    uint32_t k0, k1;
    noise_key(seed, k0, k1);
    NCVIS_LAUNCH(noise_table, ceil_div(E * nu, kThreads), kThreads, 0, s, E, (uint32_t)N, src, nu,
                 k0, k1, tag, edge_offset, out);
}

size_t nce_workspace_bytes(int64_t E) {
    return sizeof(double) * 2 * ((E + kThreads - 1) / kThreads + 1);
}

void run_nce(int mode, int64_t N, int d, int64_t E, const int32_t *src, const int32_t *dst,
             const float *Y, const float *Q, int nu, float a, float b, uint64_t seed,
             uint32_t tag, uint64_t edge_offset, const float *scale, float *dY, double *out,
             void *workspace, cudaStream_t s) {
    NceConst c;
    c.a = a;
    c.b = b;
    c.nu = nu;
    c.log_nu = logf((float)std::max(nu, 1));
    c.Q = 0.f;
    c.pow_b1_at_zero = std::pow(0.f, b - 1.f);
    noise_key(seed, c.k0, c.k1);
    c.tag = tag;
    const int blocks = (int)std::max<int64_t>((E + kThreads - 1) / kThreads, 1);
    double *part = (double *)workspace;
    // Templated kernels where a row's vector loads and reductions are aligned.
    const uintptr_t rows = (uintptr_t)Y | (uintptr_t)(mode == 1 ? dY : Y);
    const bool v2 = (rows & 7) == 0, v4 = (rows & 15) == 0;
#define NCE_T(DD)                                                                                 \
    NCVIS_LAUNCH(nce_edges_t<DD>, blocks, kThreads, 0, s, mode, E, (uint32_t)N, src, dst, Y, Q, \
                 edge_offset, c, scale, dY, part)
    if (d == 1)
        NCE_T(1);
    else if (d == 2 && v2)
        NCE_T(2);
    else if (d == 4 && v4)
        NCE_T(4);
    else if (d == 8 && v4)
        NCE_T(8);
    else if (d == 16 && v4)
        NCE_T(16);
    else
        NCVIS_LAUNCH(nce_edges, blocks, kThreads, 0, s, mode, E, d, (uint32_t)N, src, dst, Y, Q,
                     edge_offset, c, scale, dY, part);
#undef NCE_T
    NCVIS_LAUNCH(finish_sum, 1, 1024, 0, s, part, blocks, mode == 0 ? 0 : 1,
                 mode == 0 ? nullptr : scale, out);
}

}  // namespace ncvis_gpu
