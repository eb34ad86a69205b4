// ORACLE — test infrastructure, not product code.
//
// CPU restatement of NCVis::optimize (src/ncvis.cpp:275-352) and of the
// negative-sample stream one reference thread draws.  Compiled WITHOUT
// -ffast-math and with -ffp-contract=off (oracle/build_oracle.sh) so that the
// grouping written below is the arithmetic that runs, on any host: it is the
// grouping the reference's own -O3 -ffast-math build evaluates with g++ 13 on
// x86-64, which makes the oracle bit-identical to that build (checked against
// oracle/_ref) instead of to whatever re-association fast-math picks here.
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>

#include "oracle_rng.h"

using namespace orc;

namespace {

// src/ncvis.cpp:175-182 (d_sqr) in the reference build's summation order:
// left to right for d <= 3; for d >= 4 four running lane sums over the first
// 4*floor(d/4) coordinates folded as (l0 + l2) + (l1 + l3), with a remaining
// pair added into the two folded lanes before they are combined and a last
// odd coordinate added at the end (the build's 4-wide SSE reduction).
inline float sq_dist(const float *x, const float *y, size_t d) {
    float lane[4] = {0.f, 0.f, 0.f, 0.f};
    const size_t body = d >= 4 ? (d / 4) * 4 : 0;
    for (size_t t = 0; t < body; t += 4)
        for (size_t l = 0; l < 4; ++l) {
            const float u = x[t + l] - y[t + l];
            lane[l] = lane[l] + u * u;
        }
    float f0 = lane[0] + lane[2];
    float f1 = lane[1] + lane[3];
    size_t t = body;
    if (d - body >= 2) {
        const float u0 = x[t] - y[t], u1 = x[t + 1] - y[t + 1];
        f0 = u0 * u0 + f0;
        f1 = u1 * u1 + f1;
        t += 2;
    }
    float acc = f0 + f1;
    if (t < d) {
        const float u = x[t] - y[t];
        acc = acc + u * u;
    }
    return acc;
}

// One positive or noise sample of src/ncvis.cpp:304-339.  The source reads
//   Ph = 1/(1 + a d2^b);  w = Ph/(nu e^Q);  w = 1/(1+w) | -1/(1+1/w);
//   Q -= w alpha_Q;  w = 2 w Ph a b d2^(b-1);  dx = clip((y_o - y_i) w step, 4)
// and the reference's -O3 -ffast-math build (g++ 13, x86-64) evaluates it as
// written below: 1/w folded to nu e^Q (1 + a d2^b), the final weight grouped
// as (w d2^(b-1)) ((a b)(Ph + Ph)), and w*step hoisted out of the coordinate
// loop.  Spelling the same grouping here keeps the oracle on the reference's
// bits (checked against oracle/_ref).
inline void nce_sample(float *Y, size_t d, size_t i, size_t o, bool positive, uint64_t nu,
                       float a, float b, float alpha_Q, float step, float &Qc) {
    const float d2 = sq_dist(Y + i * d, Y + o * d, d);
    float w = 1.f;
    if (nu != 0) {
        const float denom = a * powf(d2, b) + 1.f;
        const float ph = 1.f / denom;
        const float ab2ph = (a * b) * (ph + ph);
        const float noise_mass = (float)nu * expf(Qc);
        w = positive ? 1.f / (ph / noise_mass + 1.f) : -1.f / (noise_mass * denom + 1.f);
        Qc = Qc - w * alpha_Q;
        w = (w * powf(d2, b - 1.f)) * ab2ph;
    }
    const float ws = w * step;
    for (size_t q = 0; q < d; ++q) {
        float dx = (Y[o * d + q] - Y[i * d + q]) * ws;
        dx = std::min(std::max(dx, -4.f), 4.f);
        Y[i * d + q] += dx;
        Y[o * d + q] -= dx;
    }
}

}  // namespace

extern "C" {

// The negatives one reference thread draws (src/ncvis.cpp:281-283, 294-302):
// pcg64(seed), for each epoch, edge and noise sample, uniform indices redrawn
// while equal to the edge's source.  Independent of Y.  Writes
// E * sum(n_noise) indices in consumption order; returns that count.
size_t orc_negative_stream(size_t N, size_t E, const int64_t *src, uint64_t seed, int n_epochs,
                           const uint64_t *n_noise, int32_t *out) {
    Pcg64 g(seed);
    size_t pos = 0;
    for (int ep = 0; ep < n_epochs; ++ep)
        for (size_t e = 0; e < E; ++e) {
            const uint64_t i = (uint64_t)src[e];
            for (uint64_t s = 0; s < n_noise[ep]; ++s) {
                uint64_t o;
                do {
                    o = draw_index(g, N - 1);
                } while (o == i);
                out[pos++] = (int32_t)o;
            }
        }
    return pos;
}

// src/ncvis.cpp:275-352, epochs [epoch_begin, epoch_end) of an n_epochs
// schedule.  Y and *Q are updated in place.  With stream == nullptr the
// negatives come from per-thread pcg64(seed + thread) generators as in the
// reference (for epoch_begin > 0 the generators restart, so use the stream
// form for partial runs); otherwise they are read from the one-thread stream
// of orc_negative_stream, starting at that stream's offset for epoch_begin.
void orc_optimize(size_t N, size_t d, size_t E, const int64_t *src, const int64_t *dst, float *Y,
                  float *Q, uint64_t seed, int epoch_begin, int epoch_end, int n_epochs,
                  const uint64_t *n_noise, float a, float b, float alpha, float alpha_Q,
                  int n_threads, const int32_t *stream) {
    if (stream != nullptr) {
        size_t pos = 0;
        for (int ep = 0; ep < epoch_begin; ++ep) pos += E * (size_t)n_noise[ep];
        for (int ep = epoch_begin; ep < epoch_end; ++ep) {
            const float frac = ((float)ep) / n_epochs;
            const float step = alpha * (1 - frac * frac);
            float Qc = *Q;
            const uint64_t nu = n_noise[ep];
            for (size_t e = 0; e < E; ++e) {
                const size_t i = (size_t)src[e];
                nce_sample(Y, d, i, (size_t)dst[e], true, nu, a, b, alpha_Q, step, Qc);
                for (uint64_t s = 0; s < nu; ++s)
                    nce_sample(Y, d, i, (size_t)stream[pos++], false, nu, a, b, alpha_Q, step, Qc);
            }
            *Q = Qc;
        }
        return;
    }
    float q_sum = 0.;
#pragma omp parallel num_threads(n_threads)
    {
        const int nthr = omp_get_num_threads();
        Pcg64 g(seed + (uint64_t)omp_get_thread_num());
        for (int ep = epoch_begin; ep < epoch_end; ++ep) {
            const float frac = ((float)ep) / n_epochs;
            const float step = alpha * (1 - frac * frac);
            float Qc = *Q;
            const uint64_t nu = n_noise[ep];
#pragma omp for schedule(static) nowait
            for (long long e = 0; e < (long long)E; ++e) {
                const size_t i = (size_t)src[e];
                nce_sample(Y, d, i, (size_t)dst[e], true, nu, a, b, alpha_Q, step, Qc);
                for (uint64_t s = 0; s < nu; ++s) {
                    size_t o;
                    do {
                        o = (size_t)draw_index(g, N - 1);
                    } while (o == i);
                    nce_sample(Y, d, i, o, false, nu, a, b, alpha_Q, step, Qc);
                }
            }
#pragma omp atomic
            q_sum += Qc;
#pragma omp barrier
#pragma omp single
            {
                *Q = q_sum / nthr;
                q_sum = 0;
            }
        }
    }
}

// One step of the one-thread optimizer: edges [edge_begin, edge_end) of epoch
// `epoch`, noise indices read from stream[stream_pos...], *Qc the running
// copy of Q at edge_begin (updated in place).  Returns the new stream_pos.
size_t orc_optimize_block(size_t d, const int64_t *src, const int64_t *dst, float *Y, float *Qc,
                          int epoch, int n_epochs, uint64_t nu, size_t edge_begin, size_t edge_end,
                          const int32_t *stream, size_t stream_pos, float a, float b, float alpha,
                          float alpha_Q) {
    const float frac = ((float)epoch) / n_epochs;
    const float step = alpha * (1 - frac * frac);
    float q = *Qc;
    for (size_t e = edge_begin; e < edge_end; ++e) {
        const size_t i = (size_t)src[e];
        nce_sample(Y, d, i, (size_t)dst[e], true, nu, a, b, alpha_Q, step, q);
        for (uint64_t s = 0; s < nu; ++s)
            nce_sample(Y, d, i, (size_t)stream[stream_pos++], false, nu, a, b, alpha_Q, step, q);
    }
    *Qc = q;
    return stream_pos;
}

}  // extern "C"
