// ORACLE — test infrastructure, not product code.
//
// A CPU restatement of the reference NCVis hot path (stat-ml/ncvis), used only
// by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg to check
// and time the CUDA engine.  Nothing in ncvis_gb300/ links or calls it.
//
// Each function names the reference lines it restates.  Floating-point
// operations are written in the reference's order so that, compiled with the
// reference's flags (-O3 -ffast-math), results agree with the reference to the
// last bits on the same machine and compiler; the tests check this against
// oracle/_ref (the reference's own code) and the golden fixtures.
//
// The random streams come from oracle_rng.h; the SGD (src/ncvis.cpp:275-352)
// lives in ncvis_oracle_sgd.cpp, compiled with strict IEEE arithmetic.
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <utility>
#include <vector>

#include "oracle_rng.h"

using namespace orc;

namespace {

// src/ncvis.cpp:32-70.
void preprocess_row(const float *x, size_t D, int dist, float *out) {
    if (dist == CORRELATION) {
        float mean = 0;
        for (size_t t = 0; t < D; ++t) mean += x[t];
        mean /= D;
        for (size_t t = 0; t < D; ++t) out[t] = x[t] - mean;
    } else {
        for (size_t t = 0; t < D; ++t) out[t] = x[t];
    }
    if (dist == CORRELATION || dist == COSINE) {
        float sq = 0;
        for (size_t t = 0; t < D; ++t) sq += out[t] * out[t];
        if (sq != 0)
            for (size_t t = 0; t < D; ++t) out[t] /= sqrtf(sq);
    }
}

// hnswlib spaces selected at src/ncvis.cpp:78-92: squared L2, or 1 - <x,y>.
float pair_distance_f32(const float *x, const float *y, size_t D, int dist) {
    if (dist == SQUARED_L2) {
        float acc = 0.f;
        for (size_t t = 0; t < D; ++t) {
            float diff = x[t] - y[t];
            acc += diff * diff;
        }
        return acc;
    }
    float dot = 0.f;
    for (size_t t = 0; t < D; ++t) dot += x[t] * y[t];
    return 1.f - dot;
}

double pair_distance_f64(const float *x, const float *y, size_t D, int dist) {
    if (dist == SQUARED_L2) {
        double acc = 0.0;
        for (size_t t = 0; t < D; ++t) {
            double diff = (double)x[t] - (double)y[t];
            acc += diff * diff;
        }
        return acc;
    }
    double dot = 0.0;
    for (size_t t = 0; t < D; ++t) dot += (double)x[t] * (double)y[t];
    return 1.0 - dot;
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------- RNG streams

void orc_pcg64(uint64_t seed, size_t n, uint64_t *out) {
    Pcg64 g(seed);
    for (size_t t = 0; t < n; ++t) out[t] = g();
}

void orc_uniform_real(uint64_t seed, size_t n, float *out) {
    Pcg64 g(seed);
    for (size_t t = 0; t < n; ++t) out[t] = draw_unit(g);
}

void orc_uniform_int(uint64_t seed, uint64_t hi, size_t n, uint64_t *out) {
    Pcg64 g(seed);
    for (size_t t = 0; t < n; ++t) out[t] = draw_index(g, hi);
}

// ------------------------------------------------------------ preprocess + kNN

void orc_preprocess(const float *X, size_t N, size_t D, int dist, float *out) {
    for (size_t i = 0; i < N; ++i) preprocess_row(X + i * D, D, dist, out + i * D);
}

// Exact kNN with the reference's table contract (src/ncvis.cpp:128-153): take
// the k+1 smallest (distance, index) pairs over all points, drop the
// smallest, store the remaining k in descending order.  Xp is already
// preprocessed.  use_f64 selects FP64 distances (the recall oracle) over the
// FP32 loop the hnswlib spaces use.
void orc_knn(const float *Xp, size_t N, size_t D, int dist, size_t k, int use_f64, int n_threads,
             int64_t *inds, float *dists) {
    const size_t kk = k + 1 < N ? k + 1 : N;
#pragma omp parallel num_threads(n_threads)
    {
        std::vector<std::pair<double, int64_t> > cand(N);
#pragma omp for schedule(dynamic, 16)
        for (long long i = 0; i < (long long)N; ++i) {
            const float *q = Xp + (size_t)i * D;
            for (size_t j = 0; j < N; ++j) {
                double dv = use_f64 ? pair_distance_f64(q, Xp + j * D, D, dist)
                                    : (double)pair_distance_f32(q, Xp + j * D, D, dist);
                cand[j] = std::make_pair(dv, (int64_t)j);
            }
            std::partial_sort(cand.begin(), cand.begin() + kk, cand.end());
            // cand[0..kk) ascending; keep ranks 1..kk-1 in descending order.
            for (size_t r = 0; r + 1 < kk; ++r) {
                const std::pair<double, int64_t> &p = cand[kk - 1 - r];
                inds[(size_t)i * k + r] = p.second;
                dists[(size_t)i * k + r] = (float)p.first;
            }
        }
    }
}

// ------------------------------------------------------------------ symmetrize

// src/knntable.cpp:24-99 with one thread: each row is its k table entries
// followed by the incoming entries in increasing source order, arg-sorted by
// distance with std::sort (introsort, unstable), then deduplicated by a loop
// whose comparisons read the row while it overwrites it in place.  The
// per-row phase is independent across rows, so it runs on n_threads threads
// with the one-thread result.  Output: row_ptr[N+1] and entries (capacity
// 2*N*k).  Returns the entry count.
size_t orc_symmetrize(size_t N, size_t k, const int64_t *inds, const float *dists, int n_threads,
                      int64_t *row_ptr, int64_t *out_inds, float *out_dists) {
    // Incoming entries, bucketed by target in (source, slot) order.
    std::vector<int64_t> in_count(N + 1, 0);
    for (size_t e = 0; e < N * k; ++e) in_count[(size_t)inds[e] + 1]++;
    for (size_t i = 0; i < N; ++i) in_count[i + 1] += in_count[i];
    std::vector<int64_t> in_src(N * k);
    std::vector<float> in_dist(N * k);
    {
        std::vector<int64_t> cursor(in_count.begin(), in_count.end() - 1);
        for (size_t s = 0; s < N; ++s)
            for (size_t j = 0; j < k; ++j) {
                const size_t t = (size_t)inds[s * k + j];
                in_src[cursor[t]] = (int64_t)s;
                in_dist[cursor[t]] = dists[s * k + j];
                cursor[t]++;
            }
    }
    // Per-row merge into a row-aligned scratch layout: row i starts at i*k +
    // in_count[i] and holds k + indegree(i) slots.
    std::vector<int64_t> kept(N, 0);
    std::vector<int64_t> scratch_inds(2 * N * k);
    std::vector<float> scratch_dists(2 * N * k);
#pragma omp parallel num_threads(n_threads)
    {
        std::vector<int64_t> row;
        std::vector<float> key;
        std::vector<int64_t> order;
#pragma omp for schedule(dynamic, 256)
        for (long long ii = 0; ii < (long long)N; ++ii) {
            const size_t i = (size_t)ii;
            const size_t nin = (size_t)(in_count[i + 1] - in_count[i]);
            const size_t len = k + nin;
            row.assign(inds + i * k, inds + i * k + k);
            key.assign(dists + i * k, dists + i * k + k);
            row.insert(row.end(), in_src.begin() + in_count[i], in_src.begin() + in_count[i + 1]);
            key.insert(key.end(), in_dist.begin() + in_count[i], in_dist.begin() + in_count[i + 1]);
            order.resize(len);
            std::iota(order.begin(), order.end(), (int64_t)0);
            std::sort(order.begin(), order.end(),
                      [&key](int64_t p, int64_t q) { return key[p] < key[q]; });
            // `live` is the row the reference compares against while it is
            // being overwritten; `row`/`key` are its untouched copies.
            int64_t *live = &scratch_inds[i * k + (size_t)in_count[i]];
            float *live_d = &scratch_dists[i * k + (size_t)in_count[i]];
            std::copy(row.begin(), row.end(), live);
            size_t n_out = 0;
            for (size_t j = 0; j < len; ++j) {
                if (j == 0 || live[order[j]] != live[order[j - 1]]) {
                    live[n_out] = row[order[j]];
                    live_d[n_out] = key[order[j]];
                    ++n_out;
                }
            }
            kept[i] = (int64_t)n_out;
        }
    }
    size_t pos = 0;
    row_ptr[0] = 0;
    for (size_t i = 0; i < N; ++i) {
        const size_t base = i * k + (size_t)in_count[i];
        for (int64_t j = 0; j < kept[i]; ++j) {
            out_inds[pos] = scratch_inds[base + j];
            out_dists[pos] = scratch_dists[base + j];
            ++pos;
        }
        row_ptr[i + 1] = (int64_t)pos;
    }
    return pos;
}

// ----------------------------------------------------------------------- init

// src/ncvis.cpp:184-273.  Edges are (src[e], dst[e]) in build_edges order
// (src/ncvis.cpp:155-173: the CSR rows flattened).  n_threads > 1 follows the
// reference's parallel form (per-thread pcg64(seed + thread), static split);
// n_threads == 1 is the deterministic form the GPU reproduces.  stats64 != 0
// (one thread only) is the checker of the engine's default statistics: the
// same sums accumulated in double and rounded once (mean = (float)sum / N,
// sigma = sqrtf((float)sum / N)), where the reference sums in float.
void orc_init_embedding_stats(size_t N, size_t d, size_t E, const int64_t *src,
                              const int64_t *dst, uint64_t seed, int n_init_epochs, float alpha,
                              int n_threads, int stats64, float *Y);

void orc_init_embedding(size_t N, size_t d, size_t E, const int64_t *src, const int64_t *dst,
                        uint64_t seed, int n_init_epochs, float alpha, int n_threads, float *Y) {
    orc_init_embedding_stats(N, d, E, src, dst, seed, n_init_epochs, alpha, n_threads, 0, Y);
}

void orc_init_embedding_stats(size_t N, size_t d, size_t E, const int64_t *src,
                              const int64_t *dst, uint64_t seed, int n_init_epochs, float alpha,
                              int n_threads, int stats64, float *Y) {
    if (stats64) n_threads = 1;
    std::vector<double> acc(d);
    std::vector<float> other(N * d);
    float *bufs[2] = {Y, other.data()};
    std::vector<float> mean(d), sigma(d);
    const long long nd = (long long)(N * d);
#pragma omp parallel num_threads(n_threads)
    {
        Pcg64 g(seed + (uint64_t)omp_get_thread_num());
#pragma omp for schedule(static)
        for (long long t = 0; t < nd; ++t) Y[t] = draw_unit(g);
        for (int ep = 0; ep < n_init_epochs; ++ep) {
            const float *src_y = bufs[ep % 2];
            float *dst_y = bufs[(ep + 1) % 2];
#pragma omp for schedule(static)
            for (long long t = 0; t < nd; ++t) dst_y[t] = 0;
#pragma omp for schedule(static)
            for (long long e = 0; e < (long long)E; ++e) {
                const size_t r = (size_t)src[e], c = (size_t)dst[e];
                for (size_t q = 0; q < d; ++q) dst_y[r * d + q] += alpha * src_y[c * d + q];
            }
#pragma omp single
            for (size_t q = 0; q < d; ++q) mean[q] = sigma[q] = 0;
            if (stats64) {
#pragma omp single
                {
                    for (size_t q = 0; q < d; ++q) acc[q] = 0;
                    for (size_t i = 0; i < N; ++i)
                        for (size_t q = 0; q < d; ++q) acc[q] += (double)dst_y[i * d + q];
                    for (size_t q = 0; q < d; ++q) mean[q] = (float)acc[q] / (float)N;
                    for (size_t q = 0; q < d; ++q) acc[q] = 0;
                    for (size_t i = 0; i < N; ++i)
                        for (size_t q = 0; q < d; ++q) {
                            float dev = dst_y[i * d + q] - mean[q];
                            dev *= dev;
                            acc[q] += (double)dev;
                        }
                    for (size_t q = 0; q < d; ++q) sigma[q] = sqrtf((float)acc[q] / (float)N);
                }
            } else {
#pragma omp for schedule(static)
                for (long long i = 0; i < (long long)N; ++i)
                    for (size_t q = 0; q < d; ++q) {
#pragma omp atomic
                        mean[q] += dst_y[i * d + q];
                    }
#pragma omp single
                for (size_t q = 0; q < d; ++q) mean[q] /= N;
#pragma omp for schedule(static)
                for (long long i = 0; i < (long long)N; ++i)
                    for (size_t q = 0; q < d; ++q) {
                        float dev = dst_y[i * d + q] - mean[q];
                        dev *= dev;
#pragma omp atomic
                        sigma[q] += dev;
                    }
#pragma omp single
                for (size_t q = 0; q < d; ++q) {
                    sigma[q] /= N;
                    sigma[q] = sqrtf(sigma[q]);
                }
            }
#pragma omp for schedule(static)
            for (long long i = 0; i < (long long)N; ++i)
                for (size_t q = 0; q < d; ++q)
                    dst_y[i * d + q] = (dst_y[i * d + q] - mean[q]) / sigma[q];
        }
        if (n_init_epochs % 2) {
#pragma omp for schedule(static)
            for (long long t = 0; t < nd; ++t) bufs[0][t] = bufs[1][t];
        }
    }
}

// ------------------------------------------------------------------- pipeline

void orc_optimize(size_t N, size_t d, size_t E, const int64_t *src, const int64_t *dst, float *Y,
                  float *Q, uint64_t seed, int epoch_begin, int epoch_end, int n_epochs,
                  const uint64_t *n_noise, float a, float b, float alpha, float alpha_Q,
                  int n_threads, const int32_t *stream);

// src/ncvis.cpp:354-459 with exact FP32 kNN in place of HNSW.  Returns 0 on
// success, 1 for the argument errors the reference throws on.
int orc_fit_transform(const float *X, size_t N, size_t D, size_t d, int n_threads,
                      size_t n_neighbors, uint64_t seed, int n_epochs, int n_init_epochs, float a,
                      float b, float alpha, float alpha_Q, const uint64_t *n_noise, int dist,
                      float *Y) {
    if (N == 0 || D == 0 || Y == nullptr) return 1;
    std::vector<float> Xp(N * D);
    orc_preprocess(X, N, D, dist, Xp.data());
    size_t k = (n_neighbors < N - 1) ? n_neighbors : (N - 1);
    k = (k > 0) ? k : 1;
    if (k + 1 > N) return 1;  // the reference leaves rows empty here (undefined later)
    std::vector<int64_t> inds(N * k);
    std::vector<float> dists(N * k);
    orc_knn(Xp.data(), N, D, dist, k, 0, n_threads, inds.data(), dists.data());
    std::vector<int64_t> row_ptr(N + 1), cols(2 * N * k);
    std::vector<float> cd(2 * N * k);
    const size_t E = orc_symmetrize(N, k, inds.data(), dists.data(), n_threads, row_ptr.data(),
                                    cols.data(), cd.data());
    std::vector<int64_t> src(E);
    for (size_t i = 0; i < N; ++i)
        for (int64_t p = row_ptr[i]; p < row_ptr[i + 1]; ++p) src[p] = (int64_t)i;
    const float init_alpha = 1. / k;
    orc_init_embedding(N, d, E, src.data(), cols.data(), seed, n_init_epochs, init_alpha, n_threads,
                       Y);
    float Q = 0.;
    orc_optimize(N, d, E, src.data(), cols.data(), Y, &Q, seed, 0, n_epochs, n_epochs, n_noise, a,
                 b, alpha, alpha_Q, n_threads, nullptr);
    return 0;
}

}  // extern "C"
