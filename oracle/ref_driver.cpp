// Test-infrastructure driver, not product code.
//
// Exposes the reference's own stages, compiled from the reference sources
// where they lie (src/ncvis.cpp, src/knntable.cpp), as C functions so that the
// oracle restatement in ncvis_oracle.cpp can be pinned against them and golden
// fixtures can be generated.  Built by oracle/build_ref.sh into
// oracle/_ref/libncvis_ref.so; it exists only where the reference checkout is
// present.
//
// The reference keeps buildKNN/findKNN/init_embedding/optimize private
// (src/ncvis.hpp:68-92); they are reached here by compiling the class
// declaration with `private` spelled `public`, which changes neither layout
// nor symbol names, so the member functions in the reference's object code
// are called unmodified.
#include <assert.h>
#include <omp.h>

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <iostream>
#include <ostream>
#include <queue>
#include <random>
#include <stdexcept>
#include <utility>
#include <vector>

#include "../lib/pcg-cpp/include/pcg_random.hpp"

#define private public
#include "ncvis.hpp"
#undef private

namespace {

std::vector<ncvis::Edge> make_edges(size_t E, const int64_t *src, const int64_t *dst) {
    std::vector<ncvis::Edge> edges;
    edges.reserve(E);
    for (size_t e = 0; e < E; ++e) edges.emplace_back((size_t)src[e], (size_t)dst[e]);
    return edges;
}

}  // namespace

extern "C" {

// src/ncvis.cpp:72-153 with the brute-force hnswlib stand-in: rows of k
// neighbours in the order findKNN stores them.  Returns 0 on success.
int ref_knn(const float *X, size_t N, size_t D, int dist, size_t k, int n_threads, int64_t *inds,
            float *dists) {
    try {
        ncvis::NCVis vis(2, (size_t)n_threads, k, 16, 200, 42, 1, 0, 1.f, 1.f, 1.f, 1.f, nullptr,
                         (ncvis::Distance)dist);
        vis.buildKNN(X, N, D);
        ncvis::KNNTable table = vis.findKNN(X, N, D, k);
        for (size_t i = 0; i < N; ++i) {
            if (table.inds[i].size() != k) return 1;
            for (size_t j = 0; j < k; ++j) {
                inds[i * k + j] = table.inds[i][j];
                dists[i * k + j] = table.dists[i][j];
            }
        }
    } catch (...) {
        return 2;
    }
    return 0;
}

// src/knntable.cpp:24-99.  Output is CSR: row_ptr[N+1], out_inds/out_dists
// with capacity 2*N*k.  Returns the number of entries.
size_t ref_symmetrize(size_t N, size_t k, const int64_t *inds, const float *dists, int n_threads,
                      int64_t *row_ptr, int64_t *out_inds, float *out_dists) {
    omp_set_num_threads(n_threads);
    ncvis::KNNTable table((long)N, (long)k);
    for (size_t i = 0; i < N; ++i) {
        for (size_t j = 0; j < k; ++j) {
            table.inds[i].push_back((long)inds[i * k + j]);
            table.dists[i].push_back(dists[i * k + j]);
        }
    }
    table.symmetrize();
    size_t pos = 0;
    row_ptr[0] = 0;
    for (size_t i = 0; i < N; ++i) {
        for (size_t j = 0; j < table.inds[i].size(); ++j) {
            out_inds[pos] = table.inds[i][j];
            out_dists[pos] = table.dists[i][j];
            ++pos;
        }
        row_ptr[i + 1] = (int64_t)pos;
    }
    return pos;
}

// src/ncvis.cpp:155-173 applied to a CSR graph (row-major flatten).
void ref_build_edges(size_t N, const int64_t *row_ptr, const int64_t *cols, int64_t *src,
                     int64_t *dst) {
    ncvis::KNNTable table((long)N, 1);
    for (size_t i = 0; i < N; ++i)
        for (int64_t p = row_ptr[i]; p < row_ptr[i + 1]; ++p) table.inds[i].push_back((long)cols[p]);
    ncvis::NCVis vis;
    std::vector<ncvis::Edge> edges = vis.build_edges(table);
    for (size_t e = 0; e < edges.size(); ++e) {
        src[e] = (int64_t)edges[e].first;
        dst[e] = (int64_t)edges[e].second;
    }
}

// src/ncvis.cpp:184-273.
void ref_init_embedding(size_t N, size_t d, size_t E, const int64_t *src, const int64_t *dst,
                        uint64_t seed, int n_init_epochs, float alpha, int n_threads, float *Y) {
    ncvis::NCVis vis(d, (size_t)n_threads, 15, 16, 200, (size_t)seed, 1, n_init_epochs);
    std::vector<ncvis::Edge> edges = make_edges(E, src, dst);
    vis.init_embedding(N, Y, alpha, edges);
}

// src/ncvis.cpp:275-352.  Y and *Q are updated in place.
void ref_optimize(size_t N, size_t d, size_t E, const int64_t *src, const int64_t *dst,
                  uint64_t seed, int n_epochs, const uint64_t *n_noise, float a, float b, float alpha,
                  float alpha_Q, int n_threads, float *Y, float *Q) {
    std::vector<size_t> plan(n_epochs);
    for (int e = 0; e < n_epochs; ++e) plan[e] = (size_t)n_noise[e];
    ncvis::NCVis vis(d, (size_t)n_threads, 15, 16, 200, (size_t)seed, n_epochs, 20, a, b, alpha,
                     alpha_Q, plan.data());
    std::vector<ncvis::Edge> edges = make_edges(E, src, dst);
    float q = *Q;
    vis.optimize(N, Y, q, edges);
    *Q = q;
}

// src/ncvis.cpp:354-459, the whole pipeline.  Returns 0 on success.
int ref_fit_transform(const float *X, size_t N, size_t D, size_t d, int n_threads,
                      size_t n_neighbors, uint64_t seed, int n_epochs, int n_init_epochs, float a,
                      float b, float alpha, float alpha_Q, const uint64_t *n_noise, int dist,
                      float *Y) {
    try {
        std::vector<size_t> plan(n_epochs);
        for (int e = 0; e < n_epochs; ++e) plan[e] = (size_t)n_noise[e];
        ncvis::NCVis vis(d, (size_t)n_threads, n_neighbors, 16, 200, (size_t)seed, n_epochs,
                         n_init_epochs, a, b, alpha, alpha_Q, plan.data(), (ncvis::Distance)dist);
        vis.fit_transform(X, N, D, Y);
    } catch (...) {
        return 2;
    }
    return 0;
}

// Raw pcg64(seed) outputs and the two libstdc++ distributions the reference
// draws from (src/ncvis.cpp:195-200, 281-283, 300).
void ref_pcg64(uint64_t seed, size_t n, uint64_t *out) {
    pcg64 g((size_t)seed);
    for (size_t t = 0; t < n; ++t) out[t] = g();
}

void ref_uniform_real(uint64_t seed, size_t n, float *out) {
    pcg64 g((size_t)seed);
    std::uniform_real_distribution<float> u(0, 1);
    for (size_t t = 0; t < n; ++t) out[t] = u(g);
}

void ref_uniform_int(uint64_t seed, uint64_t hi, size_t n, uint64_t *out) {
    pcg64 g((size_t)seed);
    std::uniform_int_distribution<size_t> u(0, (size_t)hi);
    for (size_t t = 0; t < n; ++t) out[t] = u(g);
}

}  // extern "C"
