// ncvis.hpp — header-only C++ drop-in for the reference's ncvis::NCVis
// (src/ncvis.hpp:25-93) over the C ABI of libncvis_gb300.so
// (include/ncvis_gb300.h).
//
// Same namespace, enum, constructor (with the reference's C++ defaults:
// n_neighbors 30, M 16, ef_construction 200, a = b = 1, 3 noise samples per
// epoch when n_noise is null) and fit_transform signature.  Errors are thrown
// as std::runtime_error carrying the engine's message, which for the
// reference's own checks is the reference's message
// (src/ncvis.cpp:364-369, 90).  Unlike the reference, which sets the
// process-wide OpenMP thread count, n_threads only bounds host-side work.
#ifndef NCVIS_GB300_NCVIS_HPP
#define NCVIS_GB300_NCVIS_HPP

#include <cstddef>
#include <stdexcept>
#include <string>
#include <utility>

#include "ncvis_gb300.h"

namespace ncvis {

typedef std::pair<size_t, size_t> Edge;

enum Distance { squared_L2, inner_product, cosine_similarity, correlation };

class NCVis {
   public:
    NCVis(size_t d = 2, size_t n_threads = 1, size_t n_neighbors = 30, size_t M = 16,
          size_t ef_construction = 200, size_t random_seed = 42, int n_epochs = 50,
          int n_init_epochs = 20, float a = 1., float b = 1., float alpha = 1., float alpha_Q = 1.,
          size_t *n_noise = nullptr, ncvis::Distance dist = ncvis::Distance::squared_L2) {
        ncvis_params p;
        p.d = d;
        p.n_threads = n_threads;
        p.n_neighbors = n_neighbors;
        p.M = M;
        p.ef_construction = ef_construction;
        p.random_seed = random_seed;
        p.n_epochs = n_epochs;
        p.n_init_epochs = n_init_epochs;
        p.a = a;
        p.b = b;
        p.alpha = alpha;
        p.alpha_Q = alpha_Q;
        p.n_noise = n_noise;
        p.distance = (int)dist;
        h_ = ncvis_create(&p, nullptr);
        if (!h_) throw std::runtime_error(ncvis_get_last_error());
    }
    ~NCVis() { ncvis_destroy(h_); }
    NCVis(const NCVis &) = delete;
    NCVis &operator=(const NCVis &) = delete;

    /*!
    @brief Build embedding for points.

    X [N, D] row-major (X + D*i + j), Y [N, d] row-major, written.
    */
    void fit_transform(const float *const X, size_t N, size_t D, float *Y) {
        if (ncvis_fit_transform(h_, X, N, D, Y) != NCVIS_OK)
            throw std::runtime_error(ncvis_last_error(h_));
    }

    // Extensions beyond the reference's interface.
    void set_options(const ncvis_options &o) {
        if (ncvis_set_options(h_, &o) != NCVIS_OK) throw std::runtime_error(ncvis_last_error(h_));
    }
    ncvis_stage_times stage_times() const {
        ncvis_stage_times t;
        ncvis_get_stage_times(h_, &t);
        return t;
    }

   private:
    ncvis_handle h_;
};

}  // namespace ncvis

#endif  // NCVIS_GB300_NCVIS_HPP
