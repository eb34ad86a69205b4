// Test-infrastructure shim, not product code.
//
// A brute-force stand-in with the interface that the reference's engine
// expects from nmslib/hnswlib (submodule lib/hnswlib is empty in the
// reference checkout, pinned commit unknown).  It lets oracle/_ref compile the
// reference's own src/ncvis.cpp and src/knntable.cpp unmodified.  The calls it
// has to satisfy are at src/ncvis.cpp:81,87,93,98,122,138 and the forward
// declarations at src/ncvis.hpp:17-23.
//
// Semantics: searchKnn returns a max-heap holding the k smallest
// (distance, label) pairs over every point added so far, exactly what an exact
// HNSW search would return.  L2Space is the squared Euclidean distance and
// InnerProductSpace is 1 - <x, y>, the two spaces hnswlib defines.
#ifndef ORACLE_SHIM_HNSWLIB_H
#define ORACLE_SHIM_HNSWLIB_H

#include <cstddef>
#include <cstring>
#include <queue>
#include <utility>
#include <vector>

namespace hnswlib {

typedef size_t labeltype;

template <typename T>
class SpaceInterface {
   public:
    explicit SpaceInterface(size_t dim) : dim_(dim) {}
    virtual ~SpaceInterface() {}
    size_t dim() const { return dim_; }
    virtual T distance(const T *x, const T *y) const = 0;

   protected:
    size_t dim_;
};

class L2Space : public SpaceInterface<float> {
   public:
    explicit L2Space(size_t dim) : SpaceInterface<float>(dim) {}
    float distance(const float *x, const float *y) const override {
        float acc = 0.f;
        for (size_t t = 0; t < dim_; ++t) {
            float diff = x[t] - y[t];
            acc += diff * diff;
        }
        return acc;
    }
};

class InnerProductSpace : public SpaceInterface<float> {
   public:
    explicit InnerProductSpace(size_t dim) : SpaceInterface<float>(dim) {}
    float distance(const float *x, const float *y) const override {
        float dot = 0.f;
        for (size_t t = 0; t < dim_; ++t) dot += x[t] * y[t];
        return 1.f - dot;
    }
};

template <typename T>
class HierarchicalNSW {
   public:
    HierarchicalNSW(SpaceInterface<T> *space, size_t max_elements, size_t /*M*/ = 16,
                    size_t /*ef_construction*/ = 200, size_t /*random_seed*/ = 100)
        : space_(space),
          dim_(space->dim()),
          capacity_(max_elements),
          data_(max_elements * space->dim()),
          present_(max_elements, 0) {}

    // Thread-safe for distinct labels: every label owns its own slot.
    void addPoint(const void *point, labeltype label) {
        if (label >= capacity_) return;
        std::memcpy(&data_[label * dim_], point, dim_ * sizeof(T));
        present_[label] = 1;
    }

    std::priority_queue<std::pair<T, labeltype> > searchKnn(const void *query, size_t k) const {
        std::priority_queue<std::pair<T, labeltype> > heap;
        const T *q = static_cast<const T *>(query);
        for (labeltype id = 0; id < capacity_; ++id) {
            if (!present_[id]) continue;
            std::pair<T, labeltype> cand(space_->distance(q, &data_[id * dim_]), id);
            if (heap.size() < k) {
                heap.push(cand);
            } else if (k > 0 && cand < heap.top()) {
                heap.pop();
                heap.push(cand);
            }
        }
        return heap;
    }

   private:
    SpaceInterface<T> *space_;
    size_t dim_;
    size_t capacity_;
    std::vector<T> data_;
    std::vector<char> present_;
};

}  // namespace hnswlib

#endif
