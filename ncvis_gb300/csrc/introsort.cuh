// Sequential introsort whose output permutation equals that of GCC 13
// libstdc++'s std::sort, which the reference calls to order each symmetrized
// row by distance (src/knntable.cpp:81-83: sort of an index array with the
// comparator key[i1] < key[i2]).  std::sort is unstable; rows routinely hold
// equal keys (an edge and its reverse carry the same distance), and the
// reference's deduplication (src/knntable.cpp:85-93) depends on where equal
// keys land, so the CSR is bit-exact only if the tie order is reproduced.
//
// Algorithm (libstdc++'s introsort, restated from its description):
//   * depth budget 2*floor(log2 n); ranges longer than 16 are partitioned:
//     the median of (first+1, middle, last-1) is swapped into first, then an
//     unguarded Hoare partition of [first+1, last) around *first; the right
//     part is sorted before the loop continues on the left part;
//   * a range whose budget is exhausted is heap-sorted (make_heap over the
//     range, then repeated pop_heap; sift-down moves the hole to a leaf
//     along the larger child, then sifts the saved value up);
//   * finally an insertion sort over the first 16 elements and an unguarded
//     linear insertion for every later element.
// Sorted items carry their key, so moving an item equals moving the index
// the reference moves.  The pending-range stack replaces recursion: ranges
// are disjoint, so the order they are visited in does not change the result.
// `V` is anything indexable as SortItem& (a pointer, or a strided view of a
// shared-memory row).
#pragma once

#include <cstdint>

namespace ncvis_gpu {

struct SortItem {
    float key;
    int32_t pos;
};

#ifdef __CUDACC__
#define NCVIS_HD __host__ __device__ __forceinline__
#else
#define NCVIS_HD inline
#endif

namespace introsort_detail {

NCVIS_HD bool less(const SortItem &x, const SortItem &y) { return x.key < y.key; }

NCVIS_HD void swap_items(SortItem &a, SortItem &b) {
    SortItem t = a;
    a = b;
    b = t;
}

NCVIS_HD int floor_log2(int32_t n) {
    int r = 0;
    while (n > 1) {
        n >>= 1;
        ++r;
    }
    return r;
}

// Sift the hole at `hole` down to a leaf through the larger child, then push
// `value` back up no higher than `top`.
template <class V>
NCVIS_HD void sift(V v, int32_t hole, int32_t len, SortItem value) {
    const int32_t top = hole;
    int32_t child = hole;
    while (child < (len - 1) / 2) {
        child = 2 * (child + 1);
        if (less(v[child], v[child - 1])) child--;
        v[hole] = v[child];
        hole = child;
    }
    if ((len & 1) == 0 && child == (len - 2) / 2) {
        child = 2 * (child + 1);
        v[hole] = v[child - 1];
        hole = child - 1;
    }
    int32_t parent = (hole - 1) / 2;
    while (hole > top && less(v[parent], value)) {
        v[hole] = v[parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    v[hole] = value;
}

template <class V>
NCVIS_HD void heap_sort(V v, int32_t len) {
    if (len >= 2) {
        for (int32_t parent = (len - 2) / 2;; --parent) {
            sift(v, parent, len, v[parent]);
            if (parent == 0) break;
        }
    }
    for (int32_t last = len; last > 1;) {
        --last;
        SortItem value = v[last];
        v[last] = v[0];
        sift(v, 0, last, value);
    }
}

// Median of v[a], v[b], v[c] swapped into v[dst].
template <class V>
NCVIS_HD void median_to(V v, int32_t dst, int32_t a, int32_t b, int32_t c) {
    if (less(v[a], v[b])) {
        if (less(v[b], v[c]))
            swap_items(v[dst], v[b]);
        else if (less(v[a], v[c]))
            swap_items(v[dst], v[c]);
        else
            swap_items(v[dst], v[a]);
    } else if (less(v[a], v[c])) {
        swap_items(v[dst], v[a]);
    } else if (less(v[b], v[c])) {
        swap_items(v[dst], v[c]);
    } else {
        swap_items(v[dst], v[b]);
    }
}

// Hoare partition of [lo+1, hi) around the pivot held at v[lo]; returns the cut.
template <class V>
NCVIS_HD int32_t partition(V v, int32_t lo, int32_t hi) {
    int32_t mid = lo + (hi - lo) / 2;
    median_to(v, lo, lo + 1, mid, hi - 1);
    const float pivot = v[lo].key;  // the pivot item stays at v[lo]
    int32_t f = lo + 1, l = hi;
    for (;;) {
        while (v[f].key < pivot) ++f;
        --l;
        while (pivot < v[l].key) --l;
        if (!(f < l)) return f;
        swap_items(v[f], v[l]);
        ++f;
    }
}

template <class V>
NCVIS_HD void linear_insert(V v, int32_t at) {
    SortItem value = v[at];
    int32_t prev = at - 1;
    while (less(value, v[prev])) {
        v[at] = v[prev];
        at = prev;
        --prev;
    }
    v[at] = value;
}

template <class V>
NCVIS_HD void insertion_sort(V v, int32_t lo, int32_t hi) {
    if (lo == hi) return;
    for (int32_t i = lo + 1; i != hi; ++i) {
        if (less(v[i], v[lo])) {
            SortItem value = v[i];
            for (int32_t t = i; t > lo; --t) v[t] = v[t - 1];
            v[lo] = value;
        } else {
            linear_insert(v, i);
        }
    }
}

// v shifted by `base` positions (the heap-sort fallback works on a sub-range).
template <class V>
struct Offset {
    V v;
    int32_t base;
    NCVIS_HD SortItem &operator[](int32_t i) const { return v[base + i]; }
};

}  // namespace introsort_detail

// Row `lane` of a [n][stride] shared-memory block, element i at i * stride.
struct StridedItems {
    SortItem *base;
    int32_t stride;
    NCVIS_HD SortItem &operator[](int32_t i) const { return base[i * stride]; }
};

// Sorts v[0, n) in place, n < 2^31.  The pending-range stack holds at most
// 2*floor(log2 n) + 1 <= 61 entries (one per partition level of the budget).
template <class V>
NCVIS_HD void libstdcxx_sort(V v, int32_t n) {
    using namespace introsort_detail;
    const int32_t kThreshold = 16;
    if (n <= 1) return;
    struct Range {
        int32_t lo, hi;
        int depth;
    };
    Range stack[64];
    int top = 0;
    stack[top++] = Range{0, n, 2 * floor_log2(n)};
    while (top > 0) {
        Range r = stack[--top];
        while (r.hi - r.lo > kThreshold) {
            if (r.depth == 0) {
                heap_sort(Offset<V>{v, r.lo}, r.hi - r.lo);
                break;
            }
            --r.depth;
            int32_t cut = partition(v, r.lo, r.hi);
            stack[top++] = Range{cut, r.hi, r.depth};
            r.hi = cut;
        }
    }
    if (n > kThreshold) {
        insertion_sort(v, 0, kThreshold);
        for (int32_t i = kThreshold; i < n; ++i) linear_insert(v, i);
    } else {
        insertion_sort(v, 0, n);
    }
}

}  // namespace ncvis_gpu
