// One row of the symmetrization, staged in fast memory (shared memory on the
// GPU; any indexable storage on the host): the steps of the reference's
// KNNTable::symmetrize for row i (src/knntable.cpp:60-96) on the row's own k
// table entries and its incoming entries.
//
// Inputs: ink[0, L - k) the row's incoming entry ids e = s*k + j (any order,
// distinct); own_i / own_d the row's k table entries; dists the whole table's
// distances (the incoming entry e carries dists[e]).  items and orig provide
// L slots each.  Global loads are issued four at a time, so a row waits for
// about a quarter of its entries' round trips.
// Steps:
//   * the incoming ids are sorted ascending, which is the order one thread
//     appends them in (src/knntable.cpp:40-49);
//   * orig[p] becomes the index stored at row position p, items[p] the pair
//     (distance at p, p);
//   * libstdcxx_sort orders the items as std::sort orders the reference's
//     index array (src/knntable.cpp:81-83);
//   * deduplication (src/knntable.cpp:85-93): sorted item j is kept unless
//     the row's index at its position equals the row's index at the position
//     of sorted item j-1, both read from the row while it is being overwritten
//     with the kept entries.  Kept items are compacted in place, so position
//     p < n_out of the row holds orig[items[p].pos] and position p >= n_out
//     still holds orig[p];
//   * the kept entries go to out_col / out_val in order.
// Returns the number of kept entries.
#pragma once

#include <cstdint>

#include "introsort.cuh"

namespace ncvis_gpu {

// Row `lane` of a [n][stride] block of 32-bit integers.
struct StridedInts {
    int32_t *base;
    int32_t stride;
    NCVIS_HD int32_t &operator[](int32_t i) const { return base[i * stride]; }
};

// Ascending sort of a[off, off + n), n distinct integers (any correct sort
// gives the one result): insertion sort for short runs, heap sort otherwise.
template <class V>
NCVIS_HD void sort_distinct_ints(V a, int32_t off, int32_t n) {
    if (n <= 32) {
        for (int32_t i = 1; i < n; ++i) {
            const int32_t v = a[off + i];
            int32_t j = i - 1;
            while (j >= 0 && a[off + j] > v) {
                a[off + j + 1] = a[off + j];
                --j;
            }
            a[off + j + 1] = v;
        }
        return;
    }
    auto down = [&](int32_t root, int32_t end) {
        const int32_t v = a[off + root];
        for (;;) {
            int32_t child = 2 * root + 1;
            if (child >= end) break;
            if (child + 1 < end && a[off + child] < a[off + child + 1]) ++child;
            if (v >= a[off + child]) break;
            a[off + root] = a[off + child];
            root = child;
        }
        a[off + root] = v;
    };
    for (int32_t start = n / 2 - 1; start >= 0; --start) down(start, n);
    for (int32_t end = n - 1; end > 0; --end) {
        const int32_t t = a[off];
        a[off] = a[off + end];
        a[off + end] = t;
        down(0, end);
    }
}

// The sort and the deduplication of a built row (items[p] = (distance at p,
// p), orig[p] = index at p): afterwards items[0, n_out) are the kept items in
// order, their indices orig[items[q].pos].  Returns n_out.
template <class VI, class VO>
NCVIS_HD int32_t sort_and_dedup(VI items, VO orig, int32_t L) {
    libstdcxx_sort(items, L);
    int32_t n_out = 0;
    for (int32_t j = 0; j < L; ++j) {
        const SortItem cur = items[j];
        bool keep = j == 0;
        if (!keep) {
            const int32_t p = cur.pos, q = items[j - 1].pos;
            const int32_t vp = orig[p < n_out ? items[p].pos : p];
            const int32_t vq = orig[q < n_out ? items[q].pos : q];
            keep = vp != vq;
        }
        if (keep) items[n_out++] = cur;
    }
    return n_out;
}

template <class VI, class VO>
NCVIS_HD int32_t merge_row(VI items, VO orig, int32_t L, int32_t k,
                           const int32_t *__restrict__ own_i, const float *__restrict__ own_d,
                           const int32_t *__restrict__ ink, const float *__restrict__ dists,
                           int32_t *__restrict__ out_col, float *__restrict__ out_val) {
    int32_t p = k;
    for (; p + 4 <= L; p += 4) {
        int32_t e[4];
        for (int u = 0; u < 4; ++u) e[u] = ink[p - k + u];
        for (int u = 0; u < 4; ++u) orig[p + u] = e[u];
    }
    for (; p < L; ++p) orig[p] = ink[p - k];
    sort_distinct_ints(orig, k, L - k);
    for (p = 0; p + 4 <= k; p += 4) {
        int32_t c[4];
        float d[4];
        for (int u = 0; u < 4; ++u) c[u] = own_i[p + u], d[u] = own_d[p + u];
        for (int u = 0; u < 4; ++u) items[p + u] = SortItem{d[u], p + u}, orig[p + u] = c[u];
    }
    for (; p < k; ++p) items[p] = SortItem{own_d[p], p}, orig[p] = own_i[p];
    for (; p + 4 <= L; p += 4) {
        int32_t e[4];
        float d[4];
        for (int u = 0; u < 4; ++u) e[u] = orig[p + u];
        for (int u = 0; u < 4; ++u) d[u] = dists[e[u]];
        for (int u = 0; u < 4; ++u) items[p + u] = SortItem{d[u], p + u}, orig[p + u] = e[u] / k;
    }
    for (; p < L; ++p) {
        const int32_t e = orig[p];
        items[p] = SortItem{dists[e], p};
        orig[p] = e / k;
    }
    const int32_t n_out = sort_and_dedup(items, orig, L);
    for (int32_t q = 0; q < n_out; ++q) {
        const SortItem it = items[q];
        out_col[q] = orig[it.pos];
        out_val[q] = it.key;
    }
    return n_out;
}

}  // namespace ncvis_gpu
