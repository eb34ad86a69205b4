// Test harness (CPU only): the data-parallel restatement of the row sort and
// deduplication that the GPU's warp-per-row merge uses, checked against
// libstdc++'s std::sort with the reference's comparator (src/knntable.cpp:
// 81-83) and against the sequential merge (merge_row.cuh), on random,
// tie-heavy and adversarial rows.  The restatement:
//   * each Hoare partition of std::sort's introsort is computed from two
//     position lists: G, the positions (after the pivot) whose key is not
//     below the pivot, ascending, and S, the positions whose key is not above
//     it, descending, the pivot's own position last.  The t-th swap exchanges
//     G[t] and S[t] for every t with G[t] < S[t]; with t* such swaps the cut
//     is min(G[t*], S[t*-1]) (S[-1] = the range's end);
//   * ranges left at 16 items or fewer, and ranges heap-sorted when the depth
//     budget runs out, are leaves; the final insertion sort is stable, so the
//     result is each leaf stably sorted by key in place;
//   * the deduplication's keep flags are the fixpoint of one data-parallel
//     step (keep j from the kept items of the previous guess), which reaches
//     the sequential answer after at most L steps.
// Prints "ok <rows>" or the first mismatch; exit code 0 on success.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <numeric>
#include <random>
#include <vector>

#include "merge_row.cuh"

using ncvis_gpu::SortItem;

namespace {

struct Range {
    int32_t lo, hi, depth;
};

// One partition of items[lo, hi) (hi - lo > 16), as the warp computes it.
int32_t partition_by_lists(std::vector<SortItem> &v, int32_t lo, int32_t hi) {
    ncvis_gpu::introsort_detail::median_to(v.data(), lo, lo + 1, lo + (hi - lo) / 2, hi - 1);
    const float P = v[lo].key;
    std::vector<int32_t> G, S;
    for (int32_t p = lo + 1; p < hi; ++p)
        if (!(v[p].key < P)) G.push_back(p);
    for (int32_t p = hi - 1; p >= lo + 1; --p)
        if (!(P < v[p].key)) S.push_back(p);
    S.push_back(lo);
    int32_t ts = 0;
    const int32_t m = (int32_t)std::min(G.size(), S.size());
    while (ts < m && G[ts] < S[ts]) ++ts;
    for (int32_t t = 0; t < ts; ++t) std::swap(v[G[t]], v[S[t]]);
    int32_t cut = ts > 0 ? S[ts - 1] : hi;
    if (ts < (int32_t)G.size()) cut = std::min(cut, G[ts]);
    return cut;
}

void sort_by_partitions(std::vector<SortItem> &v) {
    const int32_t n = (int32_t)v.size();
    std::vector<int32_t> blk_lo(n), blk_hi(n);
    auto leaf = [&](int32_t lo, int32_t hi) {
        for (int32_t x = lo; x < hi; ++x) blk_lo[x] = lo, blk_hi[x] = hi;
    };
    if (n > 1) {
        std::vector<Range> stack{{0, n, 2 * ncvis_gpu::introsort_detail::floor_log2(n)}};
        while (!stack.empty()) {
            Range r = stack.back();
            stack.pop_back();
            bool heaped = false;
            while (r.hi - r.lo > 16) {
                if (r.depth == 0) {
                    ncvis_gpu::introsort_detail::heap_sort(
                        ncvis_gpu::introsort_detail::Offset<SortItem *>{v.data(), r.lo},
                        r.hi - r.lo);
                    heaped = true;
                    break;
                }
                --r.depth;
                const int32_t cut = partition_by_lists(v, r.lo, r.hi);
                stack.push_back({cut, r.hi, r.depth});
                r.hi = cut;
            }
            (void)heaped;
            leaf(r.lo, r.hi);
        }
    } else {
        leaf(0, n);
    }
    // Each leaf stably sorted by key in place.
    std::vector<SortItem> out(n);
    for (int32_t x = 0; x < n; ++x) {
        int32_t rank = 0;
        for (int32_t y = blk_lo[x]; y < blk_hi[x]; ++y)
            rank += (v[y].key < v[x].key) || (v[y].key == v[x].key && y < x);
        out[blk_lo[x] + rank] = v[x];
    }
    v = out;
}

// Keep flags of the in-place deduplication as a fixpoint; returns the kept
// item indices in order.
std::vector<int32_t> dedup_by_fixpoint(const std::vector<SortItem> &v,
                                       const std::vector<int32_t> &orig, int *steps) {
    const int32_t n = (int32_t)v.size();
    std::vector<char> keep(n, 1), next(n);
    for (*steps = 1;; ++*steps) {
        std::vector<int32_t> kl, nj(n);
        for (int32_t j = 0; j < n; ++j) {
            nj[j] = (int32_t)kl.size();
            if (keep[j]) kl.push_back(j);
        }
        for (int32_t j = 0; j < n; ++j) {
            if (j == 0) {
                next[j] = 1;
                continue;
            }
            auto live = [&](int32_t p) { return orig[p < nj[j] ? v[kl[p]].pos : p]; };
            next[j] = live(v[j].pos) != live(v[j - 1].pos);
        }
        if (next == keep) return kl;
        keep = next;
        if (*steps > n + 1) return {};
    }
}

}  // namespace

int main(int argc, char **argv) {
    const int rows = argc > 1 ? std::atoi(argv[1]) : 20000;
    std::mt19937_64 rng(77);
    int done = 0, max_steps = 0;
    long total_steps = 0;
    for (int r = 0; r < rows; ++r) {
        const int32_t n = 1 + (int32_t)(rng() % (r % 5 == 0 ? 400 : 128));
        const int32_t n_key = 1 + (int32_t)(rng() % (r % 3 == 0 ? 3 : (r % 3 == 1 ? 40 : 100000)));
        const int32_t n_idx = 1 + (int32_t)(rng() % (r % 2 == 0 ? 8 : 300));
        std::vector<float> key(n);
        std::vector<int32_t> orig(n);
        const int pattern = (int)(rng() % 5);
        for (int32_t i = 0; i < n; ++i) {
            switch (pattern) {
                case 0: key[i] = (float)(rng() % n_key); break;
                case 1: key[i] = (float)std::min(i, n - 1 - i); break;            // organ pipe
                case 2: key[i] = (float)((i % 2 == 0) ? i / 2 : n / 2 + i / 2); break;
                case 3: key[i] = (float)(n - i) * 0.5f; break;
                default: key[i] = (float)((i * 7919) % (1 + n_key)) * 0.25f;
            }
            orig[i] = (int32_t)(rng() % n_idx);
        }
        // Reference: std::sort of positions, then the in-place deduplication.
        std::vector<long> idx(n);
        std::iota(idx.begin(), idx.end(), 0L);
        std::sort(idx.begin(), idx.end(), [&key](long a, long b) { return key[a] < key[b]; });
        std::vector<SortItem> v(n);
        for (int32_t i = 0; i < n; ++i) v[i] = SortItem{key[i], i};
        sort_by_partitions(v);
        for (int32_t i = 0; i < n; ++i)
            if (v[i].pos != idx[i]) {
                std::printf("sort mismatch row %d n=%d at %d: %d vs %ld\n", r, n, i, v[i].pos,
                            idx[i]);
                return 1;
            }
        std::vector<SortItem> seq(n);
        for (int32_t i = 0; i < n; ++i) seq[i] = SortItem{key[i], i};
        std::vector<int32_t> orig_seq(orig);
        const int32_t n_seq = ncvis_gpu::sort_and_dedup(seq.data(), orig_seq.data(), n);
        int steps = 0;
        const std::vector<int32_t> kl = dedup_by_fixpoint(v, orig, &steps);
        bool same = (int32_t)kl.size() == n_seq;
        for (int32_t q = 0; same && q < n_seq; ++q)
            same = v[kl[q]].pos == seq[q].pos && v[kl[q]].key == seq[q].key;
        if (!same) {
            std::printf("dedup mismatch row %d n=%d: kept %zu vs %d\n", r, n, kl.size(), n_seq);
            return 1;
        }
        max_steps = std::max(max_steps, steps);
        total_steps += steps;
        ++done;
    }
    std::printf("ok %d (dedup fixpoint steps: mean %.2f, max %d)\n", done,
                (double)total_steps / done, max_steps);
    return 0;
}
