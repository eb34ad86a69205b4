// Test harness (CPU only): checks the engine's staged row merge
// (ncvis_gb300/csrc/merge_row.cuh, compiled here as host C++, once over plain
// arrays and once over strided views like the GPU's shared-memory rows)
// against a direct statement of the reference's per-row symmetrization
// (src/knntable.cpp:40-49 append order, 81-83 std::sort of an index array by
// distance, 85-93 in-place deduplication) on random rows with repeated
// indices and tied distances.  Prints "ok <rows>" or the first mismatch.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <numeric>
#include <random>
#include <vector>

#include "merge_row.cuh"

using ncvis_gpu::SortItem;

// The reference's steps for one row: own entries, then incoming entries in
// ascending entry id; sort positions by distance; keep position idx[j] unless
// the (partly overwritten) row's index there equals the one at idx[j-1].
static int32_t reference_row(const std::vector<int32_t> &own_i, const std::vector<float> &own_d,
                             std::vector<int32_t> in_ids, const std::vector<float> &table_d,
                             int32_t k, std::vector<int32_t> &col, std::vector<float> &val) {
    std::sort(in_ids.begin(), in_ids.end());
    std::vector<int32_t> inds(own_i);
    std::vector<float> dists(own_d);
    for (int32_t e : in_ids) {
        inds.push_back(e / k);
        dists.push_back(table_d[e]);
    }
    std::vector<long> idx(inds.size());
    std::iota(idx.begin(), idx.end(), 0L);
    const std::vector<int32_t> inds_tmp(inds);
    const std::vector<float> dists_tmp(dists);
    std::sort(idx.begin(), idx.end(), [&dists](long a, long b) { return dists[a] < dists[b]; });
    int32_t n = 0;
    for (size_t j = 0; j < idx.size(); ++j) {
        if (j == 0 || inds[idx[j]] != inds[idx[j - 1]]) {
            inds[n] = inds_tmp[idx[j]];
            dists[n] = dists_tmp[idx[j]];
            ++n;
        }
    }
    col.assign(inds.begin(), inds.begin() + n);
    val.assign(dists.begin(), dists.begin() + n);
    return n;
}

int main(int argc, char **argv) {
    const int rows = argc > 1 ? std::atoi(argv[1]) : 20000;
    std::mt19937_64 rng(2024);
    const int stride = 5;  // rows interleaved like a block's threads
    int done = 0;
    for (int r = 0; r < rows; ++r) {
        const int32_t k = 1 + (int32_t)(rng() % 20);
        const int32_t n_src = 1 + (int32_t)(rng() % 400);  // table rows the incoming ids come from
        const int32_t nin = (int32_t)(rng() % (r % 7 == 0 ? 400 : 60));
        const int32_t n_idx = 1 + (int32_t)(rng() % (r % 3 == 0 ? 6 : 200));  // distinct neighbour ids
        const int32_t n_key = 1 + (int32_t)(rng() % (r % 2 == 0 ? 4 : 1000));  // distinct distances
        std::vector<float> table_d((size_t)n_src * k);
        for (auto &d : table_d) d = (float)(rng() % n_key) * 0.25f;
        std::vector<int32_t> own_i(k);
        std::vector<float> own_d(k);
        for (int32_t p = 0; p < k; ++p) {
            own_i[p] = (int32_t)(rng() % n_idx);
            own_d[p] = (float)(rng() % n_key) * 0.25f;
        }
        std::vector<int32_t> all((size_t)n_src * k);
        std::iota(all.begin(), all.end(), 0);
        std::shuffle(all.begin(), all.end(), rng);
        const int32_t m = std::min<int32_t>(nin, (int32_t)all.size());
        std::vector<int32_t> in_ids(all.begin(), all.begin() + m);
        // Incoming ids carry the source row e / k as the index: make some of
        // those equal own indices so duplicates span both halves.
        std::vector<int32_t> want_c;
        std::vector<float> want_v;
        const int32_t nw = reference_row(own_i, own_d, in_ids, table_d, k, want_c, want_v);

        const int32_t L = k + m;
        for (int form = 0; form < 2; ++form) {
            std::vector<SortItem> it_store((size_t)L * stride);
            std::vector<int32_t> og_store((size_t)L * stride);
            std::vector<int32_t> got_c(L, -7);
            std::vector<float> got_v(L, -7.f);
            int32_t ng;
            if (form == 0) {
                ng = ncvis_gpu::merge_row(it_store.data(), og_store.data(), L, k, own_i.data(),
                                          own_d.data(), in_ids.data(), table_d.data(),
                                          got_c.data(), got_v.data());
            } else {
                const int lane = r % stride;
                ncvis_gpu::StridedItems items{it_store.data() + lane, stride};
                ncvis_gpu::StridedInts orig{og_store.data() + lane, stride};
                ng = ncvis_gpu::merge_row(items, orig, L, k, own_i.data(), own_d.data(),
                                          in_ids.data(), table_d.data(), got_c.data(),
                                          got_v.data());
            }
            bool same = ng == nw;
            for (int32_t q = 0; same && q < nw; ++q)
                same = got_c[q] == want_c[q] && got_v[q] == want_v[q];
            if (!same) {
                std::printf("mismatch row %d form %d: k=%d nin=%d kept %d vs %d\n", r, form, k, m,
                            ng, nw);
                return 1;
            }
        }
        ++done;
    }
    std::printf("ok %d\n", done);
    return 0;
}
