// Test harness (CPU only): checks that the engine's introsort
// (ncvis_gb300/csrc/introsort.cuh, compiled here as host C++) yields the same
// permutation as this toolchain's std::sort with the reference's comparator
// (src/knntable.cpp:81-83) on random, tie-heavy and adversarial keys.
// Prints "ok <cases>" or the first mismatch; exit code 0 on success.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <numeric>
#include <random>
#include <vector>

#include "introsort.cuh"

using ncvis_gpu::SortItem;

static bool check(const std::vector<float> &key) {
    const int32_t n = (int32_t)key.size();
    std::vector<long> idx(n);
    std::iota(idx.begin(), idx.end(), 0L);
    std::sort(idx.begin(), idx.end(), [&key](long a, long b) { return key[a] < key[b]; });
    std::vector<SortItem> items(n);
    for (int32_t i = 0; i < n; ++i) items[i] = SortItem{key[i], i};
    ncvis_gpu::libstdcxx_sort(items.data(), n);
    for (int32_t i = 0; i < n; ++i)
        if (items[i].pos != idx[i]) {
            std::printf("mismatch n=%d at %d: %d vs %ld\n", n, i, items[i].pos, idx[i]);
            return false;
        }
    return true;
}

int main(int argc, char **argv) {
    const int cases = argc > 1 ? std::atoi(argv[1]) : 20000;
    std::mt19937_64 rng(12345);
    int done = 0;
    for (int c = 0; c < cases; ++c) {
        int n;
        switch (c % 4) {
            case 0: n = (int)(rng() % 40); break;
            case 1: n = (int)(rng() % 200); break;
            case 2: n = (int)(rng() % 3000); break;
            default: n = 16 + (int)(rng() % 3); break;
        }
        const int distinct = 1 + (int)(rng() % (c % 3 == 0 ? 4 : (c % 3 == 1 ? 64 : 1000000)));
        std::vector<float> key(n);
        const int pattern = (int)(rng() % 6);
        for (int i = 0; i < n; ++i) {
            switch (pattern) {
                case 0: key[i] = (float)(rng() % distinct); break;            // random with ties
                case 1: key[i] = (float)i; break;                             // ascending
                case 2: key[i] = (float)(n - i); break;                       // descending
                case 3: key[i] = (float)((i % 2) ? i : n - i); break;         // zig-zag
                case 4: key[i] = (float)(i % (1 + distinct % 7)); break;      // sawtooth with ties
                default: key[i] = (float)((i * 7919) % (1 + n / 2)) * 0.5f;   // permuted pairs
            }
        }
        // Pairs of equal keys, as symmetrization produces for mutual neighbours.
        if (c % 5 == 0 && n > 1) key[n - 1] = key[rng() % (n - 1)];
        if (!check(key)) return 1;
        ++done;
    }
    // Median-of-three adversary: forces the depth budget out and the heap-sort
    // fallback (organ-pipe and its variants).
    for (int n = 17; n < 5000; n = n * 3 / 2 + 1) {
        std::vector<float> key(n);
        for (int i = 0; i < n; ++i) key[i] = (float)std::min(i, n - 1 - i);
        if (!check(key)) return 1;
        for (int i = 0; i < n; ++i) key[i] = (float)((i % 2 == 0) ? i / 2 : n / 2 + i / 2);
        if (!check(key)) return 1;
        done += 2;
    }
    // Killer sequence for median-of-3 quicksort (Musser 1997): makes every
    // partition unbalanced so that the heap-sort fallback runs.
    for (int k = 9; k < 2000; k += 37) {
        const int n = 2 * k;
        std::vector<float> key(n);
        for (int i = 1; i <= k; ++i) {
            if (i % 2) {
                key[i - 1] = (float)i;
                key[i] = (float)(k + i);
            }
            key[k + i - 1] = (float)(2 * i);
        }
        if (!check(key)) return 1;
        ++done;
    }
    std::printf("ok %d\n", done);
    return 0;
}
