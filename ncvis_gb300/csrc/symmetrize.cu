// K5: symmetrization of the kNN table into CSR, bit-exact with the
// reference's KNNTable::symmetrize run on one thread (src/knntable.cpp:24-99)
// followed by NCVis::build_edges (src/ncvis.cpp:155-173).
//
// The reference's row i after symmetrization is computed from
//   row  = its k table entries, then every incoming entry (s, j) with
//          inds[s][j] == i in increasing (s, j) order (one thread pushes them
//          in that order, src/knntable.cpp:40-49),
//   order = std::sort of 0..len-1 by row distance (unstable introsort),
//   dedup = keep order[j] unless the index at order[j] equals the index at
//           order[j-1], where both are read from the row while it is being
//           overwritten with the kept entries (src/knntable.cpp:85-93).
// Here:
//   1. count_targets / scan: in-degree of every row and bucket offsets;
//   2. scatter_incoming: each table entry e = s*k + j appends e to its
//      target's bucket (atomic cursor; arrival order is not deterministic);
//   3. merge, one thread per row (merge_row.cuh): sorts its bucket by e,
//      which restores the one-thread arrival order, builds the row's
//      (distance, position) items, runs the libstdc++-equivalent introsort
//      (introsort.cuh) and the in-place deduplication, all in the thread's
//      slots of shared memory (merge_rows_thread, rows of up to 48 items);
//      longer rows are listed and merged one warp per row (merge_rows_wpar up
//      to 128 items, the sort spread over the lanes; merge_rows_warp in tiers
//      of 1,024 and 8,192 items), longer still on a row-aligned global
//      scratch;
//   4. scan of the kept counts -> row_ptr; compact_rows writes cols, vals and
//      the source row of every entry (the build_edges pairs).
#include <algorithm>

#include "common.cuh"
#include "introsort.cuh"
#include "merge_row.cuh"
#include "stages.cuh"

namespace ncvis_gpu {

namespace {

// Merge tiers by row length k + in-degree (~30 on average): up to 48 items
// one thread per row (12 B per item in shared memory: the sort item and the
// row's index at that position; 3 blocks of 128 threads per SM); up to 128
// items one warp per row with the sort spread over the lanes
// (merge_rows_wpar); longer rows one warp per row with the sort on one lane,
// in tiers of 1,024 and 8,192 items (hubs: rows of up to ~1,000 items occur in
// 64-dimensional mixtures of a few thousand points); longer still on the
// global scratch.
constexpr int kCap0 = 48, kThreads0 = 128;
constexpr int kWarps1 = 8;
constexpr int kCap2 = 1024, kWarps2 = 4;
constexpr int kCap3 = 8192, kWarps3 = 1;

// Flags any index outside [0, N) (the table must name existing points).
__global__ void check_indices(const int32_t *__restrict__ inds, int64_t nk, int64_t N,
                              int *__restrict__ bad) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nk;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t t = inds[e];
        if (t < 0 || t >= N) atomicOr(bad, 1);
    }
}

// bad = 1 if any entry of a or b (n each; b may be null) lies outside [0, N).
__global__ void check_pairs(const int32_t *__restrict__ a, const int32_t *__restrict__ b,
                            int64_t n, int64_t N, int *__restrict__ bad) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t t = a[e];
        const int32_t u = b ? b[e] : 0;
        if (t < 0 || t >= N || u < 0 || u >= N) atomicOr(bad, 1);
    }
}

__global__ void count_targets(const int32_t *__restrict__ inds, int64_t nk,
                              int32_t *__restrict__ indeg) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nk;
         e += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&indeg[inds[e]], 1);
}

__global__ void scatter_incoming(const int32_t *__restrict__ inds, int64_t nk,
                                 const int64_t *__restrict__ in_off, int32_t *__restrict__ cursor,
                                 int32_t *__restrict__ in_key) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nk;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t t = inds[e];
        const int32_t slot = atomicAdd(&cursor[t], 1);
        in_key[in_off[t] + slot] = (int32_t)e;
    }
}

template <class V>
__device__ __forceinline__ int32_t merge_one(V items, int L, int k, const int32_t *__restrict__ own_i,
                                             const float *__restrict__ own_d,
                                             const int32_t *__restrict__ ink,
                                             const float *__restrict__ dists, int32_t *out_col,
                                             float *out_val) {
    for (int p = 0; p < k; ++p) items[p] = SortItem{own_d[p], p};
    for (int p = k; p < L; ++p) items[p] = SortItem{dists[ink[p - k]], p};
    libstdcxx_sort(items, L);
    // Index stored at row position p before the dedup loop touched it.
    auto orig = [&](int p) -> int32_t { return p < k ? own_i[p] : ink[p - k] / k; };
    int32_t n_out = 0;
    for (int j = 0; j < L; ++j) {
        const SortItem cur = items[j];
        bool keep = (j == 0);
        if (!keep) {
            const int p = cur.pos, q = items[j - 1].pos;
            const int32_t vp = p < n_out ? out_col[p] : orig(p);
            const int32_t vq = q < n_out ? out_col[q] : orig(q);
            keep = (vp != vq);
        }
        if (keep) {
            out_col[n_out] = orig(cur.pos);
            out_val[n_out] = cur.key;
            ++n_out;
        }
    }
    return n_out;
}

// Rows whose k + in-degree exceeds every tier: the row-aligned global scratch.
__device__ int32_t merge_global(int64_t i, int k, const int32_t *__restrict__ inds,
                                const float *__restrict__ dists, const int64_t *__restrict__ in_off,
                                int32_t *__restrict__ in_key, SortItem *__restrict__ g_items,
                                int32_t *__restrict__ out_col, float *__restrict__ out_val) {
    const int64_t ib = in_off[i];
    const int nin = (int)(in_off[i + 1] - ib);
    const int64_t base = i * k + ib;
    int32_t *ink = in_key + ib;
    sort_distinct_ints(ink, 0, nin);
    return merge_one(g_items + base, k + nin, k, inds + i * k, dists + i * k, ink, dists,
                     out_col + base, out_val + base);
}

// First tier: every row, one thread each; its items live in the thread's
// slots of shared memory ([C][T] sort items, then [C][T] indices; slot i of
// thread t is element i * T + t).  A row of more than C items is appended to
// `next` for the warp tiers.
template <int C, int T>
__global__ void __launch_bounds__(T, 1) merge_rows_thread(
    int64_t N, int k, const int32_t *__restrict__ inds, const float *__restrict__ dists,
    const int64_t *__restrict__ in_off, const int32_t *__restrict__ in_key,
    int32_t *__restrict__ out_col, float *__restrict__ out_val, int32_t *__restrict__ kept,
    int32_t *__restrict__ next, int32_t *__restrict__ n_next) {
    extern __shared__ __align__(16) SortItem sm_items[];
    int32_t *sm_orig = reinterpret_cast<int32_t *>(sm_items + C * T);
    const int64_t i = (int64_t)blockIdx.x * T + threadIdx.x;
    if (i >= N) return;
    const int64_t ib = in_off[i];
    const int nin = (int)(in_off[i + 1] - ib);
    const int L = k + nin;
    if (L > C) {
        next[atomicAdd(n_next, 1)] = (int32_t)i;
        return;
    }
    const int64_t base = i * k + ib;  // row-aligned output offset
    StridedItems items{sm_items + threadIdx.x, T};
    StridedInts orig{sm_orig + threadIdx.x, T};
    kept[i] = merge_row(items, orig, L, k, inds + i * k, dists + i * k, in_key + ib, dists,
                        out_col + base, out_val + base);
}

// Warp tiers: the listed rows rows[0 .. *n_rows), one warp each (W warps per
// block, C items per warp in shared memory: [W][C] sort items, then [W][C]
// indices).  Long rows are rare, and one thread per row would leave a warp
// running 32 of them one after the other through divergent sorts.  The warp
// loads the row, sorts its incoming ids (each id's rank among the row's ids;
// the ids are distinct) and gathers the distances in parallel; lane 0 runs
// the sort and the deduplication (sequential: the tie order is
// libstdc++'s); the warp writes the kept entries.  A row of more than C
// items goes to `next`, or, in the last tier, to the global scratch.
template <int C, int W>
__global__ void __launch_bounds__(32 * W, 1) merge_rows_warp(
    int k, const int32_t *__restrict__ inds, const float *__restrict__ dists,
    const int64_t *__restrict__ in_off, int32_t *__restrict__ in_key, SortItem *__restrict__ g_items,
    int32_t *__restrict__ out_col, float *__restrict__ out_val, int32_t *__restrict__ kept,
    const int32_t *__restrict__ rows, const int32_t *__restrict__ n_rows, int32_t *__restrict__ next,
    int32_t *__restrict__ n_next) {
    extern __shared__ __align__(16) SortItem sm_items[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    SortItem *items = sm_items + (size_t)warp * C;
    int32_t *orig = reinterpret_cast<int32_t *>(sm_items + (size_t)W * C) + (size_t)warp * C;
    int32_t *sorted_ids = reinterpret_cast<int32_t *>(items);  // 2C ints before the items exist
    const int64_t count = *n_rows;
    for (int64_t w = (int64_t)blockIdx.x * W + warp; w < count; w += (int64_t)gridDim.x * W) {
        const int64_t i = rows[w];
        const int64_t ib = in_off[i];
        const int nin = (int)(in_off[i + 1] - ib);
        const int L = k + nin;
        const int64_t base = i * k + ib;  // row-aligned output offset
        if (L > C) {
            if (lane == 0) {
                if (next)
                    next[atomicAdd(n_next, 1)] = (int32_t)i;
                else
                    kept[i] = merge_global(i, k, inds, dists, in_off, in_key, g_items, out_col,
                                           out_val);
            }
            continue;
        }
        const int32_t *ink = in_key + ib;
        for (int q = lane; q < nin; q += 32) orig[k + q] = ink[q];
        __syncwarp();
        for (int q = lane; q < nin; q += 32) {
            const int32_t e = orig[k + q];
            int r = 0;
            for (int t = 0; t < nin; ++t) r += orig[k + t] < e;
            sorted_ids[r] = e;
        }
        __syncwarp();
        for (int q = lane; q < nin; q += 32) orig[k + q] = sorted_ids[q];
        __syncwarp();
        for (int p = lane; p < L; p += 32) {
            if (p < k) {
                items[p] = SortItem{dists[i * k + p], p};
                orig[p] = inds[i * k + p];
            } else {
                const int32_t e = orig[p];
                items[p] = SortItem{dists[e], p};
                orig[p] = e / k;
            }
        }
        __syncwarp();
        int32_t n_out = 0;
        if (lane == 0) n_out = sort_and_dedup(items, orig, L);
        n_out = __shfl_sync(0xffffffffu, n_out, 0);
        __syncwarp();
        for (int q = lane; q < n_out; q += 32) {
            const SortItem it = items[q];
            out_col[base + q] = orig[it.pos];
            out_val[base + q] = it.key;
        }
        if (lane == 0) kept[i] = n_out;
        __syncwarp();
    }
}

// Data-parallel warp tier: rows of up to 128 items, one warp each, with the
// sort and the deduplication spread over the lanes and results identical to
// the sequential ones:
//   * each Hoare partition of the introsort (median of three into the first
//     slot by lane 0) is computed from two position lists built by ballots:
//     G, the positions after the pivot whose key is not below it, ascending;
//     S, the positions whose key is not above it, descending, with the
//     pivot's own position last.  The t-th swap exchanges G[t] and S[t] for
//     every t with G[t] < S[t]; after t* swaps the cut is
//     min(G[t*], S[t*-1]) (S[-1] = the range's end);
//   * ranges left at 16 items or fewer, and ranges heap-sorted by lane 0
//     when the depth budget runs out, are leaves; std::sort's final insertion
//     sort is stable, so each leaf is then stably sorted by key in place
//     (every item's rank within its leaf);
//   * the deduplication's keep flags are the fixpoint of one parallel step
//     (item j kept or not from the kept items of the previous guess), which
//     agrees with the sequential loop from the start up to one more item per
//     step.
// Shared memory per warp: WparRow.
constexpr int kWparCap = 128;
struct WparRow {
    SortItem items[kWparCap];
    int32_t orig[kWparCap];
    int32_t ids[kWparCap];
    int16_t G[kWparCap], S[kWparCap], kl[kWparCap];
    uint8_t blo[kWparCap], bhi_m1[kWparCap];  // leaf [blo, bhi_m1 + 1)
};

__device__ __forceinline__ int32_t warp_partition(WparRow &w, int32_t lo, int32_t hi, int lane) {
    if (lane == 0)
        introsort_detail::median_to(w.items, lo, lo + 1, lo + (hi - lo) / 2, hi - 1);
    __syncwarp();
    const float P = w.items[lo].key;
    const unsigned lt = (1u << lane) - 1u;
    unsigned bg[4], bl[4];
    int nl = 1;  // the pivot's own position
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        const int32_t p = lo + 1 + 32 * m + lane;
        const bool valid = p < hi;
        const float key = valid ? w.items[p].key : 0.f;
        bg[m] = __ballot_sync(0xffffffffu, valid && !(key < P));
        bl[m] = __ballot_sync(0xffffffffu, valid && !(P < key));
        nl += __popc(bl[m]);
    }
    int ng = 0, cl = 0;
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        const int32_t p = lo + 1 + 32 * m + lane;
        if ((bg[m] >> lane) & 1u) w.G[ng + __popc(bg[m] & lt)] = (int16_t)p;
        if ((bl[m] >> lane) & 1u) w.S[nl - 2 - cl - __popc(bl[m] & lt)] = (int16_t)p;
        ng += __popc(bg[m]);
        cl += __popc(bl[m]);
    }
    if (lane == 0) w.S[nl - 1] = (int16_t)lo;
    __syncwarp();
    const int pairs = min(ng, nl);
    int ts = 0;
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        const int t = 32 * m + lane;
        ts += __popc(__ballot_sync(0xffffffffu, t < pairs && w.G[t] < w.S[t]));
    }
    // At most 64 swaps (each moves two distinct positions of <= 127).
    SortItem a[2], b[2];
#pragma unroll
    for (int m = 0; m < 2; ++m) {
        const int t = 32 * m + lane;
        if (t < ts) a[m] = w.items[w.G[t]], b[m] = w.items[w.S[t]];
    }
    __syncwarp();
#pragma unroll
    for (int m = 0; m < 2; ++m) {
        const int t = 32 * m + lane;
        if (t < ts) w.items[w.G[t]] = b[m], w.items[w.S[t]] = a[m];
    }
    int32_t cut = ts > 0 ? (int32_t)w.S[ts - 1] : hi;
    if (ts < ng) cut = min(cut, (int32_t)w.G[ts]);
    __syncwarp();
    return cut;
}

template <int W>
__global__ void __launch_bounds__(32 * W, 1) merge_rows_wpar(
    int k, const int32_t *__restrict__ inds, const float *__restrict__ dists,
    const int64_t *__restrict__ in_off, const int32_t *__restrict__ in_key,
    int32_t *__restrict__ out_col, float *__restrict__ out_val, int32_t *__restrict__ kept,
    const int32_t *__restrict__ rows, const int32_t *__restrict__ n_rows, int32_t *__restrict__ next,
    int32_t *__restrict__ n_next) {
    extern __shared__ __align__(16) unsigned char wpar_raw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    WparRow &w = reinterpret_cast<WparRow *>(wpar_raw)[warp];
    const unsigned lt = (1u << lane) - 1u;
    const int64_t count = *n_rows;
    for (int64_t r = (int64_t)blockIdx.x * W + warp; r < count; r += (int64_t)gridDim.x * W) {
        const int64_t i = rows[r];
        const int64_t ib = in_off[i];
        const int nin = (int)(in_off[i + 1] - ib);
        const int L = k + nin;
        const int64_t base = i * k + ib;  // row-aligned output offset
        if (L > kWparCap) {
            if (lane == 0) next[atomicAdd(n_next, 1)] = (int32_t)i;
            continue;
        }
        // The incoming ids, ranked (distinct), then the row's items.
        for (int q = lane; q < nin; q += 32) w.orig[k + q] = in_key[ib + q];
        __syncwarp();
        for (int q = lane; q < nin; q += 32) {
            const int32_t e = w.orig[k + q];
            int rk = 0;
            for (int t = 0; t < nin; ++t) rk += w.orig[k + t] < e;
            w.ids[rk] = e;
        }
        __syncwarp();
        for (int p = lane; p < L; p += 32) {
            if (p < k) {
                w.items[p] = SortItem{dists[i * k + p], p};
                w.orig[p] = inds[i * k + p];
            } else {
                const int32_t e = w.ids[p - k];
                w.items[p] = SortItem{dists[e], p};
                w.orig[p] = e / k;
            }
        }
        __syncwarp();
        // The introsort's partitions and leaves (a warp-uniform range stack).
        int32_t st_lo[16], st_hi[16], st_d[16];
        int top = 0;
        st_lo[0] = 0, st_hi[0] = L, st_d[0] = 2 * introsort_detail::floor_log2(max(L, 1));
        top = 1;
        while (top > 0) {
            --top;
            int32_t lo = st_lo[top], hi = st_hi[top], depth = st_d[top];
            while (hi - lo > 16) {
                if (depth == 0) {
                    if (lane == 0)
                        introsort_detail::heap_sort(
                            introsort_detail::Offset<SortItem *>{w.items, lo}, hi - lo);
                    __syncwarp();
                    break;
                }
                --depth;
                const int32_t cut = warp_partition(w, lo, hi, lane);
                st_lo[top] = cut, st_hi[top] = hi, st_d[top] = depth;
                ++top;
                hi = cut;
            }
            for (int32_t x = lo + lane; x < hi; x += 32)
                w.blo[x] = (uint8_t)lo, w.bhi_m1[x] = (uint8_t)(hi - 1);
        }
        __syncwarp();
        // Each leaf stably sorted by key in place.
        {
            SortItem mine[4];
            int dest[4];
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                const int x = lane + 32 * m;
                if (x < L) {
                    const SortItem it = w.items[x];
                    const int b0 = w.blo[x], b1 = (int)w.bhi_m1[x] + 1;
                    int rk = 0;
                    for (int y = b0; y < b1; ++y) {
                        const float ky = w.items[y].key;
                        rk += (ky < it.key) | ((ky == it.key) & (y < x));
                    }
                    mine[m] = it;
                    dest[m] = b0 + rk;
                }
            }
            __syncwarp();
#pragma unroll
            for (int m = 0; m < 4; ++m)
                if (lane + 32 * m < L) w.items[dest[m]] = mine[m];
            __syncwarp();
        }
        // Deduplication: keep flags to their fixpoint (at most L + 1 steps).
        unsigned K[4];
#pragma unroll
        for (int m = 0; m < 4; ++m) K[m] = __ballot_sync(0xffffffffu, lane + 32 * m < L);
        for (int step = 0; step <= L + 1; ++step) {
            int nj[4], before = 0;
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                nj[m] = before + __popc(K[m] & lt);
                if ((K[m] >> lane) & 1u) w.kl[nj[m]] = (int16_t)(lane + 32 * m);
                before += __popc(K[m]);
            }
            __syncwarp();
            bool same = true;
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                const int j = lane + 32 * m;
                bool kp = false;
                if (j < L) {
                    if (j == 0) {
                        kp = true;
                    } else {
                        const int p = w.items[j].pos, q = w.items[j - 1].pos, n = nj[m];
                        const int32_t vp = w.orig[p < n ? w.items[w.kl[p]].pos : p];
                        const int32_t vq = w.orig[q < n ? w.items[w.kl[q]].pos : q];
                        kp = vp != vq;
                    }
                }
                const unsigned nk = __ballot_sync(0xffffffffu, kp);
                same &= nk == K[m];
                K[m] = nk;
            }
            if (same) break;
            __syncwarp();
        }
        int n_out = 0;
#pragma unroll
        for (int m = 0; m < 4; ++m) n_out += __popc(K[m]);
        for (int q = lane; q < n_out; q += 32) {
            const SortItem it = w.items[w.kl[q]];
            out_col[base + q] = w.orig[it.pos];
            out_val[base + q] = it.key;
        }
        if (lane == 0) kept[i] = n_out;
        __syncwarp();
    }
}

template <int W>
void launch_merge_wpar(int k, const int32_t *inds, const float *dists, const int64_t *in_off,
                       int32_t *in_key, int32_t *out_col, float *out_val, int32_t *kept,
                       const int32_t *rows, const int32_t *n_rows, int32_t *next, int32_t *n_next,
                       cudaStream_t s);

// Blocks per SM for a block of `threads` threads and `smem` bytes of shared
// memory (the warp tiers use 64 registers per thread: 1,024 threads per SM).
inline int blocks_per_sm(size_t smem, int threads) {
    const int by_smem = (int)std::max<size_t>(1, (227 * 1024) / (smem + 1024));
    return std::max(1, std::min(by_smem, 1024 / threads));
}

template <int W>
void launch_merge_wpar(int k, const int32_t *inds, const float *dists, const int64_t *in_off,
                       int32_t *in_key, int32_t *out_col, float *out_val, int32_t *kept,
                       const int32_t *rows, const int32_t *n_rows, int32_t *next, int32_t *n_next,
                       cudaStream_t s) {
    const size_t smem = sizeof(WparRow) * W;
    NCVIS_CUDA(cudaFuncSetAttribute(merge_rows_wpar<W>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // A grid of resident blocks (registers, not shared memory, bound them).
    int per_sm = 0;
    NCVIS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, merge_rows_wpar<W>, 32 * W,
                                                             smem));
    const int64_t grid = (int64_t)num_sms() * std::max(per_sm, 1);
    NCVIS_LAUNCH((merge_rows_wpar<W>), grid, 32 * W, smem, s, k, inds, dists, in_off, in_key,
                 out_col, out_val, kept, rows, n_rows, next, n_next);
}

template <int C, int W>
void launch_merge_warp(int k, const int32_t *inds, const float *dists, const int64_t *in_off,
                       int32_t *in_key, SortItem *g_items, int32_t *out_col, float *out_val,
                       int32_t *kept, const int32_t *rows, const int32_t *n_rows, int32_t *next,
                       int32_t *n_next, cudaStream_t s) {
    const size_t smem = (sizeof(SortItem) + sizeof(int32_t)) * C * W;
    // Set on every launch: the attribute is per device, and a cached flag
    // would race between host threads running different engines.
    NCVIS_CUDA(cudaFuncSetAttribute(merge_rows_warp<C, W>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // A grid of resident blocks that reads the list's length on the device.
    const int64_t grid = (int64_t)num_sms() * blocks_per_sm(smem, 32 * W);
    NCVIS_LAUNCH((merge_rows_warp<C, W>), grid, 32 * W, smem, s, k, inds, dists, in_off, in_key,
                 g_items, out_col, out_val, kept, rows, n_rows, next, n_next);
}

__global__ void compact_rows(int64_t N, int k, const int64_t *__restrict__ in_off,
                             const int32_t *__restrict__ kept, const int64_t *__restrict__ row_ptr,
                             const int32_t *__restrict__ out_col, const float *__restrict__ out_val,
                             int32_t *__restrict__ cols, float *__restrict__ vals,
                             int32_t *__restrict__ src) {
    const int lane = threadIdx.x & 31;
    const int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (i >= N) return;
    const int64_t from = i * k + in_off[i];
    const int64_t to = row_ptr[i];
    const int n = kept[i];
    for (int j = lane; j < n; j += 32) {
        cols[to + j] = out_col[from + j];
        vals[to + j] = out_val[from + j];
        if (src) src[to + j] = (int32_t)i;
    }
}

struct SymWs {
    int32_t *indeg, *cursor, *in_key, *out_col, *kept, *bad, *tier1, *tier2, *n_tier;
    int64_t *in_off;
    SortItem *items;
    float *out_val;
    void *scan;
};

inline size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

SymWs carve(void *ws, int64_t N, int k) {
    char *p = (char *)ws;
    SymWs w;
    const int64_t nk = N * k;
    w.indeg = (int32_t *)p;    p += align256(sizeof(int32_t) * N);
    w.cursor = (int32_t *)p;   p += align256(sizeof(int32_t) * N);
    w.kept = (int32_t *)p;     p += align256(sizeof(int32_t) * N);
    w.bad = (int32_t *)p;      p += align256(sizeof(int32_t));
    w.n_tier = (int32_t *)p;   p += align256(3 * sizeof(int32_t));
    w.tier1 = (int32_t *)p;    p += align256(sizeof(int32_t) * N);
    w.tier2 = (int32_t *)p;    p += align256(sizeof(int32_t) * N);
    w.in_off = (int64_t *)p;   p += align256(sizeof(int64_t) * (N + 1));
    w.in_key = (int32_t *)p;   p += align256(sizeof(int32_t) * nk);
    w.items = (SortItem *)p;   p += align256(sizeof(SortItem) * 2 * nk);
    w.out_col = (int32_t *)p;  p += align256(sizeof(int32_t) * 2 * nk);
    w.out_val = (float *)p;    p += align256(sizeof(float) * 2 * nk);
    w.scan = p;
    return w;
}

}  // namespace

bool indices_in_range(const int32_t *a, int64_t n, int64_t N, cudaStream_t s) {
    return edges_in_range(a, nullptr, n, N, s);
}

// One check kernel over both arrays and one wait for its flag.
bool edges_in_range(const int32_t *a, const int32_t *b, int64_t n, int64_t N, cudaStream_t s) {
    if (n == 0) return true;
    StreamBuffer flag(sizeof(int), s);
    int *bad = (int *)flag.p;
    NCVIS_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), s));
    const unsigned grid = (unsigned)std::min<int64_t>((n + 255) / 256, 16 * num_sms());
    NCVIS_LAUNCH(check_pairs, grid, 256, 0, s, a, b, n, N, bad);
    int h = 0;
    NCVIS_CUDA(cudaMemcpyAsync(&h, bad, sizeof(int), cudaMemcpyDeviceToHost, s));
    NCVIS_CUDA(cudaStreamSynchronize(s));
    return h == 0;
}

size_t symmetrize_workspace_bytes(int64_t N, int k) {
    const int64_t nk = N * k;
    return 5 * align256(sizeof(int32_t) * N) + align256(sizeof(int32_t)) +
           align256(3 * sizeof(int32_t)) +
           align256(sizeof(int64_t) * (N + 1)) +
           align256(sizeof(int32_t) * nk) + align256(sizeof(SortItem) * 2 * nk) +
           align256(sizeof(int32_t) * 2 * nk) + align256(sizeof(float) * 2 * nk) +
           align256(scan_workspace_bytes(N));
}

int64_t run_symmetrize(int64_t N, int k, const int32_t *inds, const float *dists, void *workspace,
                       int64_t *row_ptr, int32_t *cols, float *vals, int32_t *src,
                       cudaStream_t s) {
    require(N >= 1 && k >= 1, "symmetrize: empty table");
    require(N * (int64_t)k < (int64_t(1) << 30), "symmetrize: N * k must be below 2^30");
    SymWs w = carve(workspace, N, k);
    const int64_t nk = N * k;
    const unsigned grid = (unsigned)std::min<int64_t>((nk + 255) / 256, 16 * num_sms());
    NCVIS_CUDA(cudaMemsetAsync(w.bad, 0, sizeof(int32_t), s));
    NCVIS_LAUNCH(check_indices, grid, 256, 0, s, inds, nk, N, w.bad);
    int bad = 0;
    NCVIS_CUDA(cudaMemcpyAsync(&bad, w.bad, sizeof(int), cudaMemcpyDeviceToHost, s));
    NCVIS_CUDA(cudaStreamSynchronize(s));
    require(bad == 0, "symmetrize: the kNN table holds an index outside [0, N)");
    NCVIS_CUDA(cudaMemsetAsync(w.indeg, 0, sizeof(int32_t) * N, s));
    NCVIS_CUDA(cudaMemsetAsync(w.cursor, 0, sizeof(int32_t) * N, s));
    NCVIS_LAUNCH(count_targets, grid, 256, 0, s, inds, nk, w.indeg);
    launch_exclusive_scan_i32_to_i64(w.indeg, w.in_off, N, w.scan, s);
    NCVIS_LAUNCH(scatter_incoming, grid, 256, 0, s, inds, nk, w.in_off, w.cursor, w.in_key);
    NCVIS_CUDA(cudaMemsetAsync(w.n_tier, 0, 3 * sizeof(int32_t), s));
    {
        const size_t smem = (sizeof(SortItem) + sizeof(int32_t)) * kCap0 * kThreads0;
        NCVIS_CUDA(cudaFuncSetAttribute(merge_rows_thread<kCap0, kThreads0>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        NCVIS_LAUNCH((merge_rows_thread<kCap0, kThreads0>), ceil_div(N, kThreads0), kThreads0,
                     smem, s, N, k, inds, dists, w.in_off, w.in_key, w.out_col, w.out_val, w.kept,
                     w.tier1, w.n_tier);
    }
    launch_merge_wpar<kWarps1>(k, inds, dists, w.in_off, w.in_key, w.out_col, w.out_val, w.kept,
                               w.tier1, w.n_tier, w.tier2, w.n_tier + 1, s);
    launch_merge_warp<kCap2, kWarps2>(k, inds, dists, w.in_off, w.in_key, w.items, w.out_col,
                                      w.out_val, w.kept, w.tier2, w.n_tier + 1, w.tier1,
                                      w.n_tier + 2, s);
    launch_merge_warp<kCap3, kWarps3>(k, inds, dists, w.in_off, w.in_key, w.items, w.out_col,
                                      w.out_val, w.kept, w.tier1, w.n_tier + 2, nullptr, nullptr,
                                      s);
    launch_exclusive_scan_i32_to_i64(w.kept, row_ptr, N, w.scan, s);
    NCVIS_LAUNCH(compact_rows, ceil_div(N, 8), 256, 0, s, N, k, w.in_off, w.kept, row_ptr,
                 w.out_col, w.out_val, cols, vals, src);
    int64_t E = 0;
    NCVIS_CUDA(cudaMemcpyAsync(&E, row_ptr + N, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    NCVIS_CUDA(cudaStreamSynchronize(s));
    return E;
}

}  // namespace ncvis_gpu
