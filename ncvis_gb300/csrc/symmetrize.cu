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
//      slots of shared memory.  Rows go through tiers of growing capacity:
//      every row starts in merge_tier<48> (k + in-degree is ~30 on average);
//      a row that does not fit is appended to the next tier's list
//      (merge_tier<128>, then merge_tier<320>); the few rows longer than the
//      last tier run on a row-aligned global scratch;
//   4. scan of the kept counts -> row_ptr; compact_rows writes cols, vals and
//      the source row of every entry (the build_edges pairs).
#include <algorithm>

#include "common.cuh"
#include "introsort.cuh"
#include "merge_row.cuh"
#include "stages.cuh"

namespace ncvis_gpu {

namespace {

// Merge tiers: items per row held in shared memory (12 B each: the sort item
// and the row's index at that position) and threads per block; each tier's
// blocks fit 3, 2 and 1 times per SM.
constexpr int kCap0 = 48, kThreads0 = 128;
constexpr int kCap1 = 128, kThreads1 = 64;
constexpr int kCap2 = 320, kThreads2 = 32;

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

// One merge tier.  Its rows are 0 .. N-1 (rows == null) or rows[0 .. *n_rows);
// a row of more than C items is appended to next (or, in the last tier, run
// on the global scratch).  Shared memory: [C][T] sort items, then [C][T]
// indices; thread t's slot i of either is element i * T + t.
template <int C, int T>
__global__ void __launch_bounds__(T) merge_tier(
    int64_t N, int k, const int32_t *__restrict__ inds, const float *__restrict__ dists,
    const int64_t *__restrict__ in_off, int32_t *__restrict__ in_key, SortItem *__restrict__ g_items,
    int32_t *__restrict__ out_col, float *__restrict__ out_val, int32_t *__restrict__ kept,
    const int32_t *__restrict__ rows, const int32_t *__restrict__ n_rows, int32_t *__restrict__ next,
    int32_t *__restrict__ n_next) {
    extern __shared__ __align__(16) SortItem sm_items[];
    int32_t *sm_orig = reinterpret_cast<int32_t *>(sm_items + C * T);
    const int64_t count = rows ? (int64_t)*n_rows : N;
    for (int64_t w = (int64_t)blockIdx.x * T + threadIdx.x; w < count; w += (int64_t)gridDim.x * T) {
        const int64_t i = rows ? (int64_t)rows[w] : w;
        const int64_t ib = in_off[i];
        const int nin = (int)(in_off[i + 1] - ib);
        const int L = k + nin;
        const int64_t base = i * k + ib;  // row-aligned output offset
        if (L > C) {
            if (next)
                next[atomicAdd(n_next, 1)] = (int32_t)i;
            else
                kept[i] = merge_global(i, k, inds, dists, in_off, in_key, g_items, out_col, out_val);
            continue;
        }
        StridedItems items{sm_items + threadIdx.x, T};
        StridedInts orig{sm_orig + threadIdx.x, T};
        const int32_t *ink = in_key + ib;
        for (int q = 0; q < nin; ++q) orig[k + q] = ink[q];
        kept[i] = merge_row(items, orig, L, k, inds + i * k, dists + i * k, dists, out_col + base,
                            out_val + base);
    }
}

template <int C, int T>
void launch_merge_tier(int64_t N, int k, const int32_t *inds, const float *dists,
                       const int64_t *in_off, int32_t *in_key, SortItem *g_items, int32_t *out_col,
                       float *out_val, int32_t *kept, const int32_t *rows, const int32_t *n_rows,
                       int32_t *next, int32_t *n_next, cudaStream_t s) {
    const size_t smem = (sizeof(SortItem) + sizeof(int32_t)) * C * T;
    // Set on every launch: the attribute is per device, and a cached flag
    // would race between host threads running different engines.
    NCVIS_CUDA(cudaFuncSetAttribute(merge_tier<C, T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
    // All rows: one thread each; listed rows: a grid of resident blocks that
    // reads the list's length on the device.
    const int per_sm = (int)std::max<size_t>(1, (227 * 1024) / (smem + 1024));
    const int64_t grid = rows ? (int64_t)num_sms() * per_sm : ceil_div(N, T);
    NCVIS_LAUNCH((merge_tier<C, T>), grid, T, smem, s, N, k, inds, dists, in_off, in_key, g_items,
                 out_col, out_val, kept, rows, n_rows, next, n_next);
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
    w.n_tier = (int32_t *)p;   p += align256(2 * sizeof(int32_t));
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
           align256(2 * sizeof(int32_t)) +
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
    NCVIS_CUDA(cudaMemsetAsync(w.n_tier, 0, 2 * sizeof(int32_t), s));
    launch_merge_tier<kCap0, kThreads0>(N, k, inds, dists, w.in_off, w.in_key, w.items, w.out_col,
                                        w.out_val, w.kept, nullptr, nullptr, w.tier1, w.n_tier, s);
    launch_merge_tier<kCap1, kThreads1>(N, k, inds, dists, w.in_off, w.in_key, w.items, w.out_col,
                                        w.out_val, w.kept, w.tier1, w.n_tier, w.tier2,
                                        w.n_tier + 1, s);
    launch_merge_tier<kCap2, kThreads2>(N, k, inds, dists, w.in_off, w.in_key, w.items, w.out_col,
                                        w.out_val, w.kept, w.tier2, w.n_tier + 1, nullptr, nullptr,
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
