// K10: approximate kNN candidate selection by an inverted-file partition, for
// point counts where the exact O(N^2 D) selection of K2 stops being viable;
// and the exact selection's warm start, which orders the rows by the same
// k-means cells (end of this file).
// The reference's own kNN (hnswlib, src/ncvis.cpp:72-153) is approximate too;
// its result contract is kept: the candidates found here go through the same
// exact FP32 rerank (K4), so rows hold k+1 nearest-found points, the nearest
// dropped, descending exact distances.
//
//   1. k-means with C cells on the BF16 copies: C initial centroids are rows
//      drawn with Philox from the points; each pass assigns every point to its
//      nearest centroid with the tensor-core selection kernel (queries = the
//      points, candidates = the centroids) and moves each centroid to its
//      cell's mean (kept when the cell is empty; unit length for cosine and
//      correlation, whose points are unit length);
//   2. the points are counting-sorted by cell (within a cell the order is the
//      arrival order of the scatter's atomics) and their BF16 rows gathered
//      in that order;
//   3. each cell probes its own cell and the probe-1 cells whose centroids
//      are nearest to its centroid (more while the probed cells hold fewer
//      than R points); a work list gives every 256-row query tile of a cell
//      one item per probed cell, consecutive items extending one tile;
//   4. one launch of the selection kernel runs the work list over the sorted
//      rows and writes each point's R candidates in original numbering.
#include <algorithm>
#include <numeric>
#include <vector>

#include "common.cuh"
#include "rng.cuh"
#include "stages.cuh"

namespace ncvis_gpu {

namespace {

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Centroid c = row i of Xp, i drawn uniformly with Philox block (c, seed tag).
__global__ void ivf_init(const float *__restrict__ Xp, int64_t N, int D, int C, uint32_t k0,
                         uint32_t k1, float *__restrict__ cent) {
    const int lane = threadIdx.x & 31;
    const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (c >= C) return;
    const Philox4x32 r = philox4x32_10((uint32_t)c, 0x1f5u, 0u, 0x10000000u, k0, k1);
    const int64_t i = bounded_index(r.v[0], r.v[1], (uint32_t)N);
    for (int t = lane; t < D; t += 32) cent[(int64_t)c * D + t] = Xp[i * D + t];
}

// BF16 copies of the centroids in the layout of the points' copies (K1): Cq
// on the query side and Cc on the candidate side; with the folded squared-L2
// product Cq holds 1, 1 and Cc -|c|^2/2 (BF16 high and low part) in columns
// D, D+1, otherwise Cc is not written (the caller passes Cc == Cq).
__global__ void ivf_centroid_rows(const float *__restrict__ cent, int C, int D, int ldb, int fold,
                                  __nv_bfloat16 *__restrict__ Cq, __nv_bfloat16 *__restrict__ Cc) {
    const int lane = threadIdx.x & 31;
    const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (c >= C) return;
    float sq = 0.f;
    for (int t = lane; t < D; t += 32) {
        const float v = cent[(int64_t)c * D + t];
        sq += v * v;
        Cq[(int64_t)c * ldb + t] = __float2bfloat16_rn(v);
        if (fold) Cc[(int64_t)c * ldb + t] = __float2bfloat16_rn(v);
    }
    const int extra = fold ? 2 : 0;
    for (int t = D + extra + lane; t < ldb; t += 32) {
        Cq[(int64_t)c * ldb + t] = __float2bfloat16_rn(0.f);
        if (fold) Cc[(int64_t)c * ldb + t] = __float2bfloat16_rn(0.f);
    }
    sq = warp_sum(sq);
    if (fold && lane == 0) {
        const float h = -0.5f * sq;
        const __nv_bfloat16 hi = __float2bfloat16_rn(h);
        const __nv_bfloat16 lo = __float2bfloat16_rn(h - __bfloat162float(hi));
        Cq[(int64_t)c * ldb + D] = __float2bfloat16_rn(1.f);
        Cq[(int64_t)c * ldb + D + 1] = __float2bfloat16_rn(1.f);
        Cc[(int64_t)c * ldb + D] = hi;
        Cc[(int64_t)c * ldb + D + 1] = lo;
    }
}

// Cell sums and counts: point i belongs to cell cand[i * R] (its best).
__global__ void ivf_accumulate(const float *__restrict__ Xp, int64_t N, int D,
                               const int32_t *__restrict__ cand, int R, int C,
                               float *__restrict__ sums, int *__restrict__ counts) {
    const int lane = threadIdx.x & 31;
    const int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (i >= N) return;
    const int c = cand[i * R];
    if (c < 0 || c >= C) return;
    for (int t = lane; t < D; t += 32) atomicAdd(sums + (int64_t)c * D + t, Xp[i * D + t]);
    if (lane == 0) atomicAdd(counts + c, 1);
}

// Centroids to their cells' means (unit length when `normalise`), the sums
// and counts cleared for the next pass.
__global__ void ivf_update(float *__restrict__ cent, float *__restrict__ sums,
                           int *__restrict__ counts, int C, int D, int normalise) {
    const int lane = threadIdx.x & 31;
    const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (c >= C) return;
    const int n = counts[c];
    __syncwarp();
    if (n > 0) {
        float sq = 0.f;
        for (int t = lane; t < D; t += 32) {
            const float v = sums[(int64_t)c * D + t] / (float)n;
            sq += v * v;
        }
        sq = warp_sum(sq);
        const float scale = (normalise && sq > 0.f) ? 1.f / sqrtf(sq) : 1.f;
        for (int t = lane; t < D; t += 32)
            cent[(int64_t)c * D + t] = sums[(int64_t)c * D + t] / (float)n * scale;
    }
    for (int t = lane; t < D; t += 32) sums[(int64_t)c * D + t] = 0.f;
    __syncwarp();
    if (lane == 0) counts[c] = 0;
}

// The same with per-block sums in shared memory (C * D floats and C counts),
// flushed to the global sums once per block: same-cell updates meet in the
// SM instead of the L2.
__global__ void ivf_accumulate_shared(const float *__restrict__ Xp, int64_t N, int D,
                                      const int32_t *__restrict__ cand, int R, int C,
                                      float *__restrict__ sums, int *__restrict__ counts) {
    extern __shared__ float sh[];
    float *ssum = sh;
    int *scnt = reinterpret_cast<int *>(sh + (size_t)C * D);
    for (int t = threadIdx.x; t < C * D; t += blockDim.x) ssum[t] = 0.f;
    for (int t = threadIdx.x; t < C; t += blockDim.x) scnt[t] = 0;
    __syncthreads();
    const int warps = blockDim.x >> 5, lane = threadIdx.x & 31;
    // Rows of up to 128 columns: each lane's four values of the next row are
    // loaded while the current row's are added (the cell ordering of
    // 1,024,000 x 100: 4.55 -> 3.26 ms over its three passes).
    const int64_t step = (int64_t)gridDim.x * warps;
    int64_t i = (int64_t)blockIdx.x * warps + (threadIdx.x >> 5);
    float v[4];
    int c = -1;
    auto load = [&](int64_t r) {
        c = r < N ? cand[r * R] : -1;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int t = lane + 32 * u;
            v[u] = (r < N && t < D) ? Xp[r * D + t] : 0.f;
        }
    };
    load(i);
    for (; i < N; i += step) {
        const int cc = c;
        float w[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) w[u] = v[u];
        load(i + step);
        if (cc < 0 || cc >= C) continue;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int t = lane + 32 * u;
            if (t < D) atomicAdd(ssum + cc * D + t, w[u]);
        }
        if (lane == 0) atomicAdd(scnt + cc, 1);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < C * D; t += blockDim.x)
        if (ssum[t] != 0.f) atomicAdd(sums + t, ssum[t]);
    for (int t = threadIdx.x; t < C; t += blockDim.x)
        if (scnt[t]) atomicAdd(counts + t, scnt[t]);
}

__global__ void ivf_count(const int32_t *__restrict__ cand, int R, int64_t N, int C,
                          int *__restrict__ counts) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const int c = cand[i * R];
    if (c >= 0 && c < C) atomicAdd(counts + c, 1);
}

__global__ void ivf_scatter(const int32_t *__restrict__ cand, int R, int64_t N, int C,
                            const int64_t *__restrict__ starts, int *__restrict__ cursor,
                            int32_t *__restrict__ perm) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const int c = cand[i * R];
    if (c < 0 || c >= C) return;
    perm[starts[c] + atomicAdd(cursor + c, 1)] = (int32_t)i;
}

// dst[r] = src[perm[r]] for BF16 rows of ldb elements (ldb a multiple of 8).
__global__ void ivf_gather_rows(const __nv_bfloat16 *__restrict__ src,
                                const int32_t *__restrict__ perm, int64_t N, int ldb,
                                __nv_bfloat16 *__restrict__ dst) {
    const int per = ldb / 8;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N * per) return;
    const int64_t row = t / per;
    const int v = (int)(t % per);
    reinterpret_cast<uint4 *>(dst)[row * per + v] =
        reinterpret_cast<const uint4 *>(src)[(int64_t)perm[row] * per + v];
}

// Work list of `nq` query rows in tiles of 256 against candidates [0, nc),
// tiles dealt round-robin over at most num_sms() CTAs.
struct HostWork {
    std::vector<int64_t> begin;
    std::vector<TcItem> items;
    int ctas = 0;
};

HostWork all_pairs_work(int64_t nq, int64_t nc) {
    HostWork w;
    const int64_t tiles = (nq + 255) / 256;
    w.ctas = (int)std::min<int64_t>(tiles, num_sms());
    w.begin.assign(w.ctas + 1, 0);
    for (int b = 0; b < w.ctas; ++b) {
        for (int64_t t = b; t < tiles; t += w.ctas)
            w.items.push_back(TcItem{(int)(256 * t), (int)nq, 0, (int)nc, 0, 0, 0, 0});
        w.begin[b + 1] = (int64_t)w.items.size();
    }
    return w;
}

// Device buffers of one call: carved from the caller's workspace when one is
// given (256-byte aligned, bounded by its size), else stream-ordered
// allocations freed when the owner goes out of scope (on every exit path,
// errors included).
struct DeviceArena {
    cudaStream_t s;
    char *base = nullptr;
    size_t cap = 0, used = 0;
    std::vector<void *> ptrs;
    explicit DeviceArena(cudaStream_t st, void *workspace = nullptr, size_t bytes = 0)
        : s(st), base((char *)workspace), cap(bytes) {}
    DeviceArena(const DeviceArena &) = delete;
    DeviceArena &operator=(const DeviceArena &) = delete;
    ~DeviceArena() {
        for (void *p : ptrs) cudaFreeAsync(p, s);
    }
    template <typename T>
    T *alloc(size_t count) {
        const size_t bytes = (sizeof(T) * std::max<size_t>(count, 1) + 255) & ~(size_t)255;
        if (base) {
            require(used + bytes <= cap, "knn: workspace too small for the cell ordering",
                    kInternal);
            T *p = (T *)(base + used);
            used += bytes;
            return p;
        }
        void *p = nullptr;
        NCVIS_CUDA(cudaMallocAsync(&p, bytes, s));
        ptrs.push_back(p);
        return (T *)p;
    }
};

// Device copy of a work list, owned by `arena`.
TcWork upload(const HostWork &w, const int32_t *map, DeviceArena &arena) {
    int64_t *begin = arena.alloc<int64_t>(w.begin.size());
    TcItem *items = arena.alloc<TcItem>(w.items.size());
    NCVIS_CUDA(cudaMemcpyAsync(begin, w.begin.data(), sizeof(int64_t) * w.begin.size(),
                               cudaMemcpyHostToDevice, arena.s));
    if (!w.items.empty())
        NCVIS_CUDA(cudaMemcpyAsync(items, w.items.data(), sizeof(TcItem) * w.items.size(),
                                   cudaMemcpyHostToDevice, arena.s));
    return TcWork{w.ctas, begin, items, map};
}

void check_timeout(int *flag, cudaStream_t s) {
    int timeout = 0;
    NCVIS_CUDA(cudaMemcpyAsync(&timeout, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    NCVIS_CUDA(cudaStreamSynchronize(s));
    require(timeout == 0, "knn: the tensor-core kernel timed out waiting on a barrier",
            kDeviceTimeout);
}

// k-means cells of the points and the points sorted by cell.
struct Cells {
    int C = 0;
    __nv_bfloat16 *Cq = nullptr, *Cc = nullptr;  // centroid rows: query side, candidate side
    std::vector<int> counts;                     // points per cell (host)
    std::vector<int64_t> starts;                 // C + 1 offsets of the cells (host)
    int32_t *perm = nullptr;                     // sorted position -> original row
    __nv_bfloat16 *Xs = nullptr, *Xcs = nullptr;  // rows (and folded candidate rows) in cell order
};

// Step 1: `iters` k-means moves of C centroids (initial centroids: rows drawn
// with Philox from `seed`), each after an assignment by the tensor-core
// selection kernel, and a final assignment: point i's cell is cand[i * kAssignR].
// Centroids are unit length for cosine and correlation.
constexpr int kAssignR = 8;  // candidates kept per point by the cell assignment

void kmeans_cells(const float *Xp, const __nv_bfloat16 *Xb, int64_t N, int D,
                  const KnnTcPlan &tp, int dist, int C, int iters, uint64_t seed, int32_t *cand,
                  int *timeout_flag, cudaStream_t s, DeviceArena &arena, Cells &cells) {
    const bool fold = tp.fold;
    const int ldb = tp.ldb;
    cells.C = C;
    float *cent = arena.alloc<float>((size_t)C * D);
    float *sums = arena.alloc<float>((size_t)C * D);
    int *counts = arena.alloc<int>(C);
    cells.Cq = arena.alloc<__nv_bfloat16>((size_t)C * ldb);
    cells.Cc = fold ? arena.alloc<__nv_bfloat16>((size_t)C * ldb) : cells.Cq;
    uint32_t k0, k1;
    noise_key(seed ^ 0x1f51f51full, k0, k1);
    const unsigned warps_c = ceil_div((size_t)C, 8);
    NCVIS_LAUNCH(ivf_init, warps_c, 256, 0, s, Xp, N, D, C, k0, k1, cent);
    NCVIS_CUDA(cudaMemsetAsync(sums, 0, sizeof(float) * C * D, s));
    NCVIS_CUDA(cudaMemsetAsync(counts, 0, sizeof(int) * C, s));
    // The assignment needs each point's nearest centroid only: the selection
    // keeps 8 (its shortest list), entry 0 of each row is the cell.
    KnnTcPlan ap = tp;
    ap.R = kAssignR;
    const TcWork awork = upload(all_pairs_work(N, C), nullptr, arena);
    const int normalise = (dist == kCosine || dist == kCorrelation) ? 1 : 0;
    // Per-block sums in shared memory where C * D floats fit in 110 KB (two
    // blocks per SM), else straight into the global sums.
    const size_t acc_smem = sizeof(float) * (size_t)C * D + sizeof(int) * (size_t)C;
    const bool shared_acc = acc_smem <= 110 * 1024 && D <= 128;  // four values per lane
    if (shared_acc)
        NCVIS_CUDA(cudaFuncSetAttribute(ivf_accumulate_shared,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)acc_smem));
    for (int pass = 0;; ++pass) {
        NCVIS_LAUNCH(ivf_centroid_rows, warps_c, 256, 0, s, cent, C, D, ldb, fold ? 1 : 0,
                     cells.Cq, fold ? cells.Cc : cells.Cq);
        launch_knn_select_tc_pair(Xb, N, cells.Cc, C, nullptr, ap, true, cand, timeout_flag, s,
                                  awork);
        if (pass == iters) break;
        if (shared_acc)
            NCVIS_LAUNCH(ivf_accumulate_shared, (unsigned)(2 * num_sms()), 512, acc_smem, s, Xp,
                         N, D, cand, kAssignR, C, sums, counts);
        else
            NCVIS_LAUNCH(ivf_accumulate, (unsigned)ceil_div((size_t)N, 8), 256, 0, s, Xp, N, D,
                         cand, kAssignR, C, sums, counts);
        NCVIS_LAUNCH(ivf_update, warps_c, 256, 0, s, cent, sums, counts, C, D, normalise);
    }
}

// Step 2: counting sort of the points by cell (within a cell, the order in
// which the scatter's atomics arrive) and their BF16 rows gathered in that
// order; waits on the stream for the cell sizes.
void sort_by_cell(const __nv_bfloat16 *Xb, const __nv_bfloat16 *Xc, int64_t N, int ldb,
                  const int32_t *cand, int *timeout_flag, cudaStream_t s, DeviceArena &arena,
                  Cells &cells) {
    const int C = cells.C;
    int *counts = arena.alloc<int>(C);
    int *cursor = arena.alloc<int>(C);
    int64_t *d_starts = arena.alloc<int64_t>((size_t)C + 1);
    cells.perm = arena.alloc<int32_t>((size_t)N);
    cells.Xs = arena.alloc<__nv_bfloat16>((size_t)N * ldb);
    cells.Xcs = Xc ? arena.alloc<__nv_bfloat16>((size_t)N * ldb) : nullptr;
    NCVIS_CUDA(cudaMemsetAsync(counts, 0, sizeof(int) * C, s));
    NCVIS_LAUNCH(ivf_count, (unsigned)ceil_div((size_t)N, 256), 256, 0, s, cand, kAssignR, N, C,
                 counts);
    cells.counts.assign(C, 0);
    NCVIS_CUDA(cudaMemcpyAsync(cells.counts.data(), counts, sizeof(int) * C,
                               cudaMemcpyDeviceToHost, s));
    NCVIS_CUDA(cudaStreamSynchronize(s));
    check_timeout(timeout_flag, s);
    cells.starts.assign(C + 1, 0);
    for (int c = 0; c < C; ++c) cells.starts[c + 1] = cells.starts[c] + cells.counts[c];
    require(cells.starts[C] == N, "knn: a point was not assigned to a cell", kInternal);
    NCVIS_CUDA(cudaMemcpyAsync(d_starts, cells.starts.data(), sizeof(int64_t) * (C + 1),
                               cudaMemcpyHostToDevice, s));
    NCVIS_CUDA(cudaMemsetAsync(cursor, 0, sizeof(int) * C, s));
    NCVIS_LAUNCH(ivf_scatter, (unsigned)ceil_div((size_t)N, 256), 256, 0, s, cand, kAssignR, N, C,
                 d_starts, cursor, cells.perm);
    const size_t vec = (size_t)N * (ldb / 8);
    NCVIS_LAUNCH(ivf_gather_rows, (unsigned)ceil_div(vec, 256), 256, 0, s, Xb, cells.perm, N, ldb,
                 cells.Xs);
    if (Xc)
        NCVIS_LAUNCH(ivf_gather_rows, (unsigned)ceil_div(vec, 256), 256, 0, s, Xc, cells.perm, N,
                     ldb, cells.Xcs);
}

}  // namespace

IvfPlan plan_ivf(int64_t N, int lists, int probe) {
    IvfPlan p;
    int64_t c = lists > 0 ? lists : N / 512;
    c = std::max<int64_t>(1, std::min<int64_t>({c, N, 65536}));
    p.C = (int)c;
    p.probe = std::max(1, std::min(probe > 0 ? probe : 32, std::min(p.C, 64)));
    p.iters = 4;
    return p;
}

void run_knn_ivf(const float *Xp, const __nv_bfloat16 *Xb, const __nv_bfloat16 *Xc, int64_t N,
                 int D, const KnnTcPlan &tp, int dist, const IvfPlan &ip, uint64_t seed,
                 int32_t *cand_i, int *timeout_flag, cudaStream_t s) {
    require(tp.fold || dist != kSquaredL2,
            "knn (ivf): squared L2 needs D <= 126 (the folded-norm product)", kUnsupported);
    require(N < (int64_t(1) << 31), "knn (ivf): N must be below 2^31");
    const bool fold = tp.fold;
    const int C = ip.C;
    const int Rp = ip.probe > 32 ? 64 : 32;  // nearest cells listed per cell
    DeviceArena arena(s);
    Cells cells;
    // 1. k-means.
    kmeans_cells(Xp, Xb, N, D, tp, dist, C, ip.iters, seed, cand_i, timeout_flag, s, arena, cells);

    // Nearest cells of each cell (its own first for the spaces where a
    // centroid is its own best match; the work list adds it where not).
    int32_t *pcand = arena.alloc<int32_t>((size_t)C * Rp);
    KnnTcPlan pp = tp;
    pp.R = Rp;
    launch_knn_select_tc_pair(cells.Cq, C, cells.Cc, C, nullptr, pp, true, pcand, timeout_flag, s,
                              upload(all_pairs_work(C, C), nullptr, arena));

    // 2. Counting sort by cell.
    sort_by_cell(Xb, fold ? Xc : nullptr, N, tp.ldb, cand_i, timeout_flag, s, arena, cells);
    std::vector<int32_t> h_pcand((size_t)C * Rp);
    NCVIS_CUDA(cudaMemcpyAsync(h_pcand.data(), pcand, sizeof(int32_t) * C * Rp,
                               cudaMemcpyDeviceToHost, s));
    NCVIS_CUDA(cudaStreamSynchronize(s));
    const std::vector<int> &h_counts = cells.counts;
    const std::vector<int64_t> &starts = cells.starts;

    // 3. Work list: every 256-row query tile of a cell, one item per probed cell.
    struct Tile {
        int64_t cost;
        std::vector<TcItem> items;
    };
    std::vector<Tile> tiles;
    std::vector<char> taken(C, 0);
    for (int c = 0; c < C; ++c) {
        if (h_counts[c] == 0) continue;
        std::vector<int> probes{c};
        taken[c] = 1;
        int64_t have = h_counts[c];
        auto add = [&](int p) {
            if (p < 0 || p >= C || taken[p] || h_counts[p] == 0) return;
            probes.push_back(p);
            taken[p] = 1;
            have += h_counts[p];
        };
        for (int j = 0; j < Rp && (int)probes.size() < ip.probe; ++j) add(h_pcand[(size_t)c * Rp + j]);
        for (int j = 0; j < Rp && have < tp.R; ++j) add(h_pcand[(size_t)c * Rp + j]);
        for (int p = 0; p < C && have < tp.R; ++p) add(p);
        for (int p : probes) taken[p] = 0;
        int64_t cost = 0;
        for (int p : probes) cost += (h_counts[p] + 127) / 128 + 1;
        const int64_t a = starts[c], n = h_counts[c];
        for (int64_t t = 0; t * 256 < n; ++t) {
            Tile tile{cost, {}};
            for (size_t idx = 0; idx < probes.size(); ++idx) {
                const int p = probes[idx];
                int flags = 0;
                if (idx > 0) flags |= kTcContinue;
                if (idx + 1 < probes.size()) flags |= kTcMore;
                tile.items.push_back(TcItem{(int)(a + 256 * t), (int)(a + n), (int)starts[p],
                                            (int)(starts[p] + h_counts[p]), 0, flags, 0, 0});
            }
            tiles.push_back(std::move(tile));
        }
    }
    std::stable_sort(tiles.begin(), tiles.end(),
                     [](const Tile &x, const Tile &y) { return x.cost > y.cost; });
    HostWork sw;
    sw.ctas = (int)std::min<int64_t>((int64_t)tiles.size(), num_sms());
    std::vector<std::vector<const Tile *>> per(sw.ctas);
    std::vector<int64_t> load(sw.ctas, 0);
    for (const Tile &t : tiles) {
        const int b = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        per[b].push_back(&t);
        load[b] += t.cost;
    }
    sw.begin.assign(sw.ctas + 1, 0);
    for (int b = 0; b < sw.ctas; ++b) {
        for (const Tile *t : per[b]) sw.items.insert(sw.items.end(), t->items.begin(), t->items.end());
        sw.begin[b + 1] = (int64_t)sw.items.size();
    }

    // 4. The search over the sorted rows, written in original numbering.
    launch_knn_select_tc_pair(cells.Xs, N, fold ? cells.Xcs : cells.Xs, N, nullptr, tp, true,
                              cand_i, timeout_flag, s, upload(sw, cells.perm, arena));
    check_timeout(timeout_flag, s);
}

// ---- warm start of the exact selection ---------------------------------------
// The exact search keeps each point's best R candidates in a sorted list and
// inserts a candidate only when it beats the list's worst; with the rows in
// the caller's order the lists tighten slowly (a sweep over N random
// candidates inserts ~R ln(N/R) of them per point), and every insertion costs
// the selection kernel a divergent append path.  Here the rows are ordered by
// k-means cell and every 256-row query tile sweeps the candidates starting at
// its own cell (then on to the end and around from row 0): every candidate
// tile is still scanned exactly once, so the result is the exact search's
// (the same candidate sets, up to exact score ties at the R-th place), but
// each point meets its own cell first and its list is nearly final after it.
// Consecutive query tiles go to consecutive CTAs, so the CTAs running at one
// time start at nearby rows and share their candidate tiles in the L2.

KnnOrderPlan plan_knn_order(int64_t N, int D, const KnnTcPlan &tp, int dist, int cells) {
    KnnOrderPlan p;
    if (cells < 0) return p;
    // The folded squared-L2 product or an inner-product space (the
    // assignment ranks centroids by the product); D > 126 squared L2 keeps
    // the caller's order.
    if (!(tp.fold || dist != kSquaredL2) || N < kKnnOrderMinRows) return p;
    int64_t c = cells > 0 ? cells : N / 4096;
    c = std::max<int64_t>(16, std::min<int64_t>({c, N / 256, 4096}));
    p.C = (int)c;
    p.iters = 3;
    (void)D;
    return p;
}

size_t knn_order_workspace_bytes(int64_t N, int D, const KnnTcPlan &tp, const KnnOrderPlan &op) {
    if (op.C <= 0) return 0;
    auto a = [](size_t b) { return (std::max<size_t>(b, 1) + 255) & ~(size_t)255; };
    const size_t C = (size_t)op.C, ldb = (size_t)tp.ldb, n = (size_t)N;
    const size_t tiles = (n + 255) / 256, ctas = 1024;  // work-list bounds (ctas <= SMs)
    size_t b = 0;
    // kmeans_cells: centroids, sums, counts, centroid rows, the assignment work list.
    b += 2 * a(sizeof(float) * C * D) + a(sizeof(int) * C) + 2 * a(2 * C * ldb);
    b += a(sizeof(int64_t) * (ctas + 1)) + a(sizeof(TcItem) * tiles);
    // sort_by_cell: counts, cursors, starts, permutation, sorted rows.
    b += 2 * a(sizeof(int) * C) + a(sizeof(int64_t) * (C + 1)) + a(sizeof(int32_t) * n);
    b += 2 * a(2 * n * ldb);
    // the sweep's work list.
    b += a(sizeof(int64_t) * (ctas + 1)) + a(sizeof(TcItem) * 2 * tiles);
    return b;
}

void run_knn_tc_ordered(const float *Xp, const __nv_bfloat16 *Xb, const __nv_bfloat16 *Xc,
                        int64_t N, int D, const KnnTcPlan &tp, int dist, const KnnOrderPlan &op,
                        uint64_t seed, int32_t *cand_i, int *timeout_flag, cudaStream_t s,
                        void *workspace, size_t workspace_bytes, cudaEvent_t sweep_start,
                        const int32_t **cell_order) {
    require(op.C > 0, "knn: ordered search without cells", kInternal);
    require(N < (int64_t(1) << 31), "knn: N must be below 2^31");
    require(num_sms() <= 1024, "knn: more SMs than the ordered search's work list allows",
            kUnsupported);
    const bool fold = tp.fold;
    DeviceArena arena(s, workspace, workspace_bytes);
    Cells cells;
    kmeans_cells(Xp, Xb, N, D, tp, dist, op.C, op.iters, seed, cand_i, timeout_flag, s, arena,
                 cells);
    sort_by_cell(Xb, fold ? Xc : nullptr, N, tp.ldb, cand_i, timeout_flag, s, arena, cells);

    // Work list: query tile t of the sorted rows against [s0, N) then [0, s0),
    // s0 = its first row's cell start rounded down to a candidate tile; tile t
    // goes to CTA t mod ctas.
    const int64_t tiles = (N + 255) / 256;
    HostWork w;
    w.ctas = (int)std::min<int64_t>(tiles, num_sms());
    std::vector<std::vector<TcItem>> per(w.ctas);
    int c = 0;
    for (int64_t t = 0; t < tiles; ++t) {
        const int64_t r0 = 256 * t;
        while (cells.starts[c + 1] <= r0) ++c;
        const int64_t s0 = cells.starts[c] / 128 * 128;
        std::vector<TcItem> &v = per[t % w.ctas];
        if (s0 == 0) {
            v.push_back(TcItem{(int)r0, (int)N, 0, (int)N, 0, 0, 0, 0});
        } else {
            v.push_back(TcItem{(int)r0, (int)N, (int)s0, (int)N, 0, kTcMore, 0, 0});
            v.push_back(TcItem{(int)r0, (int)N, 0, (int)s0, 0, kTcContinue, 0, 0});
        }
    }
    w.begin.assign(w.ctas + 1, 0);
    for (int b = 0; b < w.ctas; ++b) {
        w.items.insert(w.items.end(), per[b].begin(), per[b].end());
        w.begin[b + 1] = (int64_t)w.items.size();
    }
    const TcWork sweep = upload(w, cells.perm, arena);
    if (sweep_start) NCVIS_CUDA(cudaEventRecord(sweep_start, s));
    launch_knn_select_tc_pair(cells.Xs, N, fold ? cells.Xcs : cells.Xs, N, nullptr, tp, true,
                              cand_i, timeout_flag, s, sweep);
    check_timeout(timeout_flag, s);
    // The rows in cell order (sorted position -> row), for the caller's
    // rerank; only from a caller's workspace, which outlives this call.
    if (cell_order) *cell_order = workspace ? cells.perm : nullptr;
}

}  // namespace ncvis_gpu
