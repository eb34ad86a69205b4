// The engine behind the C ABI (include/ncvis_gb300.h): parameter handling of
// ncvis::NCVis (src/ncvis.cpp:12-21), the fit_transform pipeline
// (src/ncvis.cpp:354-459) over the device stages, a growable device arena,
// stage timing with CUDA events, and the handle-less stage entry points.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/ncvis_gb300.h"
#include "common.cuh"
#include "stages.cuh"

namespace ncvis_gpu {

std::atomic<uint64_t> &launch_counter() {
    static std::atomic<uint64_t> counter{0};
    return counter;
}

namespace {

thread_local std::string g_last_error;

inline size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

// Bump layout over one device allocation.
struct Layout {
    size_t total = 0;
    size_t take(size_t bytes) {
        size_t off = total;
        total += align256(bytes);
        return off;
    }
};

struct Events {
    cudaEvent_t ev[10] = {};
    Events() {
        for (auto &e : ev) {
            const cudaError_t r = cudaEventCreate(&e);
            if (r != cudaSuccess) {
                destroy();
                NCVIS_CUDA(r);
            }
        }
    }
    Events(const Events &) = delete;
    Events &operator=(const Events &) = delete;
    ~Events() { destroy(); }
    void destroy() {
        for (auto &e : ev)
            if (e) {
                cudaEventDestroy(e);
                e = nullptr;
            }
    }
    float ms(int a, int b) const {
        float t = 0.f;
        cudaEventElapsedTime(&t, ev[a], ev[b]);
        return t;
    }
};

}  // namespace

void record_error(const char *msg) { g_last_error = msg; }

// Picks, per problem signature, the fastest of a few candidate settings by
// timing one run of each with CUDA events; results are cached per engine and,
// when NCVIS_AUTOTUNE_CACHE names a file, kept there as "key value" lines.
struct Autotuner {
    std::map<std::string, int> best;
    bool loaded = false;

    static const char *cache_path() { return std::getenv("NCVIS_AUTOTUNE_CACHE"); }

    void load() {
        loaded = true;
        const char *path = cache_path();
        if (!path) return;
        std::ifstream in(path);
        std::string key;
        int value;
        while (in >> key >> value) best[key] = value;
    }

    void save() const {
        const char *path = cache_path();
        if (!path) return;
        std::ofstream out(path);
        for (const auto &kv : best) out << kv.first << " " << kv.second << "\n";
    }

    template <class Run>
    int pick(const std::string &key, const std::vector<int> &candidates, Run run, cudaStream_t s) {
        if (!loaded) load();
        auto it = best.find(key);
        if (it != best.end()) return it->second;
        EventPair t;
        int choice = candidates.front();
        float best_ms = 1e30f;
        for (int c : candidates) {
            NCVIS_CUDA(cudaEventRecord(t.a, s));
            run(c);
            NCVIS_CUDA(cudaEventRecord(t.b, s));
            NCVIS_CUDA(cudaEventSynchronize(t.b));
            const float ms = t.ms();
            if (ms < best_ms) best_ms = ms, choice = c;
        }
        best[key] = choice;
        save();
        return choice;
    }
};

namespace {

// eoff[p] = row_ptr[off[p]] for p in [0, B].
__global__ void gather_offsets(const int64_t *__restrict__ row_ptr,
                               const int64_t *__restrict__ off, int B, int64_t *__restrict__ eoff) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p <= B) eoff[p] = row_ptr[off[p]];
}

// Copies each problem's BF16 rows and squared norms to its 256-aligned place
// in the padded layout (problem p starts at row pad[p]); one warp per row.
__global__ void pad_rows(const __nv_bfloat16 *__restrict__ Xb, const float *__restrict__ sqn,
                         const int64_t *__restrict__ off, const int64_t *__restrict__ pad, int B,
                         int64_t total, int ldb, __nv_bfloat16 *__restrict__ Xb_pad,
                         float *__restrict__ sqn_pad) {
    const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= total) return;
    const int p = segment_of(off, B, row);
    const int64_t prow = pad[p] + (row - off[p]);
    const uint16_t *src = reinterpret_cast<const uint16_t *>(Xb + row * ldb);
    uint16_t *dst = reinterpret_cast<uint16_t *>(Xb_pad + prow * ldb);
    for (int c = lane; c < ldb; c += 32) dst[c] = src[c];
    if (lane == 0) sqn_pad[prow] = sqn[row];
}

}  // namespace

}  // namespace ncvis_gpu

using namespace ncvis_gpu;

// Whether the current device reads pageable host memory coherently
// (cudaDevAttrPageableMemoryAccess), cached per device.
static bool reads_pageable_host_memory() {
    static std::mutex mu;
    static std::map<int, bool> known;
    int dev = 0;
    NCVIS_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    auto it = known.find(dev);
    if (it != known.end()) return it->second;
    int v = 0;
    NCVIS_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev));
    return known[dev] = (v != 0);
}

// Query tiles of the problems for one tensor-core launch, spread over `ctas`
// CTAs by longest processing time first (a tile's cost is its problem's
// number of candidate tiles), and the problems' 256-aligned row offsets.
struct BatchedTcWork {
    std::vector<int64_t> pad;     // B + 1 padded row offsets
    std::vector<int64_t> begin;   // ctas + 1
    std::vector<TcItem> items;
    int ctas = 0;
};

static BatchedTcWork plan_batched_tc(const std::vector<int64_t> &off, int ctas_max) {
    const size_t B = off.size() - 1;
    BatchedTcWork w;
    w.pad.resize(B + 1);
    w.pad[0] = 0;
    struct Tile {
        int64_t cost;
        TcItem item;
    };
    std::vector<Tile> tiles;
    for (size_t p = 0; p < B; ++p) {
        const int64_t n = off[p + 1] - off[p];
        w.pad[p + 1] = w.pad[p] + (n + 255) / 256 * 256;
        const int64_t cost = (n + 127) / 128;
        for (int64_t t = 0; t * 256 < n; ++t)
            tiles.push_back({cost, TcItem{(int)(w.pad[p] + 256 * t), (int)(w.pad[p] + n),
                                          (int)w.pad[p], (int)(w.pad[p] + n),
                                          (int)(off[p] - w.pad[p]), 0, 0, 0}});
    }
    std::stable_sort(tiles.begin(), tiles.end(),
                     [](const Tile &a, const Tile &b) { return a.cost > b.cost; });
    w.ctas = (int)std::min<int64_t>((int64_t)tiles.size(), ctas_max);
    std::vector<std::vector<TcItem>> per(w.ctas);
    std::vector<int64_t> load(w.ctas, 0);
    for (const Tile &t : tiles) {
        const int c = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        per[c].push_back(t.item);
        load[c] += t.cost;
    }
    w.begin.assign(w.ctas + 1, 0);
    for (int c = 0; c < w.ctas; ++c) {
        w.begin[c + 1] = w.begin[c] + (int64_t)per[c].size();
        w.items.insert(w.items.end(), per[c].begin(), per[c].end());
    }
    return w;
}

struct ncvis_engine {
    ncvis_params p{};
    std::vector<size_t> noise;
    ncvis_options o{};
    std::vector<int32_t> replay_stream;  // host copy of the recorded noise stream
    std::string err;
    ncvis_stage_times times{};
    cudaStream_t own = nullptr;
    void *arena = nullptr;
    size_t arena_bytes = 0;

    // The engine's own stream is created on first use, so that constructing
    // an engine touches no GPU (as constructing the reference's NCVis only
    // stores parameters, src/ncvis.cpp:12-21).
    cudaStream_t stream() {
        if (o.stream) return (cudaStream_t)o.stream;
        if (!own) NCVIS_CUDA(cudaStreamCreateWithFlags(&own, cudaStreamNonBlocking));
        return own;
    }

    ~ncvis_engine() {
        if (arena) cudaFree(arena);
        if (own) cudaStreamDestroy(own);
    }

    char *ensure_arena(size_t bytes) {
        if (bytes > arena_bytes) {
            // A caller-set limit fails the fit as the allocation itself would.
            if (o.arena_limit && bytes > o.arena_limit)
                throw Error(kCudaError, "CUDA error out of memory: the device arena needs " +
                                            std::to_string(bytes) + " bytes, above arena_limit " +
                                            std::to_string(o.arena_limit));
            if (arena) {
                NCVIS_CUDA(cudaStreamSynchronize(stream()));
                NCVIS_CUDA(cudaFree(arena));
                arena = nullptr;
                arena_bytes = 0;
            }
            NCVIS_CUDA(cudaMalloc(&arena, bytes));
            arena_bytes = bytes;
        }
        return (char *)arena;
    }

    void fit(const float *X, size_t N, size_t D, float *Y, bool host);
    void fit_batched(const float *dX, size_t D, const int64_t *offsets, size_t B,
                     const uint64_t *seeds, float *dY);
    Autotuner tuner;
};

namespace {

// Checked when the engine is created: what the reference's constructor
// itself cannot accept (it allocates n_epochs entries, src/ncvis.cpp:16).
// Noise samples per edge and epoch: the kernels hold the sample number in
// 32-bit loop counters and Philox counter words (below 2^29 for the
// unstaged stream), and E * sum(n_noise) must fit 64 bits.  The reference
// loops over any value; a value above this bound is refused.
constexpr size_t kMaxNoise = size_t(1) << 24;

void check_noise(const size_t *n_noise, int begin, int end, const std::string &prefix) {
    if (!n_noise) return;
    for (int e = begin; e < end; ++e)
        require(n_noise[e] <= kMaxNoise,
                prefix + "n_noise entries must be at most " + std::to_string(kMaxNoise) +
                    " (epoch " + std::to_string(e) + ": " + std::to_string(n_noise[e]) + ")");
}

// The options struct as a C caller may fill it: unknown modes and negative
// counts are refused rather than falling back to a default path.
int knn_mode(int precision) { return precision & ~NCVIS_KNN_CALLER_ORDER; }

void check_options(const ncvis_options &o) {
    const int mode = knn_mode(o.knn_precision);
    require(mode == NCVIS_KNN_FP32 || mode == NCVIS_KNN_BF16_RERANK || mode == NCVIS_KNN_IVF,
            "[ncvis] options: knn_precision must be NCVIS_KNN_FP32, NCVIS_KNN_BF16_RERANK or "
            "NCVIS_KNN_IVF (optionally with the flag NCVIS_KNN_CALLER_ORDER)");
    require(o.wait_limit_cycles >= 0, "[ncvis] options: wait_limit_cycles must be non-negative");
    require(o.knn_order_cells >= 0, "[ncvis] options: knn_order_cells must be non-negative");
    require(o.sgd_mode == NCVIS_SGD_HOGWILD || o.sgd_mode == NCVIS_SGD_REPLAY ||
                o.sgd_mode == NCVIS_SGD_HOGWILD_UNSTAGED,
            "[ncvis] options: sgd_mode must be NCVIS_SGD_HOGWILD, NCVIS_SGD_REPLAY or "
            "NCVIS_SGD_HOGWILD_UNSTAGED");
    require(o.rerank_factor >= 0 && o.sgd_chains >= 0 && o.ivf_lists >= 0 && o.ivf_probe >= 0,
            "[ncvis] options: rerank_factor, sgd_chains, ivf_lists and ivf_probe must be "
            "non-negative");
    require(o.replay_len == 0 || o.replay_stream != nullptr,
            "[ncvis] options: replay_len > 0 needs a replay_stream");
}

void check_params(const ncvis_params &p) {
    require(p.n_epochs >= 0, "[ncvis] n_epochs must be non-negative");
    check_noise(p.n_noise, 0, p.n_epochs, "[ncvis] ");
}

template <class F>
int guarded(ncvis_engine *h, F &&f) {
    try {
        f();
        if (h) h->err.clear();
        return NCVIS_OK;
    } catch (const Error &e) {
        if (h) h->err = e.what();
        g_last_error = e.what();
        return e.code;
    } catch (const std::exception &e) {
        if (h) h->err = e.what();
        g_last_error = e.what();
        return NCVIS_INTERNAL;
    }
}

}  // namespace

void ncvis_engine::fit(const float *X, size_t N, size_t D, float *Y, bool host) {
    if (N == 0 || D == 0)
        throw Error(kInvalidArgument,
                    "[ncvis::NCVis::fit_transform] Dataset should have at least one element.");
    if (Y == nullptr)
        throw Error(kInvalidArgument,
                    "[ncvis::NCVis::fit_transform] Null pointer provided for output.");
    require(X != nullptr, "[ncvis::NCVis::fit_transform] Null pointer provided for input.");
    // The reference rejects an unknown distance when it builds the index
    // (src/ncvis.cpp:89-90).
    require(p.distance >= 0 && p.distance <= 3,
            "[ncvis::NCVis::buildKNN] Unrecognized distance type.");
    require(p.d >= 1 && p.d <= 32, "[ncvis] embedding dimension d must be in [1, 32]");
    require(p.n_init_epochs >= 0, "[ncvis] n_init_epochs must be non-negative");
    require(N >= 2, "[ncvis::NCVis::fit_transform] Dataset should have at least two elements.");
    require(N < (size_t(1) << 31) && D < (size_t(1) << 31), "[ncvis] N and D must be below 2^31");
    // Number of neighbours cannot exceed the number of other points
    // (src/ncvis.cpp:381-382).
    size_t kk = (p.n_neighbors < N - 1) ? p.n_neighbors : (N - 1);
    kk = (kk > 0) ? kk : 1;
    require(kk <= 255, "[ncvis] n_neighbors above 255 is not supported");
    const int k = (int)kk;
    const int d = (int)p.d;
    const int dist = p.distance;
    const bool ivf = (knn_mode(o.knn_precision) == NCVIS_KNN_IVF);
    const bool bf16 = (knn_mode(o.knn_precision) == NCVIS_KNN_BF16_RERANK) || ivf;
    require((int64_t)N * k < (int64_t(1) << 30), "[ncvis] N * n_neighbors must be below 2^30");
    require(host || ((uintptr_t)Y & (p.d == 4 ? 15 : 7)) == 0,
            "[ncvis] device Y must be 8-byte aligned (16-byte for d = 4)");
    const bool replay = (o.sgd_mode == NCVIS_SGD_REPLAY);

    cudaStream_t s = stream();
    KnnPlan kp = plan_knn_f32((int64_t)N, k, o.rerank_factor);
    KnnTcPlan tp = plan_knn_tc((int64_t)N, (int)D, k, o.rerank_factor, dist);
    tp.wait_cycles = o.wait_limit_cycles;
    tp.stall = o.inject_stall != 0;
    if (bf16)
        require(knn_tc_supported((int)D, tp.R),
                "[ncvis] the BF16 tensor-core kNN supports D <= 128", kUnsupported);
    const bool fold = bf16 && tp.fold;
    const int C = bf16 ? tp.R : kp.C();
    const int64_t nk = (int64_t)N * k;
    // The exact BF16 search with the rows ordered by k-means cell (warm start).
    const KnnOrderPlan op =
        (bf16 && !ivf)
            ? plan_knn_order((int64_t)N, (int)D, tp, dist,
                             (o.knn_precision & NCVIS_KNN_CALLER_ORDER) ? -1 : o.knn_order_cells)
            : KnnOrderPlan();
    const int chains = o.sgd_chains > 0 ? o.sgd_chains : 0;  // 0: sized once E is known

    Layout L;
    // Host X is read in place by the preprocessing kernel where the device
    // reads pageable host memory coherently (e.g. through the host's page
    // tables); elsewhere it is first copied to the device.
    const bool read_host = host && reads_pageable_host_memory();
    const size_t o_X = (host && !read_host) ? L.take(sizeof(float) * N * D) : 0;
    const size_t o_Y = host ? L.take(sizeof(float) * N * d) : 0;
    const size_t o_Xp = L.take(sizeof(float) * N * D);
    const size_t o_sqn = L.take(sizeof(float) * N);
    const size_t o_flag = L.take(sizeof(int) * 4);
    const size_t o_Xb = bf16 ? L.take(sizeof(__nv_bfloat16) * N * tp.ldb) : 0;
    const size_t o_Xc = fold ? L.take(sizeof(__nv_bfloat16) * N * tp.ldb) : 0;
    const size_t o_ci = L.take(sizeof(int32_t) * N * C);
    const size_t o_cd = L.take(sizeof(float) * N * C);
    const size_t o_ki = L.take(sizeof(int32_t) * nk);
    const size_t o_kd = L.take(sizeof(float) * nk);
    const size_t o_rp = L.take(sizeof(int64_t) * (N + 1));
    const size_t o_cols = L.take(sizeof(int32_t) * 2 * nk);
    const size_t o_vals = L.take(sizeof(float) * 2 * nk);
    const size_t o_src = L.take(sizeof(int32_t) * 2 * nk);
    const size_t o_Q = L.take(sizeof(float) * 4);
    const size_t o_sym = L.take(symmetrize_workspace_bytes((int64_t)N, k));
    const size_t o_init = L.take(init_workspace_bytes((int64_t)N, d));
    const size_t o_sgd = L.take(sgd_workspace_bytes(chains));
    const size_t o_stream = replay ? L.take(sizeof(int32_t) * std::max<size_t>(o.replay_len, 1)) : 0;
    const size_t ord_bytes = knn_order_workspace_bytes((int64_t)N, (int)D, tp, op);
    const size_t o_ord = ord_bytes ? L.take(ord_bytes) : 0;
    char *base = ensure_arena(L.total);

    const float *dX = (host && !read_host) ? (float *)(base + o_X) : X;
    float *dY = host ? (float *)(base + o_Y) : Y;
    float *Xp = (float *)(base + o_Xp);
    float *sqn = (float *)(base + o_sqn);
    int *flag = (int *)(base + o_flag);
    __nv_bfloat16 *Xb = bf16 ? (__nv_bfloat16 *)(base + o_Xb) : nullptr;
    __nv_bfloat16 *Xc = fold ? (__nv_bfloat16 *)(base + o_Xc) : nullptr;
    int32_t *cand_i = (int32_t *)(base + o_ci);
    float *cand_d = (float *)(base + o_cd);
    int32_t *knn_i = (int32_t *)(base + o_ki);
    float *knn_d = (float *)(base + o_kd);
    int64_t *row_ptr = (int64_t *)(base + o_rp);
    int32_t *cols = (int32_t *)(base + o_cols);
    float *vals = (float *)(base + o_vals);
    int32_t *src = (int32_t *)(base + o_src);
    float *dQ = (float *)(base + o_Q);

    Events ev;
    StageRanges nv;
    nv.next("ncvis.h2d");
    NCVIS_CUDA(cudaEventRecord(ev.ev[0], s));
    if (host && !read_host)
        NCVIS_CUDA(cudaMemcpyAsync((void *)dX, X, sizeof(float) * N * D, cudaMemcpyHostToDevice, s));
    NCVIS_CUDA(cudaEventRecord(ev.ev[1], s));
    nv.next("ncvis.preprocess");
    NCVIS_CUDA(cudaMemsetAsync(flag, 0, sizeof(int) * 4, s));
    launch_preprocess(dX, (int64_t)N, (int)D, dist, Xp, sqn, Xb, bf16 ? tp.ldb : 0, flag, s, Xc);
    NCVIS_CUDA(cudaEventRecord(ev.ev[2], s));
    {
        int bad = 0;
        NCVIS_CUDA(cudaMemcpyAsync(&bad, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
        NCVIS_CUDA(cudaStreamSynchronize(s));
        require(bad == 0, "[ncvis] input contains non-finite values");
    }
    nv.next("ncvis.knn");
    const int32_t *cell_order = nullptr;  // rows in k-means cell order (ordered sweep only)
    NCVIS_CUDA(cudaMemsetAsync(knn_i, 0xff, sizeof(int32_t) * nk, s));
    if (ivf)
        run_knn_ivf(Xp, Xb, Xc, (int64_t)N, (int)D, tp, dist,
                    plan_ivf((int64_t)N, o.ivf_lists, o.ivf_probe), (uint64_t)p.random_seed,
                    cand_i, flag + 2, s);
    else if (op.C > 0)
        run_knn_tc_ordered(Xp, Xb, Xc, (int64_t)N, (int)D, tp, dist, op, (uint64_t)p.random_seed,
                           cand_i, flag + 2, s, base + o_ord, ord_bytes, ev.ev[9], &cell_order);
    else if (bf16)
        launch_knn_select_tc(Xb, sqn, (int64_t)N, tp, dist, cand_i, cand_d, flag + 2, s, nullptr,
                             Xc);
    else
        launch_knn_select_f32(Xp, sqn, (int64_t)N, (int)D, dist, kp, cand_i, cand_d, s);
    NCVIS_CUDA(cudaEventRecord(ev.ev[3], s));
    nv.next("ncvis.rerank");
    launch_rerank(Xp, (int64_t)N, (int)D, dist, cand_i, C, k, knn_i, knn_d, s, cell_order);
    NCVIS_CUDA(cudaEventRecord(ev.ev[4], s));
    nv.next("ncvis.symmetrize");
    if (bf16) {
        int timeout = 0;
        NCVIS_CUDA(cudaMemcpyAsync(&timeout, flag + 2, sizeof(int), cudaMemcpyDeviceToHost, s));
        NCVIS_CUDA(cudaStreamSynchronize(s));
        require(timeout == 0, "[ncvis] the tensor-core kNN kernel timed out waiting on a barrier",
                kDeviceTimeout);
    }
    const int64_t E = run_symmetrize((int64_t)N, k, knn_i, knn_d, base + o_sym, row_ptr, cols, vals,
                                     src, s);
    NCVIS_CUDA(cudaEventRecord(ev.ev[5], s));

    nv.next("ncvis.init");
    const float init_alpha = (float)(1. / k);
    run_init_embedding((int64_t)N, d, row_ptr, cols, (uint64_t)p.random_seed, p.n_init_epochs,
                       init_alpha, dY, base + o_init, s, o.init_sequential_stats != 0);
    NCVIS_CUDA(cudaEventRecord(ev.ev[6], s));
    nv.next("ncvis.optimize");

    NCVIS_CUDA(cudaMemsetAsync(dQ, 0, sizeof(float), s));
    SgdArgs g;
    g.N = (int64_t)N;
    g.d = d;
    g.E = E;
    g.src = src;
    g.dst = cols;
    g.Y = dY;
    g.Q = dQ;
    g.seed = (uint64_t)p.random_seed;
    g.n_epochs = p.n_epochs;
    g.a = p.a;
    g.b = p.b;
    g.alpha = p.alpha;
    g.alpha_Q = p.alpha_Q;
    if (replay) {
        size_t need = 0;
        for (int e = 0; e < p.n_epochs; ++e) need += (size_t)E * noise[e];
        require(replay_stream.size() >= need,
                "[ncvis] replay stream shorter than E * sum(n_noise) = " + std::to_string(need));
        int32_t *dstream = (int32_t *)(base + o_stream);
        if (need)
            NCVIS_CUDA(cudaMemcpyAsync(dstream, replay_stream.data(), sizeof(int32_t) * need,
                                       cudaMemcpyHostToDevice, s));
        int *err = flag + 1;
        size_t pos = 0;
        for (int e = 0; e < p.n_epochs; ++e) {
            launch_sgd_replay(g, e, noise[e], 0, E, dstream, (int64_t)pos, err, s);
            pos += (size_t)E * noise[e];
        }
        int rerr = 0;
        NCVIS_CUDA(cudaMemcpyAsync(&rerr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
        NCVIS_CUDA(cudaStreamSynchronize(s));
        require(rerr == 0, "[ncvis] replay stream holds an index outside [0, N)");
    } else if (p.n_epochs > 0 && E > 0) {
        if (o.sgd_mode == NCVIS_SGD_HOGWILD && sgd_window_applies(g.N, g.d))
            run_sgd_window(g, 0, p.n_epochs, noise.data(), chains, 0, base + o_sgd, s);
        else
            run_sgd_hogwild(g, 0, p.n_epochs, noise.data(), chains, base + o_sgd, s);
    }
    NCVIS_CUDA(cudaEventRecord(ev.ev[7], s));
    nv.next("ncvis.d2h");
    if (host)
        NCVIS_CUDA(cudaMemcpyAsync(Y, dY, sizeof(float) * N * d, cudaMemcpyDeviceToHost, s));
    NCVIS_CUDA(cudaEventRecord(ev.ev[8], s));
    nv.close();
    NCVIS_CUDA(cudaEventSynchronize(ev.ev[8]));

    times.h2d_ms = ev.ms(0, 1);
    times.preprocess_ms = ev.ms(1, 2);
    times.knn_ms = ev.ms(2, 3);
    times.rerank_ms = ev.ms(3, 4);
    times.symmetrize_ms = ev.ms(4, 5);
    times.build_edges_ms = 0.f;  // fused into the CSR compaction
    times.init_ms = ev.ms(5, 6);
    times.optimize_ms = ev.ms(6, 7);
    times.d2h_ms = ev.ms(7, 8);
    times.total_ms = ev.ms(0, 8);
    times.n_edges = E;
    times.k = k;
    times.knn_order_ms = op.C > 0 ? ev.ms(2, 9) : 0.f;
}

void ncvis_engine::fit_batched(const float *dX, size_t D, const int64_t *offsets, size_t B,
                               const uint64_t *seeds, float *dY) {
    require(dX && dY && offsets && B >= 1, "[ncvis] batched: null pointer or no problems");
    require(B < (size_t(1) << 20), "[ncvis] batched: too many problems");
    require(offsets[0] == 0, "[ncvis] batched: offsets[0] must be 0");
    int64_t min_n = INT64_MAX;
    for (size_t q = 0; q < B; ++q) {
        const int64_t n = offsets[q + 1] - offsets[q];
        require(n >= 2, "[ncvis] batched: every problem needs at least two points");
        min_n = std::min(min_n, n);
    }
    const int64_t total = offsets[B];
    require(D >= 1 && total < (int64_t(1) << 31), "[ncvis] batched: need D >= 1 and total N < 2^31");
    require(p.distance >= 0 && p.distance <= 3,
            "[ncvis::NCVis::buildKNN] Unrecognized distance type.");
    require(p.d >= 1 && p.d <= 4, "[ncvis] batched: embedding dimension d must be in [1, 4]");
    require(o.sgd_mode != NCVIS_SGD_REPLAY,
            "[ncvis] batched: the replay mode (one recorded noise stream per fit) is not available "
            "for batched problems");
    // Batched problems are small: the IVF mode runs the exact BF16 search here.
    const bool bf16 = (knn_mode(o.knn_precision) == NCVIS_KNN_BF16_RERANK ||
                       knn_mode(o.knn_precision) == NCVIS_KNN_IVF);
    require(((uintptr_t)dY & 7) == 0, "[ncvis] device Y must be 8-byte aligned");
    // k is clamped by the smallest problem (src/ncvis.cpp:381-382 per problem).
    int64_t kk = std::min<int64_t>((int64_t)p.n_neighbors, min_n - 1);
    kk = std::max<int64_t>(kk, 1);
    require(kk <= 255, "[ncvis] n_neighbors above 255 is not supported");
    const int k = (int)kk, d = (int)p.d, dist = p.distance;
    const int64_t nk = total * k;
    require(nk < (int64_t(1) << 30), "[ncvis] batched: total N * n_neighbors must be below 2^30");
    cudaStream_t s = stream();

    // Host-side layout of the problems.
    const int qt = knn_f32_query_tile(), it = init_tile_rows();
    std::vector<int64_t> h_off(offsets, offsets + B + 1), h_tq(B + 1), h_ti(B + 1);
    std::vector<uint64_t> h_seed(B);
    h_tq[0] = h_ti[0] = 0;
    for (size_t q = 0; q < B; ++q) {
        const int64_t n = h_off[q + 1] - h_off[q];
        h_tq[q + 1] = h_tq[q] + (n + qt - 1) / qt;
        h_ti[q + 1] = h_ti[q] + (n + it - 1) / it;
        h_seed[q] = seeds ? seeds[q] : (uint64_t)p.random_seed;
    }
    KnnPlan kp;
    kp.R = (int)std::min<int64_t>(std::min<int64_t>(
        std::max<int64_t>((int64_t)(o.rerank_factor > 0 ? o.rerank_factor : 2) * k, k + 1), min_n), 256);
    kp.splits = 1;
    while (h_tq[B] * kp.splits < 2 * num_sms() && kp.splits * 2 * kp.R <= 1024 &&
           min_n / (kp.splits * 2) >= 64)
        kp.splits *= 2;
    KnnTcPlan tp = plan_knn_tc(total, (int)D, k, o.rerank_factor, dist);
    tp.wait_cycles = o.wait_limit_cycles;
    tp.stall = o.inject_stall != 0;
    const bool fold = bf16 && tp.fold;
    BatchedTcWork tw;
    if (bf16) {
        require(knn_tc_supported((int)D, tp.R),
                "[ncvis] the BF16 tensor-core kNN supports D <= 128", kUnsupported);
        tw = plan_batched_tc(h_off, num_sms());
        require(tw.pad[B] < (int64_t(1) << 31), "[ncvis] batched: too many rows");
    }
    const int C = bf16 ? tp.R : kp.C();
    const int64_t max_chains = std::max<int64_t>(sgd_batched_resident_chains(d), (int64_t)B);

    Layout L;
    const size_t o_Xp = L.take(sizeof(float) * total * D);
    const size_t o_sqn = L.take(sizeof(float) * total);
    const size_t o_flag = L.take(sizeof(int) * 4);
    const size_t o_ci = L.take(sizeof(int32_t) * total * C);
    const size_t o_cd = L.take(sizeof(float) * total * C);
    const size_t o_ki = L.take(sizeof(int32_t) * nk);
    const size_t o_kd = L.take(sizeof(float) * nk);
    const size_t o_rp = L.take(sizeof(int64_t) * (total + 1));
    const size_t o_cols = L.take(sizeof(int32_t) * 2 * nk);
    const size_t o_vals = L.take(sizeof(float) * 2 * nk);
    const size_t o_src = L.take(sizeof(int32_t) * 2 * nk);
    const size_t o_sym = L.take(symmetrize_workspace_bytes(total, k));
    const size_t o_init = L.take(init_batched_workspace_bytes(total, h_ti[B], (int)B, d));
    const size_t o_off = L.take(sizeof(int64_t) * (B + 1));
    const size_t o_tq = L.take(sizeof(int64_t) * (B + 1));
    const size_t o_ti = L.take(sizeof(int64_t) * (B + 1));
    const size_t o_eoff = L.take(sizeof(int64_t) * (B + 1));
    const size_t o_cp = L.take(sizeof(int64_t) * (B + 1));
    const size_t o_bp = L.take(sizeof(int64_t) * (B + 1));
    const size_t o_seed = L.take(sizeof(uint64_t) * B);
    const size_t o_Qs = L.take(sizeof(float) * B);
    const size_t o_cq = L.take(sizeof(float) * max_chains);
    const size_t o_Yt = L.take(sizeof(float) * total * d);
    const size_t o_Qt = L.take(sizeof(float) * B);
    const int64_t total_pad = bf16 ? tw.pad[B] : 0;
    const size_t o_Xb = bf16 ? L.take(sizeof(__nv_bfloat16) * total * tp.ldb) : 0;
    const size_t o_Xbp = bf16 ? L.take(sizeof(__nv_bfloat16) * total_pad * tp.ldb) : 0;
    const size_t o_Xc = fold ? L.take(sizeof(__nv_bfloat16) * total * tp.ldb) : 0;
    const size_t o_Xcp = fold ? L.take(sizeof(__nv_bfloat16) * total_pad * tp.ldb) : 0;
    const size_t o_sqp = bf16 ? L.take(sizeof(float) * total_pad) : 0;
    const size_t o_pad = bf16 ? L.take(sizeof(int64_t) * (B + 1)) : 0;
    const size_t o_wb = bf16 ? L.take(sizeof(int64_t) * (tw.ctas + 1)) : 0;
    const size_t o_wi = bf16 ? L.take(sizeof(TcItem) * std::max<size_t>(tw.items.size(), 1)) : 0;
    char *base = ensure_arena(L.total);
    float *Xp = (float *)(base + o_Xp);
    float *sqn = (float *)(base + o_sqn);
    int *flag = (int *)(base + o_flag);
    int32_t *cand_i = (int32_t *)(base + o_ci);
    float *cand_d = (float *)(base + o_cd);
    int32_t *knn_i = (int32_t *)(base + o_ki);
    float *knn_d = (float *)(base + o_kd);
    int64_t *row_ptr = (int64_t *)(base + o_rp);
    int32_t *cols = (int32_t *)(base + o_cols);
    float *vals = (float *)(base + o_vals);
    int32_t *src = (int32_t *)(base + o_src);
    int64_t *d_off = (int64_t *)(base + o_off), *d_tq = (int64_t *)(base + o_tq);
    int64_t *d_ti = (int64_t *)(base + o_ti), *d_eoff = (int64_t *)(base + o_eoff);
    int64_t *d_cp = (int64_t *)(base + o_cp);
    int64_t *d_bp = (int64_t *)(base + o_bp);
    uint64_t *d_seed = (uint64_t *)(base + o_seed);
    float *Qs = (float *)(base + o_Qs), *chain_q = (float *)(base + o_cq);
    float *Ytune = (float *)(base + o_Yt), *Qtune = (float *)(base + o_Qt);

    Events ev;
    StageRanges nv;
    nv.next("ncvis.batched.h2d");
    NCVIS_CUDA(cudaEventRecord(ev.ev[0], s));
    NCVIS_CUDA(cudaMemcpyAsync(d_off, h_off.data(), sizeof(int64_t) * (B + 1), cudaMemcpyHostToDevice, s));
    NCVIS_CUDA(cudaMemcpyAsync(d_tq, h_tq.data(), sizeof(int64_t) * (B + 1), cudaMemcpyHostToDevice, s));
    NCVIS_CUDA(cudaMemcpyAsync(d_ti, h_ti.data(), sizeof(int64_t) * (B + 1), cudaMemcpyHostToDevice, s));
    NCVIS_CUDA(cudaMemcpyAsync(d_seed, h_seed.data(), sizeof(uint64_t) * B, cudaMemcpyHostToDevice, s));
    NCVIS_CUDA(cudaEventRecord(ev.ev[1], s));
    nv.next("ncvis.batched.preprocess");
    NCVIS_CUDA(cudaMemsetAsync(flag, 0, sizeof(int) * 4, s));
    __nv_bfloat16 *Xb = bf16 ? (__nv_bfloat16 *)(base + o_Xb) : nullptr;
    __nv_bfloat16 *Xc = fold ? (__nv_bfloat16 *)(base + o_Xc) : nullptr;
    launch_preprocess(dX, total, (int)D, dist, Xp, sqn, Xb, bf16 ? tp.ldb : 0, flag, s, Xc);
    NCVIS_CUDA(cudaEventRecord(ev.ev[2], s));
    {
        int bad = 0;
        NCVIS_CUDA(cudaMemcpyAsync(&bad, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
        NCVIS_CUDA(cudaStreamSynchronize(s));
        require(bad == 0, "[ncvis] input contains non-finite values");
    }
    nv.next("ncvis.batched.knn");
    NCVIS_CUDA(cudaMemsetAsync(knn_i, 0xff, sizeof(int32_t) * nk, s));
    if (bf16) {
        // Problems at 256-aligned rows of a padded copy; one tensor-core launch
        // over every problem's query tiles, each against its own rows.
        __nv_bfloat16 *Xb_pad = (__nv_bfloat16 *)(base + o_Xbp);
        float *sqn_pad = (float *)(base + o_sqp);
        int64_t *d_pad = (int64_t *)(base + o_pad), *d_wb = (int64_t *)(base + o_wb);
        TcItem *d_wi = (TcItem *)(base + o_wi);
        NCVIS_CUDA(cudaMemcpyAsync(d_pad, tw.pad.data(), sizeof(int64_t) * (B + 1),
                                   cudaMemcpyHostToDevice, s));
        NCVIS_CUDA(cudaMemcpyAsync(d_wb, tw.begin.data(), sizeof(int64_t) * (tw.ctas + 1),
                                   cudaMemcpyHostToDevice, s));
        NCVIS_CUDA(cudaMemcpyAsync(d_wi, tw.items.data(), sizeof(TcItem) * tw.items.size(),
                                   cudaMemcpyHostToDevice, s));
        NCVIS_CUDA(cudaMemsetAsync(Xb_pad, 0, sizeof(__nv_bfloat16) * total_pad * tp.ldb, s));
        NCVIS_CUDA(cudaMemsetAsync(sqn_pad, 0, sizeof(float) * total_pad, s));
        NCVIS_LAUNCH(pad_rows, (unsigned)ceil_div(total * 32, 256), 256, 0, s, Xb, sqn, d_off,
                     d_pad, (int)B, total, tp.ldb, Xb_pad, sqn_pad);
        __nv_bfloat16 *Xc_pad = nullptr;
        if (fold) {
            Xc_pad = (__nv_bfloat16 *)(base + o_Xcp);
            NCVIS_CUDA(cudaMemsetAsync(Xc_pad, 0, sizeof(__nv_bfloat16) * total_pad * tp.ldb, s));
            NCVIS_LAUNCH(pad_rows, (unsigned)ceil_div(total * 32, 256), 256, 0, s, Xc, sqn, d_off,
                         d_pad, (int)B, total, tp.ldb, Xc_pad, sqn_pad);
        }
        TcWork work{tw.ctas, d_wb, d_wi, nullptr};
        launch_knn_select_tc(Xb_pad, sqn_pad, total_pad, tp, dist, cand_i, cand_d, flag + 2, s,
                             &work, Xc_pad);
        int timeout = 0;
        NCVIS_CUDA(cudaMemcpyAsync(&timeout, flag + 2, sizeof(int), cudaMemcpyDeviceToHost, s));
        NCVIS_CUDA(cudaStreamSynchronize(s));
        require(timeout == 0, "[ncvis] kNN: the tensor-core kernel timed out waiting on a barrier",
                kDeviceTimeout);
    } else {
        Segments seg;
        seg.offsets = d_off;
        seg.tile_prefix = d_tq;
        seg.B = (int)B;
        seg.n_tiles = h_tq[B];
        launch_knn_select_f32(Xp, sqn, total, (int)D, dist, kp, cand_i, cand_d, s, seg);
    }
    NCVIS_CUDA(cudaEventRecord(ev.ev[3], s));
    nv.next("ncvis.batched.rerank");
    launch_rerank(Xp, total, (int)D, dist, cand_i, C, k, knn_i, knn_d, s);
    NCVIS_CUDA(cudaEventRecord(ev.ev[4], s));
    nv.next("ncvis.batched.symmetrize");
    const int64_t E = run_symmetrize(total, k, knn_i, knn_d, base + o_sym, row_ptr, cols, vals, src, s);
    NCVIS_CUDA(cudaEventRecord(ev.ev[5], s));

    // Edge ranges per problem, then chains per problem in proportion to edges.
    NCVIS_LAUNCH(gather_offsets, ceil_div(B + 1, 256), 256, 0, s, row_ptr, d_off, (int)B, d_eoff);
    std::vector<int64_t> h_eoff(B + 1);
    NCVIS_CUDA(cudaMemcpyAsync(h_eoff.data(), d_eoff, sizeof(int64_t) * (B + 1),
                               cudaMemcpyDeviceToHost, s));
    NCVIS_CUDA(cudaStreamSynchronize(s));
    auto chain_layout = [&](int edges_per_chain, std::vector<int64_t> &cp) {
        const int64_t target = std::min<int64_t>(max_chains, std::max<int64_t>(E / edges_per_chain, (int64_t)B));
        cp.assign(B + 1, 0);
        for (size_t q = 0; q < B; ++q) {
            const int64_t Ep = h_eoff[q + 1] - h_eoff[q];
            int64_t c = (int64_t)((double)target * (double)Ep / (double)std::max<int64_t>(E, 1));
            const int64_t Np = h_off[q + 1] - h_off[q];
            c = std::max<int64_t>(1, std::min<int64_t>(c, std::max<int64_t>(Ep / 16, 1)));
            c = std::min<int64_t>(c, std::max<int64_t>(Np / 8, 1));
            cp[q + 1] = cp[q] + c;
        }
        return cp[B];
    };

    nv.next("ncvis.batched.init");
    const float init_alpha = (float)(1. / k);
    run_init_embedding_batched(total, d, d_off, d_ti, (int)B, h_ti[B], d_seed, row_ptr, cols,
                               p.n_init_epochs, init_alpha, dY, base + o_init, s);
    NCVIS_CUDA(cudaEventRecord(ev.ev[6], s));
    nv.next("ncvis.batched.optimize");

    SgdBatch g{};
    g.d = d;
    g.B = (int)B;
    g.src = src;
    g.dst = cols;
    g.off = d_off;
    g.eoff = d_eoff;
    g.cp = d_cp;
    g.chain_q = chain_q;
    g.seed = (uint64_t)p.random_seed;
    g.a = p.a;
    g.b = p.b;
    g.alpha = p.alpha;
    g.alpha_Q = p.alpha_Q;
    std::vector<int64_t> h_cp, h_bp;
    // Noise staged in shared memory (d <= 4, the default Hogwild mode): every
    // block of chains within one problem.
    const bool staged = d <= 4 && o.sgd_mode == NCVIS_SGD_HOGWILD;
    int64_t n_blocks = 0;
    int block_chains = 128;
    // A shape: edges per chain (high 16 bits) and, staged, chains per block.
    auto set_layout = [&](int shape) {
        g.n_chains = chain_layout(shape >> 16, h_cp);
        block_chains = shape & 0xffff;
        const int64_t T = block_chains;
        h_bp.assign(B + 1, 0);
        for (size_t q = 0; q < B; ++q) h_bp[q + 1] = h_bp[q] + (h_cp[q + 1] - h_cp[q] + T - 1) / T;
        n_blocks = h_bp[B];
        NCVIS_CUDA(cudaMemcpyAsync(d_cp, h_cp.data(), sizeof(int64_t) * (B + 1),
                                   cudaMemcpyHostToDevice, s));
        NCVIS_CUDA(cudaMemcpyAsync(d_bp, h_bp.data(), sizeof(int64_t) * (B + 1),
                                   cudaMemcpyHostToDevice, s));
    };
    auto run_epochs = [&](const SgdBatch &t, const size_t *plan, cudaStream_t st) {
        if (staged)
            run_sgd_window_batched(t, d_bp, n_blocks, block_chains, plan, st);
        else
            run_sgd_hogwild_batched(t, plan, st);
    };
    if (p.n_epochs > 0 && E > 0) {
        // Autotune the shape on a scratch copy of the embedding (one epoch
        // each): edges per chain (16..128) and, with staged noise, chains per
        // block (64, 128, 256: more chains share a window's copy-in and
        // write-back, fewer leave more blocks for small problems).
        const std::string key = std::string(staged ? "sgd_batched_staged_shape" : "sgd_batched") +
                                " d=" + std::to_string(d) + " B=" + std::to_string(B) +
                                " E~2^" + std::to_string((int)std::log2((double)std::max<int64_t>(E, 1)));
        std::vector<int> shapes;
        for (int epc : {16, 32, 64, 128})
            for (int t : {64, 128, 256})
                if (staged || t == 128) shapes.push_back(epc << 16 | t);
        const int chosen = tuner.pick(key, shapes, [&](int shape) {
            set_layout(shape);
            NCVIS_CUDA(cudaMemcpyAsync(Ytune, dY, sizeof(float) * total * d, cudaMemcpyDeviceToDevice, s));
            NCVIS_CUDA(cudaMemsetAsync(Qtune, 0, sizeof(float) * B, s));
            SgdBatch t = g;
            t.Y = Ytune;
            t.Qs = Qtune;
            t.n_epochs = 1;
            run_epochs(t, noise.data() + (p.n_epochs - 1), s);
        }, s);
        set_layout(chosen);
        NCVIS_CUDA(cudaMemsetAsync(Qs, 0, sizeof(float) * B, s));
        g.Y = dY;
        g.Qs = Qs;
        g.n_epochs = p.n_epochs;
        // The whole epoch loop as one CUDA graph, launched once; the capture
        // stream, graph and executable graph are released on every exit path.
        struct Captured {
            cudaStream_t cs = nullptr;
            cudaGraph_t graph = nullptr;
            cudaGraphExec_t exec = nullptr;
            ~Captured() {
                if (exec) cudaGraphExecDestroy(exec);
                if (graph) cudaGraphDestroy(graph);
                if (cs) cudaStreamDestroy(cs);
            }
        } cap;
        NCVIS_CUDA(cudaStreamCreateWithFlags(&cap.cs, cudaStreamNonBlocking));
        NCVIS_CUDA(cudaStreamBeginCapture(cap.cs, cudaStreamCaptureModeThreadLocal));
        try {
            run_epochs(g, noise.data(), cap.cs);
        } catch (...) {
            cudaStreamEndCapture(cap.cs, &cap.graph);
            throw;
        }
        NCVIS_CUDA(cudaStreamEndCapture(cap.cs, &cap.graph));
        NCVIS_CUDA(cudaGraphInstantiate(&cap.exec, cap.graph, 0));
        NCVIS_CUDA(cudaEventRecord(ev.ev[9], s));
        NCVIS_CUDA(cudaGraphLaunch(cap.exec, s));
        NCVIS_CUDA(cudaEventRecord(ev.ev[7], s));
        NCVIS_CUDA(cudaEventSynchronize(ev.ev[7]));
    } else {
        NCVIS_CUDA(cudaEventRecord(ev.ev[9], s));
        NCVIS_CUDA(cudaEventRecord(ev.ev[7], s));
    }
    NCVIS_CUDA(cudaEventRecord(ev.ev[8], s));
    nv.close();
    NCVIS_CUDA(cudaEventSynchronize(ev.ev[8]));
    times.h2d_ms = ev.ms(0, 1);
    times.preprocess_ms = ev.ms(1, 2);
    times.knn_ms = ev.ms(2, 3);
    times.rerank_ms = ev.ms(3, 4);
    times.symmetrize_ms = ev.ms(4, 5);
    times.build_edges_ms = 0.f;
    times.init_ms = ev.ms(5, 6);
    times.optimize_ms = ev.ms(9, 7);
    times.d2h_ms = 0.f;
    times.total_ms = ev.ms(0, 8);
    times.n_edges = E;
    times.k = k;
    times.knn_order_ms = 0.f;
}

// ------------------------------------------------------------------------ C ABI

extern "C" {

ncvis_handle ncvis_create(const ncvis_params *params, const ncvis_options *options) {
    ncvis_engine *h = nullptr;
    int rc = guarded(nullptr, [&] {
        require(params != nullptr, "[ncvis] null parameters");
        check_params(*params);
        std::unique_ptr<ncvis_engine> e(new ncvis_engine());
        e->p = *params;
        // n_noise is copied; nullptr means 3 noise samples per epoch
        // (src/ncvis.cpp:16-20).
        e->noise.resize((size_t)params->n_epochs);
        for (int i = 0; i < params->n_epochs; ++i)
            e->noise[i] = params->n_noise ? params->n_noise[i] : 3;
        e->p.n_noise = nullptr;
        if (options) {
            check_options(*options);
            e->o = *options;
            if (options->replay_stream && options->replay_len)
                e->replay_stream.assign(options->replay_stream, options->replay_stream + options->replay_len);
            e->o.replay_stream = nullptr;
        }
        h = e.release();
    });
    return rc == NCVIS_OK ? h : nullptr;
}

void ncvis_destroy(ncvis_handle h) { delete h; }

int ncvis_set_options(ncvis_handle h, const ncvis_options *options) {
    if (!h) return NCVIS_INVALID_ARGUMENT;
    return guarded(h, [&] {
        require(options != nullptr, "[ncvis] null options");
        check_options(*options);
        h->o = *options;
        h->replay_stream.clear();
        if (options->replay_stream && options->replay_len)
            h->replay_stream.assign(options->replay_stream, options->replay_stream + options->replay_len);
        h->o.replay_stream = nullptr;
    });
}

int ncvis_fit_transform(ncvis_handle h, const float *X, size_t N, size_t D, float *Y) {
    if (!h) return NCVIS_INVALID_ARGUMENT;
    return guarded(h, [&] { h->fit(X, N, D, Y, true); });
}

int ncvis_fit_transform_device(ncvis_handle h, const float *dX, size_t N, size_t D, float *dY) {
    if (!h) return NCVIS_INVALID_ARGUMENT;
    return guarded(h, [&] { h->fit(dX, N, D, dY, false); });
}

int ncvis_fit_transform_batched_device(ncvis_handle h, const float *dX, size_t D,
                                       const int64_t *offsets, size_t n_problems,
                                       const uint64_t *seeds, float *dY) {
    if (!h) return NCVIS_INVALID_ARGUMENT;
    return guarded(h, [&] { h->fit_batched(dX, D, offsets, n_problems, seeds, dY); });
}

const char *ncvis_last_error(ncvis_handle h) { return h ? h->err.c_str() : "null handle"; }

const char *ncvis_get_last_error(void) { return g_last_error.c_str(); }

int ncvis_get_stage_times(ncvis_handle h, ncvis_stage_times *out) {
    if (!h || !out) return NCVIS_INVALID_ARGUMENT;
    *out = h->times;
    return NCVIS_OK;
}

namespace {

void knn_device(const float *dX, size_t N, size_t D, int distance, size_t k, int precision,
                int rerank_factor, int lists, int probe, int32_t *d_inds, float *d_dists,
                void *stream) {
    {
        require(dX && d_inds && d_dists, "knn: null pointer");
        require(N >= 2 && k >= 1 && k <= N - 1 && k <= 255, "knn: need 2 <= N and 1 <= k <= min(N-1, 255)");
        require(D >= 1 && N < (size_t(1) << 31) && N * k < (size_t(1) << 30),
                "knn: need D >= 1, N < 2^31 and N * k < 2^30");
        require(distance >= 0 && distance <= 3, "[ncvis::NCVis::buildKNN] Unrecognized distance type.");
        const int mode = knn_mode(precision);
        require(mode == NCVIS_KNN_FP32 || mode == NCVIS_KNN_BF16_RERANK || mode == NCVIS_KNN_IVF,
                "knn: unknown precision mode");
        const bool ivf = (mode == NCVIS_KNN_IVF);
        const bool bf16 = (mode == NCVIS_KNN_BF16_RERANK) || ivf;
        cudaStream_t s = (cudaStream_t)stream;
        KnnPlan kp = plan_knn_f32((int64_t)N, (int)k, rerank_factor);
        KnnTcPlan tp = plan_knn_tc((int64_t)N, (int)D, (int)k, rerank_factor, distance);
        const bool fold = bf16 && tp.fold;
        if (bf16)
            require(knn_tc_supported((int)D, tp.R),
                    "knn: the BF16 tensor-core kNN supports D <= 128", kUnsupported);
        const int C = bf16 ? tp.R : kp.C();
        const KnnOrderPlan op = (bf16 && !ivf) ? plan_knn_order((int64_t)N, (int)D, tp, distance,
                                                                (precision & NCVIS_KNN_CALLER_ORDER)
                                                                    ? -1
                                                                    : 0)
                                               : KnnOrderPlan();
        const size_t ord_bytes = knn_order_workspace_bytes((int64_t)N, (int)D, tp, op);
        Layout L;
        const size_t o_Xp = L.take(sizeof(float) * N * D);
        const size_t o_sqn = L.take(sizeof(float) * N);
        const size_t o_flag = L.take(sizeof(int) * 2);
        const size_t o_ci = L.take(sizeof(int32_t) * N * C);
        const size_t o_cd = L.take(sizeof(float) * N * C);
        const size_t o_Xb = bf16 ? L.take(sizeof(__nv_bfloat16) * N * tp.ldb) : 0;
        const size_t o_Xc = fold ? L.take(sizeof(__nv_bfloat16) * N * tp.ldb) : 0;
        const size_t o_ord = ord_bytes ? L.take(ord_bytes) : 0;
        StreamBuffer buf(L.total, s);
        char *base = (char *)buf.p;
        NCVIS_CUDA(cudaMemsetAsync(base + o_flag, 0, sizeof(int) * 2, s));
        __nv_bfloat16 *Xb = bf16 ? (__nv_bfloat16 *)(base + o_Xb) : nullptr;
        __nv_bfloat16 *Xc = fold ? (__nv_bfloat16 *)(base + o_Xc) : nullptr;
        launch_preprocess(dX, (int64_t)N, (int)D, distance, (float *)(base + o_Xp),
                          (float *)(base + o_sqn), Xb, bf16 ? tp.ldb : 0, (int *)(base + o_flag),
                          s, Xc);
        int bad = 0;
        NCVIS_CUDA(cudaMemcpyAsync(&bad, base + o_flag, sizeof(int), cudaMemcpyDeviceToHost, s));
        NCVIS_CUDA(cudaStreamSynchronize(s));
        require(!bad, "knn: input contains non-finite values");
        NCVIS_CUDA(cudaMemsetAsync(d_inds, 0xff, sizeof(int32_t) * N * k, s));
        const int32_t *cell_order = nullptr;
        if (ivf) {
            run_knn_ivf((float *)(base + o_Xp), Xb, Xc, (int64_t)N, (int)D, tp, distance,
                        plan_ivf((int64_t)N, lists, probe), 42, (int32_t *)(base + o_ci),
                        (int *)(base + o_flag) + 1, s);
        } else if (op.C > 0) {
            run_knn_tc_ordered((float *)(base + o_Xp), Xb, Xc, (int64_t)N, (int)D, tp, distance,
                               op, 42, (int32_t *)(base + o_ci), (int *)(base + o_flag) + 1, s,
                               base + o_ord, ord_bytes, nullptr, &cell_order);
        } else if (bf16) {
            launch_knn_select_tc(Xb, (float *)(base + o_sqn), (int64_t)N, tp, distance,
                                 (int32_t *)(base + o_ci), (float *)(base + o_cd),
                                 (int *)(base + o_flag) + 1, s, nullptr, Xc);
            int timeout = 0;
            NCVIS_CUDA(cudaMemcpyAsync(&timeout, (int *)(base + o_flag) + 1, sizeof(int),
                                       cudaMemcpyDeviceToHost, s));
            NCVIS_CUDA(cudaStreamSynchronize(s));
            require(!timeout, "knn: the tensor-core kernel timed out waiting on a barrier",
                    kDeviceTimeout);
        } else {
            launch_knn_select_f32((float *)(base + o_Xp), (float *)(base + o_sqn), (int64_t)N,
                                  (int)D, distance, kp, (int32_t *)(base + o_ci),
                                  (float *)(base + o_cd), s);
        }
        launch_rerank((float *)(base + o_Xp), (int64_t)N, (int)D, distance,
                      (int32_t *)(base + o_ci), C, (int)k, d_inds, d_dists, s, cell_order);
    }
}

}  // namespace

int ncvis_knn_device(const float *dX, size_t N, size_t D, int distance, size_t k, int precision,
                     int rerank_factor, int32_t *d_inds, float *d_dists, void *stream) {
    return guarded(nullptr, [&] {
        knn_device(dX, N, D, distance, k, precision, rerank_factor, 0, 0, d_inds, d_dists, stream);
    });
}

int ncvis_knn_ivf_device(const float *dX, size_t N, size_t D, int distance, size_t k,
                         int rerank_factor, int lists, int probe, int32_t *d_inds,
                         float *d_dists, void *stream) {
    return guarded(nullptr, [&] {
        require(lists >= 0 && probe >= 0, "knn (ivf): lists and probe must be non-negative");
        knn_device(dX, N, D, distance, k, NCVIS_KNN_IVF, rerank_factor, lists, probe, d_inds,
                   d_dists, stream);
    });
}

int ncvis_symmetrize_device(size_t N, size_t k, const int32_t *d_inds, const float *d_dists,
                            int64_t *d_row_ptr, int32_t *d_cols, float *d_vals, int32_t *d_src,
                            size_t *n_edges, void *stream) {
    return guarded(nullptr, [&] {
        require(d_inds && d_dists && d_row_ptr && d_cols && d_vals && n_edges,
                "symmetrize: null pointer");
        require(N >= 1 && k >= 1, "symmetrize: empty table");
        cudaStream_t s = (cudaStream_t)stream;
        StreamBuffer ws(symmetrize_workspace_bytes((int64_t)N, (int)k), s);
        const int64_t E = run_symmetrize((int64_t)N, (int)k, d_inds, d_dists, ws.p, d_row_ptr,
                                         d_cols, d_vals, d_src, s);
        *n_edges = (size_t)E;
    });
}

int ncvis_init_embedding_device(size_t N, size_t d, const int64_t *d_row_ptr,
                                const int32_t *d_cols, uint64_t seed, int n_init_epochs,
                                float alpha, int sequential_stats, float *dY, void *stream) {
    return guarded(nullptr, [&] {
        require(d_row_ptr && d_cols && dY, "init_embedding: null pointer");
        require(N >= 1 && d >= 1 && d <= 32 && n_init_epochs >= 0,
                "init_embedding: need N >= 1, 1 <= d <= 32, n_init_epochs >= 0");
        cudaStream_t s = (cudaStream_t)stream;
        // The graph must be a CSR over N rows: offsets from 0, non-decreasing,
        // columns in [0, N).
        std::vector<int64_t> rp(N + 1);
        NCVIS_CUDA(cudaMemcpyAsync(rp.data(), d_row_ptr, sizeof(int64_t) * (N + 1),
                                   cudaMemcpyDeviceToHost, s));
        NCVIS_CUDA(cudaStreamSynchronize(s));
        require(rp[0] == 0, "init_embedding: row_ptr[0] must be 0");
        for (size_t i = 0; i < N; ++i)
            require(rp[i + 1] >= rp[i], "init_embedding: row_ptr must be non-decreasing");
        require(rp[N] < (int64_t(1) << 31), "init_embedding: too many edges");
        require(indices_in_range(d_cols, rp[N], (int64_t)N, s),
                "init_embedding: a column index is outside [0, N)");
        StreamBuffer ws(init_workspace_bytes((int64_t)N, (int)d), s);
        run_init_embedding((int64_t)N, (int)d, d_row_ptr, d_cols, seed, n_init_epochs, alpha, dY,
                           ws.p, s, sequential_stats != 0);
    });
}

int ncvis_optimize_device(size_t N, size_t d, size_t E, const int32_t *d_src,
                          const int32_t *d_dst, float *dY, float *dQ, uint64_t seed,
                          int epoch_begin, int epoch_end, int n_epochs, const size_t *n_noise,
                          float a, float b, float alpha, float alpha_Q, int chains, void *stream) {
    return guarded(nullptr, [&] {
        require(d_src && d_dst && dY && dQ && n_noise, "optimize: null pointer");
        require(N >= 2 && d >= 1 && d <= 32, "optimize: need N >= 2 and 1 <= d <= 32");
        require(((uintptr_t)dY & (d == 4 ? 15 : 7)) == 0,
                "optimize: Y must be 8-byte aligned (16-byte for d = 4)");
        require((((uintptr_t)d_src | (uintptr_t)d_dst) & 15) == 0,
                "optimize: src and dst must be 16-byte aligned");
        require(0 <= epoch_begin && epoch_begin <= epoch_end && epoch_end <= n_epochs,
                "optimize: need 0 <= epoch_begin <= epoch_end <= n_epochs");
        check_noise(n_noise, epoch_begin, epoch_end, "optimize: ");
        cudaStream_t s = (cudaStream_t)stream;
        if (E == 0 || epoch_begin == epoch_end) return;
        require(edges_in_range(d_src, d_dst, (int64_t)E, (int64_t)N, s),
                "optimize: an edge endpoint is outside [0, N)");
        if (chains <= 0) chains = sgd_default_chains((int64_t)E, (int64_t)N, (int)d);
        StreamBuffer ws(sgd_workspace_bytes(chains), s);
        SgdArgs g{(int64_t)N, (int)d, (int64_t)E, d_src, d_dst, dY, dQ, seed, n_epochs,
                  a, b, alpha, alpha_Q};
        run_sgd_hogwild(g, epoch_begin, epoch_end, n_noise, chains, ws.p, s);
    });
}

int ncvis_optimize_staged_device(size_t N, size_t d, size_t E, const int32_t *d_src,
                                 const int32_t *d_dst, float *dY, float *dQ, uint64_t seed,
                                 int epoch_begin, int epoch_end, int n_epochs,
                                 const size_t *n_noise, float a, float b, float alpha,
                                 float alpha_Q, int chains, int round_edges, void *stream) {
    return guarded(nullptr, [&] {
        require(d_src && d_dst && dY && dQ && n_noise, "optimize_staged: null pointer");
        require(N >= 2 && N < (size_t(1) << 31), "optimize_staged: N must be in [2, 2^31)");
        require(sgd_window_applies((int64_t)N, (int)d),
                "optimize_staged: needs 1 <= d <= 4 and N >= 16 * " +
                    std::to_string(d >= 1 && d <= 4 ? sgd_window_rows((int)d) : 0u) +
                    " (16 noise windows)");
        require(((uintptr_t)dY & (d == 4 ? 15 : 7)) == 0,
                "optimize_staged: Y must be 8-byte aligned (16-byte for d = 4)");
        require((((uintptr_t)d_src | (uintptr_t)d_dst) & 15) == 0,
                "optimize_staged: src and dst must be 16-byte aligned");
        require(0 <= epoch_begin && epoch_begin <= epoch_end && epoch_end <= n_epochs,
                "optimize_staged: need 0 <= epoch_begin <= epoch_end <= n_epochs");
        check_noise(n_noise, epoch_begin, epoch_end, "optimize_staged: ");
        cudaStream_t s = (cudaStream_t)stream;
        if (E == 0 || epoch_begin == epoch_end) return;
        require(edges_in_range(d_src, d_dst, (int64_t)E, (int64_t)N, s),
                "optimize_staged: an edge endpoint is outside [0, N)");
        if (chains <= 0) chains = sgd_window_default_chains((int64_t)E, (int64_t)N, (int)d);
        StreamBuffer ws(sgd_workspace_bytes(chains), s);
        SgdArgs g{(int64_t)N, (int)d, (int64_t)E, d_src, d_dst, dY, dQ, seed, n_epochs,
                  a, b, alpha, alpha_Q};
        run_sgd_window(g, epoch_begin, epoch_end, n_noise, chains, round_edges, ws.p, s);
    });
}

int ncvis_optimize_replay_device(size_t N, size_t d, const int32_t *d_src, const int32_t *d_dst,
                                 size_t edge_begin, size_t edge_end, const int32_t *d_stream,
                                 size_t stream_offset, float *dY, float *dQ, int epoch,
                                 int n_epochs, size_t n_noise_epoch, float a, float b, float alpha,
                                 float alpha_Q, void *stream) {
    return guarded(nullptr, [&] {
        require(d_src && d_dst && dY && dQ, "optimize_replay: null pointer");
        require(d_stream || n_noise_epoch == 0, "optimize_replay: null noise stream");
        require(N >= 2 && d >= 1 && d <= 32, "optimize_replay: need N >= 2 and 1 <= d <= 32");
        require(edge_begin <= edge_end && epoch >= 0 && epoch < n_epochs,
                "optimize_replay: bad edge or epoch range");
        check_noise(&n_noise_epoch, 0, 1, "optimize_replay: ");
        cudaStream_t s = (cudaStream_t)stream;
        StreamBuffer err_buf(sizeof(int), s);
        int *err = (int *)err_buf.p;
        NCVIS_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
        SgdArgs g{(int64_t)N, (int)d, 0, d_src, d_dst, dY, dQ, 0, n_epochs, a, b, alpha, alpha_Q};
        launch_sgd_replay(g, epoch, n_noise_epoch, (int64_t)edge_begin, (int64_t)edge_end,
                          d_stream, (int64_t)stream_offset, err, s);
        int herr = 0;
        NCVIS_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
        NCVIS_CUDA(cudaStreamSynchronize(s));
        require(herr == 0, "optimize_replay: an index outside [0, N) was met; replay stopped");
    });
}

int ncvis_nce_loss_device(size_t N, size_t d, size_t E, const int32_t *d_src, const int32_t *d_dst,
                          const float *dY, const float *dQ, size_t n_noise, float a, float b,
                          uint64_t seed, uint32_t tag, uint64_t edge_offset, double *d_loss,
                          void *stream) {
    return guarded(nullptr, [&] {
        require(d_src && d_dst && dY && dQ && d_loss, "nce_loss: null pointer");
        require(N >= 2 && N < (size_t(1) << 31) && d >= 1 && d <= 32 && n_noise >= 1 &&
                    n_noise <= 1024,
                "nce_loss: need 2 <= N < 2^31, 1 <= d <= 32, 1 <= n_noise <= 1024");
        cudaStream_t s = (cudaStream_t)stream;
        require(edges_in_range(d_src, d_dst, (int64_t)E, (int64_t)N, s),
                "nce_loss: an edge endpoint is outside [0, N)");
        StreamBuffer ws(nce_workspace_bytes((int64_t)E), s);
        run_nce(0, (int64_t)N, (int)d, (int64_t)E, d_src, d_dst, dY, dQ, (int)n_noise, a, b, seed,
                tag, edge_offset, nullptr, nullptr, d_loss, ws.p, s);
    });
}

int ncvis_nce_grad_device(size_t N, size_t d, size_t E, const int32_t *d_src, const int32_t *d_dst,
                          const float *dY, const float *dQ, size_t n_noise, float a, float b,
                          uint64_t seed, uint32_t tag, uint64_t edge_offset, const float *d_scale,
                          float *d_gradY, double *d_gradQ, void *stream) {
    return guarded(nullptr, [&] {
        require(d_src && d_dst && dY && dQ && d_scale && d_gradY && d_gradQ,
                "nce_grad: null pointer");
        require(N >= 2 && N < (size_t(1) << 31) && d >= 1 && d <= 32 && n_noise >= 1 &&
                    n_noise <= 1024,
                "nce_grad: need 2 <= N < 2^31, 1 <= d <= 32, 1 <= n_noise <= 1024");
        cudaStream_t s = (cudaStream_t)stream;
        require(edges_in_range(d_src, d_dst, (int64_t)E, (int64_t)N, s),
                "nce_grad: an edge endpoint is outside [0, N)");
        StreamBuffer ws(nce_workspace_bytes((int64_t)E), s);
        run_nce(1, (int64_t)N, (int)d, (int64_t)E, d_src, d_dst, dY, dQ, (int)n_noise, a, b, seed,
                tag, edge_offset, d_scale, d_gradY, d_gradQ, ws.p, s);
    });
}

int ncvis_nce_noise_device(size_t N, size_t E, const int32_t *d_src, size_t n_noise, uint64_t seed,
                           uint32_t tag, uint64_t edge_offset, int32_t *d_out, void *stream) {
    return guarded(nullptr, [&] {
        require(d_src && d_out, "nce_noise: null pointer");
        require(N >= 2 && N < (size_t(1) << 31), "nce_noise: need 2 <= N < 2^31");
        cudaStream_t s = (cudaStream_t)stream;
        require(indices_in_range(d_src, (int64_t)E, (int64_t)N, s),
                "nce_noise: a source is outside [0, N)");
        launch_noise_table((int64_t)N, (int64_t)E, d_src, (int)n_noise, seed, tag, edge_offset,
                           d_out, s);
    });
}

uint64_t ncvis_kernel_launch_count(void) { return launch_counter().load(); }

const char *ncvis_version(void) { return "ncvis_gb300 0.1.0 (sm_103a)"; }

}  // extern "C"
