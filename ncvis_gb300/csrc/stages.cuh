// Host-side launchers of the engine's stages.  Every launcher only enqueues
// work on `stream` (no synchronisation) unless its comment says otherwise.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace ncvis_gpu {

enum Distance { kSquaredL2 = 0, kInnerProduct = 1, kCosine = 2, kCorrelation = 3 };

// ---- K1 preprocess (src/ncvis.cpp:32-70) -------------------------------------
// Xp[N, D] f32 preprocessed rows, sqnorm[N] = |xp|^2, and (if Xb != nullptr)
// Xb[N, ldb] bf16 copies zero-padded to ldb columns.  bad_flag (device int)
// is set to 1 if any input is not finite.
// Xc (optional, squared L2 on the tensor cores): candidate copy whose columns
// D, D + 1 hold -|x|^2 / 2 as BF16 high + low parts; Xb then holds 1, 1 there.
void launch_preprocess(const float *X, int64_t N, int D, int dist, float *Xp, float *sqnorm,
                       __nv_bfloat16 *Xb, int ldb, int *bad_flag, cudaStream_t s,
                       __nv_bfloat16 *Xc = nullptr);

// Independent problems packed in one point array: problem p owns rows
// [offsets[p], offsets[p+1]) (device arrays).  B == 0: one problem, all rows.
struct Segments {
    const int64_t *offsets = nullptr;      // [B+1]
    const int64_t *tile_prefix = nullptr;  // [B+1] query tiles of the kNN kernel per problem
    int B = 0;
    int64_t n_tiles = 0;
};

// ---- K3 exact FP32 candidate selection + K4 rerank ---------------------------
struct KnnPlan {
    int R;       // candidates kept per (point, split)
    int splits;  // candidate-range splits
    int C() const { return R * splits; }
};
KnnPlan plan_knn_f32(int64_t N, int k, int rerank_factor);
// cand_i/cand_d: [N, plan.C()]; -1 marks an empty slot.
void launch_knn_select_f32(const float *Xp, const float *sqnorm, int64_t N, int D, int dist,
                           const KnnPlan &plan, int32_t *cand_i, float *cand_d, cudaStream_t s,
                           const Segments &seg = Segments());
int knn_f32_query_tile();
// Exact distances of the candidates, top k+1 by (distance, index), smallest
// dropped, k written in descending order: inds/dists [N, k].  `order` (a
// permutation of the rows, or nullptr) is the order the rows are processed
// in; the result does not depend on it.
void launch_rerank(const float *Xp, int64_t N, int D, int dist, const int32_t *cand_i, int C,
                   int k, int32_t *inds, float *dists, cudaStream_t s,
                   const int32_t *order = nullptr);

// ---- K2 BF16 tensor-core candidate selection ---------------------------------
struct KnnTcPlan {
    int R;       // candidates kept per point (multiple of 4 is not required)
    int ldb;     // padded row length of Xb (bf16 elements)
    bool fold;   // squared L2 with the norms folded into the product (needs Xc)
    int64_t Npad;
    // Diagnostics: limit of the kernel's waits between its roles in SM cycles
    // (<= 0: about 2 s), and a stall on a barrier nothing completes (the
    // timeout path's test).
    long long wait_cycles = 0;
    bool stall = false;
};
KnnTcPlan plan_knn_tc(int64_t N, int D, int k, int rerank_factor, int dist);
bool knn_tc_supported(int D, int R);
// One item of a tensor-core launch's work list: the 256 query rows from row0
// (rows at or past qend are not outputs) against candidate rows [lo, hi).
// Outputs go to row + out_off with entries c + out_off, or, when the work has
// a row map, to map[row] with entries map[c].  kTcContinue: the item extends
// the previous item's query tile (same row0: the tile is not reloaded and its
// lists carry over); kTcMore: a later item continues this one (the lists are
// written after the last item of a query tile).
constexpr int kTcContinue = 1;
constexpr int kTcMore = 2;
struct alignas(16) TcItem {
    int32_t row0, qend, lo, hi;
    int32_t out_off, flags, pad0, pad1;
};
// Work of one launch (device arrays): CTA b takes items[begin[b] .. begin[b+1]).
struct TcWork {
    int ctas;
    const int64_t *begin;
    const TcItem *items;
    const int32_t *map;  // optional row map (sorted row -> output row), or null
};
void launch_knn_select_tc(const __nv_bfloat16 *Xb, const float *sqnorm, int64_t N,
                          const KnnTcPlan &plan, int dist, int32_t *cand_i, float *cand_d,
                          int *timeout_flag, cudaStream_t s, const TcWork *work = nullptr,
                          const __nv_bfloat16 *Xc = nullptr);
// Approximate candidate selection (inverted file): C cells from k-means on
// the BF16 rows, each cell searched against its `probe` nearest cells.
struct IvfPlan {
    int C = 1, probe = 1, iters = 4;
};
IvfPlan plan_ivf(int64_t N, int lists, int probe);
// Xp: preprocessed FP32 rows; Xb (and Xc with the folded squared-L2 product)
// as for launch_knn_select_tc; cand_i [N, tp.R] receives the candidates in
// original numbering (its first N * 32 entries also serve as scratch).
void run_knn_ivf(const float *Xp, const __nv_bfloat16 *Xb, const __nv_bfloat16 *Xc, int64_t N,
                 int D, const KnnTcPlan &tp, int dist, const IvfPlan &ip, uint64_t seed,
                 int32_t *cand_i, int *timeout_flag, cudaStream_t s);

// The exact selection with the rows ordered by k-means cell, each query
// tile's sweep starting at its own cell (warm start; same candidates as
// launch_knn_select_tc up to exact score ties at the R-th place).  Applies
// to the inner-product spaces and the folded squared-L2 product, from
// kKnnOrderMinRows points; C == 0 means the caller's order.
constexpr int64_t kKnnOrderMinRows = 32768;
struct KnnOrderPlan {
    int C = 0, iters = 0;
};
// cells: 0 automatic (N / 4096, at least 16), -1 never, > 0 that many.
KnnOrderPlan plan_knn_order(int64_t N, int D, const KnnTcPlan &tp, int dist, int cells);
// Workspace of run_knn_tc_ordered (0 when op.C == 0).  With workspace ==
// nullptr the call allocates stream-ordered memory instead.  Waits on the
// stream (cell sizes, timeout flag).
size_t knn_order_workspace_bytes(int64_t N, int D, const KnnTcPlan &tp, const KnnOrderPlan &op);
void run_knn_tc_ordered(const float *Xp, const __nv_bfloat16 *Xb, const __nv_bfloat16 *Xc,
                        int64_t N, int D, const KnnTcPlan &tp, int dist, const KnnOrderPlan &op,
                        uint64_t seed, int32_t *cand_i, int *timeout_flag, cudaStream_t s,
                        void *workspace = nullptr, size_t workspace_bytes = 0,
                        cudaEvent_t sweep_start = nullptr, const int32_t **cell_order = nullptr);

// Queries from Q (nq rows) against candidates from Cm (nc rows), both bf16
// [rows, plan.ldb]; c_sqnorm: candidate squared norms (used for squared L2
// without the folded norms); `ip`: rank by the product (inner-product spaces,
// or squared L2 with the folded candidate copy).  A work list is required.
void launch_knn_select_tc_pair(const __nv_bfloat16 *Q, int64_t nq, const __nv_bfloat16 *Cm,
                               int64_t nc, const float *c_sqnorm, const KnnTcPlan &plan, bool ip,
                               int32_t *cand_i, int *timeout_flag, cudaStream_t s,
                               const TcWork &work);

// ---- K5 symmetrize (src/knntable.cpp:24-99, src/ncvis.cpp:155-173) -----------
size_t symmetrize_workspace_bytes(int64_t N, int k);
// Enqueues the CSR build and returns E (waits on the stream for the count).
int64_t run_symmetrize(int64_t N, int k, const int32_t *inds, const float *dists, void *workspace,
                       int64_t *row_ptr, int32_t *cols, float *vals, int32_t *src,
                       cudaStream_t s);

// True when every a[0..n) lies in [0, N) (waits on the stream).
bool indices_in_range(const int32_t *a, int64_t n, int64_t N, cudaStream_t s);
bool edges_in_range(const int32_t *a, const int32_t *b, int64_t n, int64_t N, cudaStream_t s);

// ---- device-wide exclusive scan ----------------------------------------------
size_t scan_workspace_bytes(int64_t n);
// out[0..n]: out[0] = 0, out[i+1] = out[i] + in[i].
void launch_exclusive_scan_i32_to_i64(const int32_t *in, int64_t *out, int64_t n, void *ws,
                                      cudaStream_t s);

// ---- K6 init (src/ncvis.cpp:184-273) ------------------------------------------
size_t init_workspace_bytes(int64_t N, int d);
// sequential_stats: the per-dimension mean and std as the reference's one
// thread sums them (FP32, rows in order; slower: one dependent add chain per
// dimension) instead of FP64 partial sums.
void run_init_embedding(int64_t N, int d, const int64_t *row_ptr, const int32_t *cols,
                        uint64_t seed, int n_init_epochs, float alpha, float *Y, void *workspace,
                        cudaStream_t s, bool sequential_stats = false);

// Batched problems (rows [off[p], off[p+1]), seeds[p]); tp[p] = first row tile
// of problem p, tiles of init_tile_rows() rows never straddle problems.
int init_tile_rows();
size_t init_batched_workspace_bytes(int64_t total_rows, int64_t n_tiles, int B, int d);
void run_init_embedding_batched(int64_t total_rows, int d, const int64_t *off, const int64_t *tp,
                                int B, int64_t n_tiles, const uint64_t *seeds,
                                const int64_t *row_ptr, const int32_t *cols, int n_init_epochs,
                                float alpha, float *Y, void *workspace, cudaStream_t s);

// ---- K7 SGD (src/ncvis.cpp:275-352) -------------------------------------------
struct SgdArgs {
    int64_t N;
    int d;
    int64_t E;
    const int32_t *src;
    const int32_t *dst;
    float *Y;
    float *Q;  // device scalar
    uint64_t seed;
    int n_epochs;
    float a, b, alpha, alpha_Q;
};
size_t sgd_workspace_bytes(int chains);
int sgd_default_chains(int64_t E, int64_t N, int d);
void run_sgd_hogwild(const SgdArgs &args, int epoch_begin, int epoch_end, const size_t *n_noise,
                     int chains, void *workspace, cudaStream_t s);
// Hogwild with noise staged in shared-memory windows of Y (d <= 4, N >= 16
// window rows); round_edges <= 0: the default (8 edges per chain per round).
uint32_t sgd_window_rows(int d);
bool sgd_window_applies(int64_t N, int d);
int sgd_window_default_chains(int64_t E, int64_t N, int d);
void run_sgd_window(const SgdArgs &args, int epoch_begin, int epoch_end, const size_t *n_noise,
                    int chains, int round_edges, void *workspace, cudaStream_t s);
// Batched Hogwild: problem p owns rows [off[p], off[p+1]), edges
// [eoff[p], eoff[p+1]) and chains [cp[p], cp[p+1]) (device arrays); Qs[B] and
// chain_q[n_chains] device floats.  d <= 4.
struct SgdBatch {
    int d;
    int B;
    int64_t n_chains;
    const int32_t *src, *dst;
    const int64_t *off, *eoff, *cp;
    float *Y, *Qs, *chain_q;
    uint64_t seed;
    int n_epochs;
    float a, b, alpha, alpha_Q;
};
void run_sgd_hogwild_batched(const SgdBatch &g, const size_t *n_noise, cudaStream_t s);
// The same with the noise staged in shared memory (d <= 4): problem p's chains
// [cp[p], cp[p+1]) run in blocks [bp[p], bp[p+1]) of `threads` chains each
// (64, 128 or 256; device array bp of B + 1 entries, n_blocks = bp[B]).
bool sgd_window_batched_threads_ok(int threads);
void run_sgd_window_batched(const SgdBatch &g, const int64_t *bp, int64_t n_blocks, int threads,
                            const size_t *n_noise, cudaStream_t s);
int64_t sgd_batched_resident_chains(int d);
// *err (device int) is set to 1 if an index outside [0, N) is met.
void launch_sgd_replay(const SgdArgs &args, int epoch, size_t nu, int64_t edge_begin,
                       int64_t edge_end, const int32_t *stream, int64_t stream_offset, int *err,
                       cudaStream_t s);

// ---- K8 NCE loss (the objective of src/ncvis.cpp:275-352) --------------------
// Threads per block of the loss kernels; the workspace holds two FP64
// partials per block plus two: nce_workspace_bytes(E) =
// 16 * ((E + kNceThreads - 1) / kNceThreads + 1).
constexpr int kNceThreads = 256;
size_t nce_workspace_bytes(int64_t E);
// mode 0: *out = loss (FP64 sum); mode 1: dY += (*scale) dL/dY (atomic FP32),
// *out = (*scale) dL/dQ (FP64).
void run_nce(int mode, int64_t N, int d, int64_t E, const int32_t *src, const int32_t *dst,
             const float *Y, const float *Q, int nu, float a, float b, uint64_t seed,
             uint32_t tag, uint64_t edge_offset, const float *scale, float *dY, double *out,
             void *workspace, cudaStream_t s);
// The loss's noise indices for edges [0, E): out [E, nu].
void launch_noise_table(int64_t N, int64_t E, const int32_t *src, int nu, uint64_t seed,
                        uint32_t tag, uint64_t edge_offset, int32_t *out, cudaStream_t s);

}  // namespace ncvis_gpu
