/*
 * ncvis_gb300.h — C ABI of the GB300 NCVis engine (libncvis_gb300.so).
 *
 * Plain pointers and sizes only.  Every function returns an int status
 * (NCVIS_OK == 0) unless stated otherwise; the message of the last failure is
 * available from ncvis_last_error(handle) or, for the handle-less stage
 * functions, ncvis_get_last_error() (per calling thread).
 *
 * Reference interfaces replaced (stat-ml/ncvis):
 *   ncvis_params / ncvis_create  <- ncvis::NCVis::NCVis(...)   src/ncvis.hpp:54, src/ncvis.cpp:12-21
 *   ncvis_destroy                <- ncvis::NCVis::~NCVis()      src/ncvis.hpp:55, src/ncvis.cpp:23-30
 *   ncvis_fit_transform          <- ncvis::NCVis::fit_transform src/ncvis.hpp:66, src/ncvis.cpp:354-459
 *   ncvis_distance               <- enum ncvis::Distance        src/ncvis.hpp:27-32
 *   ncvis_knn_device             <- NCVis::buildKNN + findKNN   src/ncvis.cpp:72-153
 *   ncvis_knn_ivf_device         <- NCVis::buildKNN + findKNN (approximate) src/ncvis.cpp:72-153
 *   ncvis_symmetrize_device      <- KNNTable::symmetrize + NCVis::build_edges
 *                                   src/knntable.cpp:24-99, src/ncvis.cpp:155-173
 *   ncvis_init_embedding_device  <- NCVis::init_embedding       src/ncvis.cpp:184-273
 *   ncvis_optimize_device        <- NCVis::optimize             src/ncvis.cpp:275-352
 *   ncvis_optimize_staged_device <- NCVis::optimize, noise staged src/ncvis.cpp:275-352
 *   ncvis_optimize_replay_device <- NCVis::optimize, one thread src/ncvis.cpp:275-352
 * The C++ header include/ncvis.hpp wraps this ABI in a class with the
 * reference's exact constructor and fit_transform signatures.
 */
#ifndef NCVIS_GB300_H
#define NCVIS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define NCVIS_OK 0
#define NCVIS_INVALID_ARGUMENT 1
#define NCVIS_CUDA_ERROR 2
#define NCVIS_UNSUPPORTED 3
#define NCVIS_DEVICE_TIMEOUT 4
#define NCVIS_INTERNAL 5

/* Same values and order as ncvis::Distance (src/ncvis.hpp:27-32). */
typedef enum ncvis_distance {
    NCVIS_SQUARED_L2 = 0,
    NCVIS_INNER_PRODUCT = 1,
    NCVIS_COSINE_SIMILARITY = 2,
    NCVIS_CORRELATION = 3
} ncvis_distance;

/* kNN precision modes (ncvis_options.knn_precision). */
#define NCVIS_KNN_FP32 0      /* exact FP32 distances: the plain drop-in form */
#define NCVIS_KNN_BF16_RERANK 1 /* BF16 tensor-core distances, exact FP32 rerank */
#define NCVIS_KNN_IVF 2 /* approximate: k-means cells, each searched against its nearest cells
                           with BF16 tensor-core distances, exact FP32 rerank */
/* Flag, or-ed into knn_precision (or ncvis_knn_device's precision) with
 * NCVIS_KNN_BF16_RERANK: search the rows in the caller's order.  Without it
 * the exact BF16 search first orders the rows by k-means cell and sweeps each
 * query tile's candidates from its own cell onwards (from 32,768 points; the
 * inner-product spaces, and squared L2 with D <= 126), so that every point's
 * candidate list is nearly final early; the candidates found are the same up
 * to exact score ties at the last kept place. */
#define NCVIS_KNN_CALLER_ORDER 0x100

/* SGD modes (ncvis_options.sgd_mode). */
#define NCVIS_SGD_HOGWILD 0 /* parallel chains, counter-based noise samples; staged in
                               shared-memory windows of Y where N is large enough */
#define NCVIS_SGD_REPLAY 1  /* one chain consuming a recorded noise stream */
#define NCVIS_SGD_HOGWILD_UNSTAGED 2 /* parallel chains, every noise row read from Y itself */

/* Constructor arguments of ncvis::NCVis (src/ncvis.hpp:54), same meaning.
 * M and ef_construction configure HNSW in the reference and are accepted and
 * ignored here (the kNN is exact).  n_threads bounds host-side work only.
 * n_noise: n_epochs entries (copied at create), or NULL for 3 per epoch;
 * each at most 2^24 (16,777,216), larger values are refused. */
typedef struct ncvis_params {
    size_t d;
    size_t n_threads;
    size_t n_neighbors;
    size_t M;
    size_t ef_construction;
    size_t random_seed;
    int n_epochs;
    int n_init_epochs;
    float a;
    float b;
    float alpha;
    float alpha_Q;
    const size_t *n_noise;
    int distance; /* ncvis_distance */
} ncvis_params;

/* Engine options beyond the reference's constructor (all zero = defaults:
 * FP32 exact kNN, Hogwild SGD, engine-owned stream, automatic chain count). */
typedef struct ncvis_options {
    int knn_precision;      /* NCVIS_KNN_FP32 | NCVIS_KNN_BF16_RERANK | NCVIS_KNN_IVF */
    int rerank_factor;      /* candidates kept per point ~ rerank_factor * k (0: 2; BF16 keeps 32 or 64) */
    int sgd_mode;           /* NCVIS_SGD_HOGWILD | NCVIS_SGD_REPLAY | NCVIS_SGD_HOGWILD_UNSTAGED */
    const int32_t *replay_stream; /* host array of noise indices in one-thread draw order (replay) */
    size_t replay_len;      /* entries in replay_stream: E * sum(n_noise) */
    void *stream;           /* cudaStream_t to run on; NULL: the engine's own stream */
    int sgd_chains;         /* parallel SGD chains; 0: automatic */
    int ivf_lists;          /* NCVIS_KNN_IVF: k-means cells; 0: N / 512 (at most 65,536) */
    int ivf_probe;          /* NCVIS_KNN_IVF: cells searched per cell, its own included, at
                               most 64; 0: 32 */
    long long wait_limit_cycles; /* limit of the tensor-core kNN kernel's waits between its
                               roles, in SM clock cycles (0: 4e9, about 2 s); a wait that runs
                               out stops the kernel and the call returns NCVIS_DEVICE_TIMEOUT */
    int inject_stall;       /* diagnostics: nonzero makes the tensor-core kNN kernel first wait
                               on a barrier that nothing completes, so that the wait runs out
                               (a test of the timeout path); 0 in normal use */
    size_t arena_limit;     /* largest device arena (the fit's device buffers) the engine may
                               hold, in bytes (0: no limit); a fit that needs more fails as an
                               allocation failure (NCVIS_CUDA_ERROR) */
    int init_sequential_stats; /* init_embedding's mean and std: 0 from FP64 partial sums;
                               nonzero as the reference's one thread sums them (see
                               ncvis_init_embedding_device) */
    int knn_order_cells;    /* k-means cells that order the rows before the exact BF16 search
                               (see NCVIS_KNN_CALLER_ORDER); 0: N / 4096, at least 16 */
} ncvis_options;

/* Per-stage device times of the last fit_transform, in milliseconds, named
 * after the reference's DEBUG stage timers (src/ncvis.cpp:370-437). */
typedef struct ncvis_stage_times {
    float h2d_ms;
    float preprocess_ms;
    float knn_ms;        /* candidate selection (buildKNN + findKNN) */
    float rerank_ms;     /* exact rerank of the candidates */
    float symmetrize_ms;
    float build_edges_ms;
    float init_ms;
    float optimize_ms;
    float d2h_ms;
    float total_ms;
    int64_t n_edges;     /* symmetrized directed edges E */
    int64_t k;           /* neighbours per point after clamping */
    float knn_order_ms;  /* part of knn_ms: the k-means cell ordering before the exact BF16
                            search's sweep (0 when the rows keep the caller's order) */
} ncvis_stage_times;

typedef struct ncvis_engine *ncvis_handle;

/* Engine lifetime.  ncvis_create returns NULL on invalid parameters (the
 * reason is in ncvis_get_last_error()).  `options` may be NULL. */
ncvis_handle ncvis_create(const ncvis_params *params, const ncvis_options *options);
void ncvis_destroy(ncvis_handle h);
int ncvis_set_options(ncvis_handle h, const ncvis_options *options);

/* Host buffers: X [N, D] row-major float32 (read), Y [N, d] row-major float32
 * (written).  Errors as the reference: N == 0 || D == 0, Y == NULL. */
int ncvis_fit_transform(ncvis_handle h, const float *X, size_t N, size_t D, float *Y);

/* Device buffers (same layout), enqueued on the engine's stream; returns
 * after the work is enqueued and the edge count is known. */
int ncvis_fit_transform_device(ncvis_handle h, const float *dX, size_t N, size_t D, float *dY);

/* Many independent embeddings in one run.  Problem p is rows
 * [offsets[p], offsets[p+1]) of dX [offsets[n], D] (device) and gets rows of
 * dY [offsets[n], d] (device); offsets (n+1 entries) and seeds (n entries,
 * NULL: every problem uses random_seed) are host arrays.  Every problem
 * follows the engine's parameters (k clamped by the smallest problem) with
 * its own kNN graph, initialisation stream, noise range and Q; the SGD epoch
 * loop of all problems runs as one captured CUDA graph.  d <= 4.  The kNN
 * follows knn_precision: exact FP32, or BF16 on the tensor cores with the
 * exact rerank (also for NCVIS_KNN_IVF: the problems are searched exactly).
 * The optimizer stages noise samples per problem unless sgd_mode is
 * NCVIS_SGD_HOGWILD_UNSTAGED; NCVIS_SGD_REPLAY is refused (NCVIS_INVALID_ARGUMENT).
 * No reference counterpart (the reference
 * embeds one dataset per call). */
int ncvis_fit_transform_batched_device(ncvis_handle h, const float *dX, size_t D,
                                       const int64_t *offsets, size_t n_problems,
                                       const uint64_t *seeds, float *dY);

const char *ncvis_last_error(ncvis_handle h);
const char *ncvis_get_last_error(void);
int ncvis_get_stage_times(ncvis_handle h, ncvis_stage_times *out);

/* ----------------------------------------------------------------------
 * Stage-level entry points.  Device pointers, enqueued on `stream`
 * (cudaStream_t, NULL = legacy default stream).  Indices are int32, so
 * N < 2^31 and N * k < 2^30.
 * -------------------------------------------------------------------- */

/* Exact kNN table with the reference's row contract (src/ncvis.cpp:128-153):
 * the k+1 smallest (distance, index) pairs of each preprocessed point over all
 * points, the smallest dropped, the other k stored in descending order.
 * Distances: squared L2, or 1 - <x, y> after the reference's preprocessing
 * (centring for correlation, unit norm for cosine/correlation). */
int ncvis_knn_device(const float *dX, size_t N, size_t D, int distance, size_t k, int precision,
                     int rerank_factor, int32_t *d_inds, float *d_dists, void *stream);

/* The approximate kNN of NCVIS_KNN_IVF with explicit cells and probes (0:
 * the defaults); the row contract and distances as ncvis_knn_device.  The
 * reference's kNN (hnswlib, src/ncvis.cpp:72-153) is approximate too; this
 * is the GPU counterpart for point counts where the exact search's O(N^2 D)
 * work is too large.  Needs D <= 128 (D <= 126 for squared L2). */
int ncvis_knn_ivf_device(const float *dX, size_t N, size_t D, int distance, size_t k,
                         int rerank_factor, int lists, int probe, int32_t *d_inds,
                         float *d_dists, void *stream);

/* Symmetrization, bit-exact with the reference's one-thread
 * KNNTable::symmetrize on the same table, emitted as CSR.  Rows are the
 * reference's rows after sorting and deduplication; flattening them row by
 * row gives NCVis::build_edges' edge list.  Capacity of d_cols / d_vals /
 * d_src must be 2 * N * k.  d_src (optional, may be NULL) receives the source
 * row of every entry.  *n_edges receives E (host). */
int ncvis_symmetrize_device(size_t N, size_t k, const int32_t *d_inds, const float *d_dists,
                            int64_t *d_row_ptr, int32_t *d_cols, float *d_vals, int32_t *d_src,
                            size_t *n_edges, void *stream);

/* init_embedding over a CSR graph: Y [N, d] ~ U(0,1) from the one-thread
 * pcg64(seed) stream, then n_init_epochs of neighbour averaging with weight
 * alpha followed by per-dimension standardisation.  sequential_stats = 0:
 * mean and std from FP64 partial sums (the exact statistics rounded once);
 * nonzero: FP32 sums over the rows in order, as the reference's one thread
 * forms them (its rounding drifts ~1e-4 relative from the exact statistics at
 * a million rows; slower, one dependent add chain per dimension). */
int ncvis_init_embedding_device(size_t N, size_t d, const int64_t *d_row_ptr,
                                const int32_t *d_cols, uint64_t seed, int n_init_epochs,
                                float alpha, int sequential_stats, float *dY, void *stream);

/* Parallel (Hogwild) NCE SGD over epochs [epoch_begin, epoch_end) of an
 * n_epochs schedule; Y and *dQ (device float) updated in place.  n_noise:
 * host array of n_epochs entries, each at most 2^24.  chains: 0 = automatic. */
int ncvis_optimize_device(size_t N, size_t d, size_t E, const int32_t *d_src,
                          const int32_t *d_dst, float *dY, float *dQ, uint64_t seed,
                          int epoch_begin, int epoch_end, int n_epochs, const size_t *n_noise,
                          float a, float b, float alpha, float alpha_Q, int chains, void *stream);

/* The same optimizer with its noise samples staged in shared memory
 * (NCVis::optimize, src/ncvis.cpp:275-352, with the noise draw of :300
 * restated): the chains run their edges in rounds of round_edges edges
 * (0 = 16; rounded up to a multiple of 4); per round each block of chains copies a window of Y (4096 rows
 * for d <= 2, 2048 for d = 3 and 4, in segments of 256 consecutive rows,
 * each starting at a uniform row and wrapping at N) into shared memory and draws every noise sample of the round uniformly
 * from the window, so each noise row is uniform over the N rows before the
 * source row is excluded (a pick equal to it, probability 1/N, is redrawn
 * within the window).  Updates of noise rows go to the window and are added to Y at the
 * end of the round.  Needs 1 <= d <= 4 and N >= 16 * window rows (65,536
 * for d <= 2, 32,768 for d = 3 and 4).  chains: 0 = automatic. */
int ncvis_optimize_staged_device(size_t N, size_t d, size_t E, const int32_t *d_src,
                                 const int32_t *d_dst, float *dY, float *dQ, uint64_t seed,
                                 int epoch_begin, int epoch_end, int n_epochs,
                                 const size_t *n_noise, float a, float b, float alpha,
                                 float alpha_Q, int chains, int round_edges, void *stream);

/* Replay: one chain runs edges [edge_begin, edge_end) of epoch `epoch` in
 * order, reading noise samples from d_stream starting at stream_offset, with
 * *dQ as the running normaliser copy (updated in place).  The arithmetic is
 * the reference's one-thread optimizer's, sample by sample. */
int ncvis_optimize_replay_device(size_t N, size_t d, const int32_t *d_src, const int32_t *d_dst,
                                 size_t edge_begin, size_t edge_end, const int32_t *d_stream,
                                 size_t stream_offset, float *dY, float *dQ, int epoch,
                                 int n_epochs, size_t n_noise_epoch, float a, float b, float alpha,
                                 float alpha_Q, void *stream);

/* Noise-contrastive loss of a batch of E edges (src[e], dst[e]) with n_noise
 * uniform noise samples each, drawn from the counter-based stream keyed by
 * (seed, tag) and counted by the global edge index edge_offset + e; the
 * objective whose per-sample gradient NCVis::optimize follows
 * (src/ncvis.cpp:304-323).  *d_loss (device double) = the summed loss. */
int ncvis_nce_loss_device(size_t N, size_t d, size_t E, const int32_t *d_src, const int32_t *d_dst,
                          const float *dY, const float *dQ, size_t n_noise, float a, float b,
                          uint64_t seed, uint32_t tag, uint64_t edge_offset, double *d_loss,
                          void *stream);

/* Gradient of the same loss scaled by *d_scale (device float): d_gradY [N, d]
 * is accumulated into (+=), *d_gradQ (device double) is written. */
int ncvis_nce_grad_device(size_t N, size_t d, size_t E, const int32_t *d_src, const int32_t *d_dst,
                          const float *dY, const float *dQ, size_t n_noise, float a, float b,
                          uint64_t seed, uint32_t tag, uint64_t edge_offset, const float *d_scale,
                          float *d_gradY, double *d_gradQ, void *stream);

/* The noise indices the loss uses for edges [0, E): out [E, n_noise] (device
 * int32), for checking the loss against an independent implementation. */
int ncvis_nce_noise_device(size_t N, size_t E, const int32_t *d_src, size_t n_noise, uint64_t seed,
                           uint32_t tag, uint64_t edge_offset, int32_t *d_out, void *stream);

/* ncvis_nce_loss_device without any device allocation, for callers that
 * cannot allocate device memory when they need the loss (a process whose
 * memory pool already holds all free HBM, a latency-critical loop that must
 * not take the allocator's synchronisation, a framework that forbids
 * allocations outside its own pool).  Same arguments and result.  Its scratch
 * is one fixed device array of 65,568 bytes inside the library (kept on every
 * GPU that loads it until exit), so E <= 2^20 per call; larger E is rejected.
 * The first call on each device (and the first after that device's context
 * was re-created) looks up the array's device address and loads the
 * library's device code there: make it at start-up, while device memory is
 * free, and before any stream capture.  Each call waits for `stream` (it reads
 * an argument-check flag back).  Calls share the array: calls whose GPU work
 * overlaps in time race.  No counterpart in the reference (an addition).
 * Errors: ncvis_get_last_error(). */
int ncvis_nce_loss_device_noalloc(size_t N, size_t d, size_t E, const int32_t *d_src,
                                  const int32_t *d_dst, const float *dY, const float *dQ,
                                  size_t n_noise, float a, float b, uint64_t seed, uint32_t tag,
                                  uint64_t edge_offset, double *d_loss, void *stream);

/* Trustworthiness at k (Venna & Kaski 2001, as scikit-learn's
 * manifold.trustworthiness defines it) of the embedding dY [N, d] of dX
 * [N, D] (device float32, row-major), at full size: the embedding's exact kNN
 * (squared L2), then for every point the rank in X, under `distance` (the
 * engine's distances after its preprocessing), of each embedding neighbour,
 * counted over all N points in one FP32 pass.  1 <= k <= 16, 2k + 2 <= N.
 * *out receives T(k).  Allocates its scratch on `stream`; waits for it.
 * Replaces the reference's (and the tests') subsampled CPU check; no
 * counterpart in the reference's code (an addition).  Errors:
 * ncvis_get_last_error(). */
int ncvis_trustworthiness_device(const float *dX, size_t N, size_t D, int distance,
                                 const float *dY, size_t d, size_t k, double *out, void *stream);

/* Diagnostic: the rate at which this GPU serves the optimizer's memory
 * pattern, the ceiling for ncvis_optimize_device's pair-update rate.  On the
 * optimizer's launch shape it times random row gathers over a zeroed array of
 * `rows` rows of d floats (d = 1, 2 or 4), and random row gathers each followed
 * by a reduction into the same row (the optimizer's per-sample traffic):
 * *gathers_per_s and *updates_per_s.  Allocates and frees the array; runs on
 * `stream` and waits for it.  No counterpart in the reference (an addition).
 * Errors: ncvis_get_last_error(). */
int ncvis_measure_update_rate(size_t rows, size_t d, double *gathers_per_s, double *updates_per_s,
                              void *stream);

/* Number of kernels this library has launched in the process so far. */
uint64_t ncvis_kernel_launch_count(void);

/* Library version string. */
const char *ncvis_version(void);

#ifdef __cplusplus
}
#endif

#endif /* NCVIS_GB300_H */
