// K2: kNN candidate selection on the 5th-generation tensor cores (tcgen05),
// BF16 operands with FP32 accumulation; the candidates are re-ranked exactly
// in FP32 afterwards (K4, knn_simt.cu), which restores the reference's
// distances (src/ncvis.cpp:72-153) on the selected set.
//
// Work decomposition (one persistent CTA per SM, 11 warps):
//   * a query tile is 256 preprocessed points (two M=128 halves), held in
//     shared memory for the whole sweep (TMA, 128-byte swizzle, K-major);
//   * candidate tiles of 128 points stream through a 3-stage TMA ring;
//   * warp 0 issues TMA; warps 1 and 10 issue tcgen05.mma (M=128, N=128,
//     K=16 steps), one query half each, into one of two double-buffered
//     2x128-column FP32 accumulators (512 TMEM columns; warp 1 allocates);
//     each half hands its accumulators to its own four epilogue warps;
//   * warps 2..9 own one query row each (TMEM lane = row; warp % 4 selects
//     the lane quadrant): they read the accumulator with tcgen05.ld in
//     32-column chunks, turn dot products into ranking scores (-<q,c> for the
//     inner-product spaces, |c|^2 - 2<q,c> for squared L2), reduce each chunk
//     with 3-input min/max trees and compare its best with the row's worst;
//     qualifying candidates go to a per-row queue in shared memory, which the
//     warp inserts into the rows' register-resident sorted lists in lockstep
//     rounds (R compare-exchanges each) when a queue passes half full;
//   * a CTA takes query tiles round-robin over one problem, or items from its
//     own work list: an item is a query tile's rows and one candidate range
//     (masked at both ends), and may continue the previous item's tile, so
//     one tile's lists are built over several ranges (batched problems: the
//     tile's own problem; the inverted file: the tile's probed cells), with
//     an optional map from sorted rows back to the caller's numbering;
//   * squared L2 with D <= 126 folds the candidate norms into the product:
//     candidates come from a second BF16 copy whose columns D, D + 1 hold
//     -|c|^2 / 2 as a BF16 high and low part, the queries' copy 1, 1 there, so
//     the accumulator holds <q, c> - |c|^2 / 2 and the scan is the
//     inner-product one (otherwise the scan adds the FP32 norms per column).
// Every mbarrier wait is bounded in time: on expiry the CTA sets *err,
// stops, drains its MMAs and in-flight TMA copies, frees TMEM and returns.
// The waits between roles use the plan's limit (default ~2 s); the drain
// waits always use the long one.  An epilogue warp decides as a warp (votes)
// whether to stop, so its lanes never part at a warp-collective instruction.
// A diagnostic stall makes the producer first wait on a barrier that nothing
// completes, so that the timeout path runs deterministically.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cfloat>
#include <string>

#include "common.cuh"
#include "stages.cuh"

namespace ncvis_gpu {

namespace {

constexpr int kQueryTile = 256;   // queries per CTA tile (2 x M=128)
constexpr int kCandTile = 128;    // candidates per tile (N=128)
constexpr int kStages = 3;        // candidate-tile ring
constexpr int kAtomBytes = 128 * 128;  // 128 rows x 128 bytes (64 bf16) per swizzle atom column
constexpr int kMaxAtoms = 2;      // K <= 128
constexpr int kThreads = 352;
constexpr int kEpiWarp0 = 2;
constexpr int kEpiWarps = 8;
constexpr int kMmaWarp1 = 10;  // issues the second query half's MMAs (warp 1 the first)
constexpr int kEpiThreads = kEpiWarps * 32;
constexpr int kQueue = 32;  // per-row insertion queue slots (shared memory)
constexpr uint32_t kTmemCols = 512;
constexpr long long kWaitCycles = 4000000000LL;  // ~2 s at 2 GHz

struct SharedStorage {
    // 1024-byte aligned tiles first (128B swizzle atoms repeat every 1024 B).
    uint8_t a[2][kMaxAtoms][kAtomBytes];
    uint8_t b[kStages][kMaxAtoms][kAtomBytes];
    float queue_v[kQueue][kEpiThreads];    // queued candidate scores, [slot][thread]
    int32_t queue_i[kQueue][kEpiThreads];  // and their candidate indices
    uint64_t full[kStages];
    uint64_t empty[kStages];
    uint64_t a_full, a_empty;
    uint64_t acc_full[2][2], acc_empty[2][2];  // [buffer][query half]
    uint64_t drain;
    uint64_t never;  // completed by nothing: the diagnostic stall waits on it
    uint32_t tmem_base;
    volatile int abort;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait (`limit` SM cycles) for the phase of `parity`; false if it
// expired or the CTA aborted.
__device__ __forceinline__ bool mbar_wait(SharedStorage &s, uint64_t *bar, uint32_t parity,
                                          int *err, int code, long long limit) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (s.abort) return false;
        if (clock64() - t0 > limit) {
            s.abort = 1;
            atomicExch(err, code);
            return false;
        }
    }
    return true;
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int x,
                                            int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%3, %4}], [%2];" ::"r"(smem_u32(dst)),
        "l"(map), "r"(smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (stride byte offset), descriptor version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)1 << 16;             // leading byte offset (unused with 128B swizzle, K-major)
    d |= (uint64_t)(1024 >> 4) << 32;   // stride byte offset
    d |= (uint64_t)1 << 46;             // version
    d |= (uint64_t)2 << 61;             // 128-byte swizzle
    return d;
}

// Instruction descriptor, kind::f16: D f32, A and B bf16, both K-major, M=128, N=128.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kCandTile >> 3) << 17) |
                            ((uint32_t)(128 >> 4) << 24);

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %3, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %4, p;\n\t}" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(acc), "r"(kIdesc));
}

__device__ __forceinline__ void umma_commit(uint64_t *bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tmem_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tmem_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tmem_ld(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
          "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
          "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ void tmem_ld(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ float max3f(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// Minimum (kMax false) or maximum of n values, as a tree of 3-input operations.
template <bool kMax, int n>
__device__ __forceinline__ float tree_reduce(const float (&a)[n]) {
    if constexpr (n == 1) {
        return a[0];
    } else if constexpr (n == 2) {
        return kMax ? fmaxf(a[0], a[1]) : fminf(a[0], a[1]);
    } else {
        constexpr int m = (n + 2) / 3;
        float b[m];
#pragma unroll
        for (int j = 0; j < m; ++j) {
            if (3 * j + 2 < n)
                b[j] = kMax ? max3f(a[3 * j], a[3 * j + 1], a[3 * j + 2])
                            : min3f(a[3 * j], a[3 * j + 1], a[3 * j + 2]);
            else if (3 * j + 1 < n)
                b[j] = kMax ? fmaxf(a[3 * j], a[3 * j + 1]) : fminf(a[3 * j], a[3 * j + 1]);
            else
                b[j] = a[3 * j];
        }
        return tree_reduce<kMax, m>(b);
    }
}

// Insert (v, vi) into the ascending list (ls, li) of R entries, dropping the
// largest: one compare-exchange per slot, indices follow their scores.
template <int R>
__device__ __forceinline__ void list_push(float (&ls)[R], int32_t (&li)[R], float v, int32_t vi) {
#pragma unroll
    for (int t = 0; t < R; ++t) {
        const bool lt = v < ls[t];
        const float a = lt ? v : ls[t];
        const int32_t ai = lt ? vi : li[t];
        const float b = lt ? ls[t] : v;
        const int32_t bi = lt ? li[t] : vi;
        ls[t] = a;
        li[t] = ai;
        v = b;
        vi = bi;
    }
}

// Every queued candidate of the warp's rows goes into its row's list, in
// lockstep rounds (one per slot of the fullest queue); queues end empty.
template <int R>
__device__ __forceinline__ void flush_queue(float (&ls)[R], int32_t (&li)[R], float &worst,
                                            int &qlen, const float (*queue_v)[kEpiThreads],
                                            const int32_t (*queue_i)[kEpiThreads], int etid) {
    const int rounds = __reduce_max_sync(0xffffffffu, qlen);
#pragma unroll 1
    for (int t = 0; t < rounds; ++t) {
        if (t < qlen) {
            const float x = queue_v[t][etid];
            if (x < worst) {
                list_push<R>(ls, li, x, queue_i[t][etid]);
                worst = ls[R - 1];
            }
        }
    }
    qlen = 0;
    __syncwarp();
}

// One item of work: the query tile of 256 rows from row0 (rows at or past
// qend are not outputs) against candidate rows [lo, hi); `cont`: the item
// extends the previous item's query tile (no reload, lists carry over);
// `more`: a later item extends this one (lists written after the last).
// Without a work list a CTA takes the query tiles blockIdx.x,
// blockIdx.x + gridDim.x, ... of one problem of N rows, each against all N.
struct QueryTile {
    int32_t row0, qend, lo, hi, out_off;  // N < 2^31
    bool cont, more;
};

__device__ __forceinline__ int64_t work_items(const int64_t *__restrict__ work_begin,
                                              int64_t n_qt) {
    if (work_begin) return work_begin[blockIdx.x + 1] - work_begin[blockIdx.x];
    return blockIdx.x < n_qt ? (n_qt - 1 - blockIdx.x) / gridDim.x + 1 : 0;
}

__device__ __forceinline__ QueryTile work_item(const int64_t *__restrict__ work_begin,
                                               const TcItem *__restrict__ work, int64_t it,
                                               int64_t N) {
    QueryTile q;
    if (work_begin) {
        const TcItem w = work[work_begin[blockIdx.x] + it];
        q.row0 = w.row0;
        q.qend = w.qend;
        q.lo = w.lo;
        q.hi = w.hi;
        q.out_off = w.out_off;
        q.cont = (w.flags & kTcContinue) != 0;
        q.more = (w.flags & kTcMore) != 0;
    } else {
        q.row0 = (int32_t)(((int64_t)blockIdx.x + it * gridDim.x) * kQueryTile);
        q.qend = (int32_t)N;
        q.lo = 0;
        q.hi = (int32_t)N;
        q.out_off = 0;
        q.cont = q.more = false;
    }
    return q;
}

template <int R, bool kIP>
__global__ void __launch_bounds__(kThreads, 1)
    knn_select_tc(const __grid_constant__ CUtensorMap tmap,
                  const __grid_constant__ CUtensorMap tmap_c, const float *__restrict__ sqnorm,
                  int64_t N, int ksteps, int katoms, const int64_t *__restrict__ work_begin,
                  const TcItem *__restrict__ work, const int32_t *__restrict__ row_map,
                  int32_t *__restrict__ cand_i, int *__restrict__ err, long long wait_limit,
                  int stall) {
    extern __shared__ uint8_t smem_raw[];
    SharedStorage &s = *reinterpret_cast<SharedStorage *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t n_qt = (N + kQueryTile - 1) / kQueryTile;
    const int64_t n_items = work_items(work_begin, n_qt);
    const uint32_t a_bytes = 2u * katoms * kAtomBytes;
    const uint32_t b_bytes = (uint32_t)katoms * kAtomBytes;

    if (threadIdx.x == 0) {
        // Barriers the MMA issuers commit to take one arrival from each of the two.
        for (int i = 0; i < kStages; ++i) {
            mbar_init(&s.full[i], 1);
            mbar_init(&s.empty[i], 2);
        }
        mbar_init(&s.a_full, 1);
        mbar_init(&s.a_empty, 2);
        // Each query half has its own accumulator hand-off: its MMA warp and
        // its four epilogue warps, so one half's slow tile does not hold the other.
        for (int i = 0; i < 2; ++i)
            for (int hh = 0; hh < 2; ++hh) {
                mbar_init(&s.acc_full[i][hh], 1);
                mbar_init(&s.acc_empty[i][hh], kEpiWarps / 2);
            }
        mbar_init(&s.drain, 2);
        mbar_init(&s.never, 1);
        s.abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&s.tmem_base)),
                     "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    tmem_fence_before();
    __syncthreads();
    tmem_fence_after();
    const uint32_t tmem = s.tmem_base;

    if (warp == 0 && lane == 0) {
        // ---------------------------------------------------------- TMA producer
        int stage = 0;
        uint32_t phase = 0, a_phase = 0;
        uint32_t issued_parity[kStages];
        bool issued[kStages];
        for (int i = 0; i < kStages; ++i) issued[i] = false, issued_parity[i] = 0;
        bool a_issued = false;
        uint32_t a_parity = 0;
        if (stall) mbar_wait(s, &s.never, 0, err, 7, wait_limit);
        for (int64_t it = 0; it < n_items && !s.abort; ++it) {
            const QueryTile q = work_item(work_begin, work, it, N);
            if (!q.cont) {
                if (!mbar_wait(s, &s.a_empty, a_phase ^ 1, err, 1, wait_limit)) break;
                mbar_expect_tx(&s.a_full, a_bytes);
                for (int h = 0; h < 2; ++h)
                    for (int at = 0; at < katoms; ++at)
                        tma_load_2d(s.a[h][at], &tmap, &s.a_full, at * 64,
                                    (int)(q.row0 + h * 128));
                a_issued = true;
                a_parity = a_phase;
                a_phase ^= 1;
            }
            for (int64_t ct = q.lo / kCandTile; ct * kCandTile < q.hi; ++ct) {
                if (!mbar_wait(s, &s.empty[stage], phase ^ 1, err, 2, wait_limit)) break;
                mbar_expect_tx(&s.full[stage], b_bytes);
                for (int at = 0; at < katoms; ++at)
                    tma_load_2d(s.b[stage][at], &tmap_c, &s.full[stage], at * 64,
                                (int)(ct * kCandTile));
                issued[stage] = true;
                issued_parity[stage] = phase;
                if (++stage == kStages) stage = 0, phase ^= 1;
            }
        }
        // Copies still in flight must land before the CTA's shared memory goes away.
        const long long t0 = clock64();
        for (int i = 0; i < kStages; ++i)
            if (issued[i])
                while (!mbar_try_wait(&s.full[i], issued_parity[i]) && clock64() - t0 < kWaitCycles) {
                }
        if (a_issued)
            while (!mbar_try_wait(&s.a_full, a_parity) && clock64() - t0 < kWaitCycles) {
            }
    } else if ((warp == 1 || warp == kMmaWarp1) && lane == 0) {
        // ---------------------------------------------------------- MMA issuers
        // Warp 1 issues query half 0's MMAs, warp kMmaWarp1 half 1's: two
        // schedulers share the descriptor work of a tile.
        const int h = (warp == 1) ? 0 : 1;
        int stage = 0;
        uint32_t phase = 0, a_phase = 0, acc_phase = 0;
        int acc = 0;
        for (int64_t it = 0; it < n_items && !s.abort; ++it) {
            const QueryTile q = work_item(work_begin, work, it, N);
            if (!q.cont) {
                if (!mbar_wait(s, &s.a_full, a_phase, err, 3, wait_limit)) break;
                a_phase ^= 1;
            }
            tmem_fence_after();
            for (int64_t ct = q.lo / kCandTile; ct * kCandTile < q.hi; ++ct) {
                if (!mbar_wait(s, &s.acc_empty[acc][h], acc_phase ^ 1, err, 4, wait_limit)) break;
                if (!mbar_wait(s, &s.full[stage], phase, err, 5, wait_limit)) break;
                tmem_fence_after();
                {
                    const uint32_t d_tmem = tmem + (uint32_t)(acc * 256 + h * 128);
                    for (int ks = 0; ks < ksteps; ++ks) {
                        const int at = ks >> 2;
                        const uint32_t off = (uint32_t)(ks & 3) * 32;
                        const uint64_t ad = smem_desc(smem_u32(s.a[h][at]) + off);
                        const uint64_t bd = smem_desc(smem_u32(s.b[stage][at]) + off);
                        umma_bf16(d_tmem, ad, bd, ks > 0 ? 1u : 0u);
                    }
                }
                umma_commit(&s.empty[stage]);
                umma_commit(&s.acc_full[acc][h]);
                if (++stage == kStages) stage = 0, phase ^= 1;
                acc ^= 1;
                if (acc == 0) acc_phase ^= 1;
            }
            if (!q.more) umma_commit(&s.a_empty);
        }
        // Every issued MMA completes before TMEM is released.
        umma_commit(&s.drain);
        const long long t0 = clock64();
        while (!mbar_try_wait(&s.drain, 0) && clock64() - t0 < kWaitCycles) {
        }
    } else if (warp >= kEpiWarp0 && warp < kEpiWarp0 + kEpiWarps) {
        // ---------------------------------------------------------- epilogue
        const int h = (warp - kEpiWarp0) >> 2;
        const int quad = warp & 3;
        const int etid = threadIdx.x - kEpiWarp0 * 32;
        const int row_in_tile = h * 128 + quad * 32 + lane;
        // Accumulator columns per tcgen05.ld: 32 with 32-entry lists; 64-entry
        // lists leave registers for 16.
        constexpr int kC = R <= 32 ? 32 : 16;
        uint32_t acc_phase = 0;
        int acc = 0;
        float ls[R];
        int32_t li[R];
        float worst = FLT_MAX;
        int qlen = 0;
        for (int64_t it = 0; it < n_items; ++it) {
            // Lanes read the abort flag at different times: the warp stops as one.
            if (__any_sync(0xffffffffu, s.abort != 0)) break;
            const QueryTile q = work_item(work_begin, work, it, N);
            const int64_t grow = q.row0 + row_in_tile;
            const bool live = grow < q.qend;
            if (!q.cont) {
#pragma unroll
                for (int t = 0; t < R; ++t) {
                    ls[t] = FLT_MAX;
                    li[t] = -1;
                }
                worst = FLT_MAX;
                qlen = 0;
            }
            bool ok = true;
            for (int64_t ct = q.lo / kCandTile; ct * kCandTile < q.hi; ++ct) {
                const bool got = mbar_wait(s, &s.acc_full[acc][h], acc_phase, err, 6, wait_limit);
                if (!__all_sync(0xffffffffu, got)) {
                    ok = false;
                    break;
                }
                tmem_fence_after();
                const int64_t c0 = ct * kCandTile;
                // A tile reaching outside [lo, hi): its outside columns are masked.
                const bool tail = c0 < q.lo || c0 + kCandTile > q.hi;
#pragma unroll 1
                for (int chunk = 0; chunk < kCandTile / kC; ++chunk) {
                    float v[kC];
                    __syncwarp();
                    tmem_ld(tmem + ((uint32_t)(quad * 32) << 16) +
                                (uint32_t)(acc * 256 + h * 128 + chunk * kC),
                            v);
                    if (chunk == kCandTile / kC - 1) {
                        // The tile's last columns are in registers: the
                        // accumulator goes back to the MMA warp before their
                        // scan, so the next MMAs into it start meanwhile.
                        tmem_fence_before();
                        __syncwarp();
                        if (lane == 0) mbar_arrive(&s.acc_empty[acc][h]);
                    }
                    const int64_t cb = c0 + chunk * kC;
                    // Scores, lower is better: |c|^2 - 2<q,c> (squared L2) or
                    // -<q,c> (kept as +<q,c>, compared against -worst).
                    if constexpr (!kIP) {
                        // The chunk's candidate norms, the same for every lane:
                        // 16-byte loads where the chunk lies inside the rows.
                        if (cb >= q.lo && cb + kC <= q.hi) {
#pragma unroll
                            for (int j = 0; j < kC; j += 4) {
                                const float4 nc =
                                    __ldg(reinterpret_cast<const float4 *>(sqnorm + cb + j));
                                v[j] = fmaf(-2.f, v[j], nc.x);
                                v[j + 1] = fmaf(-2.f, v[j + 1], nc.y);
                                v[j + 2] = fmaf(-2.f, v[j + 2], nc.z);
                                v[j + 3] = fmaf(-2.f, v[j + 3], nc.w);
                            }
                        } else {
#pragma unroll
                            for (int j = 0; j < kC; ++j) {
                                const int64_t c = cb + j;
                                const float nc =
                                    (c >= q.lo && c < q.hi) ? __ldg(sqnorm + c) : 0.f;
                                v[j] = fmaf(-2.f, v[j], nc);
                            }
                        }
                    }
                    if (tail) {
#pragma unroll
                        for (int j = 0; j < kC; ++j)
                            if (cb + j < q.lo || cb + j >= q.hi) v[j] = kIP ? -FLT_MAX : FLT_MAX;
                    }
                    // Best score of each 8-column group, then of the chunk.
                    constexpr int kG = kC / 8;
                    float gb[kG];
#pragma unroll
                    for (int g = 0; g < kG; ++g) {
                        const float *w = v + 8 * g;
                        gb[g] = kIP ? -max3f(max3f(w[0], w[1], w[2]), max3f(w[3], w[4], w[5]),
                                             fmaxf(w[6], w[7]))
                                    : min3f(min3f(w[0], w[1], w[2]), min3f(w[3], w[4], w[5]),
                                            fminf(w[6], w[7]));
                    }
                    const float best = tree_reduce<false, kG>(gb);
                    const bool hit = live && best < worst;
                    if (!__any_sync(0xffffffffu, hit)) continue;
                    // Qualifying candidates are queued 16 columns at a time,
                    // looking only into the 8-column groups whose best beats
                    // the row's worst; a queue past half full is flushed into
                    // the lists first.
#pragma unroll
                    for (int half = 0; half < kC / 16; ++half) {
                        if (__any_sync(0xffffffffu, qlen > kQueue - 16))
                            flush_queue<R>(ls, li, worst, qlen, s.queue_v, s.queue_i, etid);
                        if (hit) {
#pragma unroll
                            for (int g = 2 * half; g < 2 * half + 2; ++g) {
                                if (gb[g] < worst) {
#pragma unroll
                                    for (int j = 8 * g; j < 8 * g + 8; ++j) {
                                        const float x = kIP ? -v[j] : v[j];
                                        if (x < worst) {
                                            s.queue_v[qlen][etid] = x;
                                            s.queue_i[qlen][etid] = (int32_t)(cb + j);
                                            ++qlen;
                                        }
                                    }
                                }
                            }
                        }
                    }
                }
                acc ^= 1;
                if (acc == 0) acc_phase ^= 1;
                // Queues past half full are flushed here, after the accumulator
                // is released, so that the MMAs of the next tiles go on meanwhile;
                // a flush inside the tile happens only when one tile overfills a
                // queue (early in the sweep).
                if (__any_sync(0xffffffffu, qlen > kQueue - 16))
                    flush_queue<R>(ls, li, worst, qlen, s.queue_v, s.queue_i, etid);
            }
            if (!ok) break;
            if (q.more) continue;  // the next item extends this query tile
            flush_queue<R>(ls, li, worst, qlen, s.queue_v, s.queue_i, etid);
            if (live) {
                const int64_t orow = row_map ? (int64_t)row_map[grow] : grow + q.out_off;
#pragma unroll
                for (int t = 0; t < R; ++t)
                    cand_i[orow * R + t] =
                        li[t] < 0 ? -1
                                  : (row_map ? row_map[li[t]] : (int32_t)(li[t] + q.out_off));
            }
        }
    }
    __syncthreads();
    if (warp == 1) {
        tmem_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(kTmemCols));
    }
}

// The driver's tensor-map encoder, looked up once (thread-safe static
// initialisation; a failed lookup throws and is retried on the next call).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        NCVIS_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                                    cudaEnableDefault, &q));
        require(q == cudaDriverEntryPointSuccess && p != nullptr,
                "knn: cuTensorMapEncodeTiled is unavailable", kCudaError);
        return (PFN_cuTensorMapEncodeTiled_v12000)p;
    }();
    return fn;
}

}  // namespace

KnnTcPlan plan_knn_tc(int64_t N, int D, int k, int rerank_factor, int dist) {
    KnnTcPlan p;
    // Default: 2k candidates (32 for k = 15), which measured recall@15 = 1.0
    // against FP64 search at 1,024,000 x 100; rerank_factor = 4 keeps 64.
    if (rerank_factor <= 0) rerank_factor = 2;
    const int64_t want = std::max<int64_t>((int64_t)rerank_factor * k, (int64_t)k + 1);
    p.R = want <= 32 ? 32 : 64;  // the kernel keeps 32 or 64 candidates per point
    // Squared L2 folds -|c|^2 / 2 into two extra K columns when they fit (D <= 126).
    p.fold = (dist == kSquaredL2) && D + 2 <= 64 * kMaxAtoms;
    p.ldb = (D + (p.fold ? 2 : 0) + 7) / 8 * 8;
    p.Npad = N;
    (void)N;
    return p;
}

bool knn_tc_supported(int D, int R) { return D >= 1 && D <= 64 * kMaxAtoms && (R == 32 || R == 64); }


namespace {

void encode_rows(const __nv_bfloat16 *base, int64_t rows, int ldb, CUtensorMap &map) {
    cuuint64_t dims[2] = {(cuuint64_t)ldb, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)ldb * 2};
    cuuint32_t box[2] = {64, 128};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = tensor_map_encoder()(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void *)base,
                                      dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                      CU_TENSOR_MAP_SWIZZLE_128B,
                                      CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    require(r == CUDA_SUCCESS,
            "knn: cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")", kCudaError);
}

void launch_select(const CUtensorMap &map, const CUtensorMap &map_c, const float *sqnorm,
                   int64_t N, const KnnTcPlan &plan, bool ip, int32_t *cand_i, int *timeout_flag,
                   cudaStream_t s, const TcWork *work) {
    const int ksteps = (plan.ldb + 15) / 16;
    const int katoms = (ksteps * 16 + 63) / 64;
    const size_t smem = sizeof(SharedStorage) + 1024;
    const int64_t n_qt = (N + kQueryTile - 1) / kQueryTile;
    const unsigned grid =
        work ? (unsigned)work->ctas : (unsigned)std::min<int64_t>(n_qt, num_sms());
    const int64_t *work_begin = work ? work->begin : nullptr;
    const TcItem *items = work ? work->items : nullptr;
    const int32_t *row_map = work ? work->map : nullptr;
    if (grid == 0) return;
    auto go = [&](auto kernel) {
        NCVIS_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem));
        NCVIS_LAUNCH(kernel, grid, kThreads, smem, s, map, map_c, sqnorm, N, ksteps, katoms,
                     work_begin, items, row_map, cand_i, timeout_flag,
                     plan.wait_cycles > 0 ? plan.wait_cycles : kWaitCycles, plan.stall ? 1 : 0);
    };
    if (plan.R == 8)
        ip ? go(knn_select_tc<8, true>) : go(knn_select_tc<8, false>);
    else if (plan.R == 32)
        ip ? go(knn_select_tc<32, true>) : go(knn_select_tc<32, false>);
    else
        ip ? go(knn_select_tc<64, true>) : go(knn_select_tc<64, false>);
}

void check_plan(const KnnTcPlan &plan) {
    const int ksteps = (plan.ldb + 15) / 16;
    const int katoms = (ksteps * 16 + 63) / 64;
    require(katoms <= kMaxAtoms, "knn: the tensor-core path supports D <= 128", kUnsupported);
    require(plan.R == 8 || plan.R == 32 || plan.R == 64,
            "knn: the tensor-core kernel keeps 8, 32 or 64 candidates");
}

}  // namespace

void launch_knn_select_tc(const __nv_bfloat16 *Xb, const float *sqnorm, int64_t N,
                          const KnnTcPlan &plan, int dist, int32_t *cand_i, float * /*cand_d*/,
                          int *timeout_flag, cudaStream_t s, const TcWork *work,
                          const __nv_bfloat16 *Xc) {
    require(N < (int64_t(1) << 31), "knn: N must be below 2^31");
    check_plan(plan);
    require(((uintptr_t)Xb & 15) == 0, "knn: BF16 rows must be 16-byte aligned");
    require(((uintptr_t)sqnorm & 15) == 0, "knn: squared norms must be 16-byte aligned");
    require(!plan.fold || (Xc && ((uintptr_t)Xc & 15) == 0),
            "knn: the folded squared-L2 mode needs a 16-byte aligned candidate copy");
    // Queries come from Xb, candidates from Xc in the folded mode (else Xb).
    CUtensorMap map, map_c;
    encode_rows(Xb, N, plan.ldb, map);
    encode_rows(plan.fold ? Xc : Xb, N, plan.ldb, map_c);
    // The folded squared-L2 product <q, c> - |c|^2 / 2 ranks like an inner product.
    const bool ip = dist != kSquaredL2 || plan.fold;
    launch_select(map, map_c, sqnorm, N, plan, ip, cand_i, timeout_flag, s, work);
}

void launch_knn_select_tc_pair(const __nv_bfloat16 *Q, int64_t nq, const __nv_bfloat16 *Cm,
                               int64_t nc, const float *c_sqnorm, const KnnTcPlan &plan, bool ip,
                               int32_t *cand_i, int *timeout_flag, cudaStream_t s,
                               const TcWork &work) {
    require(nq < (int64_t(1) << 31) && nc < (int64_t(1) << 31), "knn: rows must be below 2^31");
    check_plan(plan);
    require((((uintptr_t)Q | (uintptr_t)Cm) & 15) == 0, "knn: BF16 rows must be 16-byte aligned");
    require(ip || (c_sqnorm && ((uintptr_t)c_sqnorm & 15) == 0),
            "knn: squared L2 without folded norms needs 16-byte aligned candidate norms");
    CUtensorMap map, map_c;
    encode_rows(Q, nq, plan.ldb, map);
    encode_rows(Cm, nc, plan.ldb, map_c);
    launch_select(map, map_c, c_sqnorm, nq, plan, ip, cand_i, timeout_flag, s, &work);
}

}  // namespace ncvis_gpu
