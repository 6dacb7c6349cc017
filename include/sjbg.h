/*
 * sjbg.h - C ABI of the GB300 stream-join library (libsjbg.so).
 *
 * The library is a drop-in for the windowed stream-join execution path of
 * gpu-stream-join-benchmark: the joiner interfaces
 *   Windowing::Lazy::Executor::BaseLazyExecutor::execute
 *       (include/sjb/windowing/lazy/executor/BaseLazyExecutor.hpp:26-30)
 *   Windowing::Eager::Executor::BaseEagerExecutor::{execute,clearStates,onEndOfStream}
 *       (include/sjb/windowing/eager/executor/BaseEagerExecutor.hpp:16-20)
 * and the executor selection of WindowingFactory::create
 *       (src/sjb/windowing/WindowingFactory.cpp:52-298).
 *
 * Conventions
 *  - Plain C, no exceptions cross the boundary, every entry point returns an
 *    int status (SJBG_OK or an SJBG_E_* code); sjbg_last_error() gives text.
 *    The reference instead calls exit(1) through CUDA_CHECK
 *    (include/sjb/utils/ErrorChecking.cuh:7-14) and throws
 *    std::runtime_error("Not Implemented") for unsupported combinations
 *    (WindowingFactory.cpp:86,123,211,264,283); those become SJBG_E_CUDA and
 *    SJBG_E_UNSUPPORTED here.
 *  - Input spans are host memory (pinned or pageable) or device memory, named
 *    by the `mem` argument (SJBG_MEM_HOST / SJBG_MEM_DEVICE).
 *  - One handle is used by one host thread at a time (the reference's lazy
 *    joiner pool gives each window to one executor, CountBased.cuh:129-138).
 *  - "left" = stream R = build side, "right" = stream S = probe side, as in
 *    CPU_HJ::execute (src/sjb/windowing/lazy/executor/CPU/CPU_HJ.cpp:41-65).
 *  - Join predicate: equal 32-bit keys (CPU_NLJ.cpp:18-27).
 *
 * Per-window result (sjbg_window_result):
 *  count          number of matching (left, right) tuple pairs; this is the
 *                 reference's ExecutionStatistic::resultCount
 *                 (include/sjb/utils/ExecutionStatistic.hpp:6-20).
 *  xor_checksum   XOR over pairs of splitmix64((u64)left.val << 32 | right.val);
 *                 computed only when pairs are enumerated (SJBG_F_XOR or a
 *                 pair-writing result mode), flagged by SJBG_WR_XOR.
 *  prod_checksum  sum over pairs of fr(left.val) * gs(right.val) mod 2^64
 *                 (fr, gs: odd 64-bit hashes, see csrc/sjbg_gen.h); always
 *                 computed, in O(|L|+|R|), also for windows whose pairs
 *                 cannot be enumerated.
 *  pairs          optional (left.val, right.val) list, unsorted.
 */
#ifndef SJBG_H
#define SJBG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SJBG_ABI_VERSION 1

#if defined(__GNUC__)
#define SJBG_API __attribute__((visibility("default")))
#else
#define SJBG_API
#endif

/* 16-byte stream tuple, layout of the reference's Tuple
 * (include/sjb/utils/Tuple.hpp:6-11). */
typedef struct sjbg_tuple {
    uint32_t key;
    uint32_t val;
    uint64_t ts;
} sjbg_tuple;

/* One join result: val of the left tuple and val of the right tuple.  It
 * replaces the reference's 32-byte ResultTuple (include/sjb/utils/ResultTuple.hpp:5-13):
 * keys are equal by construction and the timestamps are recoverable from the
 * inputs, so 8 bytes per pair are written instead of 32. */
typedef struct sjbg_pair {
    uint32_t r;
    uint32_t s;
} sjbg_pair;

/* ---- status codes ---------------------------------------------------------- */
enum {
    SJBG_OK = 0,
    SJBG_E_INVALID = 1,     /* bad argument */
    SJBG_E_NOMEM = 2,       /* device or host allocation failed */
    SJBG_E_CUDA = 3,        /* a CUDA runtime call failed */
    SJBG_E_TIMEOUT = 4,     /* a bounded device-side wait gave up */
    SJBG_E_CAPACITY = 5,    /* a window exceeds max_tuples_per_window */
    SJBG_E_UNSUPPORTED = 6, /* combination not provided (reference: "Not Implemented") */
    SJBG_E_BUDGET = 7,      /* streaming admission refused: over the HBM budget */
    SJBG_E_STATE = 8,       /* call out of order (e.g. eager call on a lazy handle) */
    SJBG_E_MISMATCH = 9     /* SJBG_F_VERIFY: learned and radix results differ */
};

/* ---- enumerations mirroring the reference's (include/sjb/windowing/BaseWindowing.cuh:9-41) */
enum { SJBG_ALG_NLJ = 1, SJBG_ALG_HJ = 2, SJBG_ALG_SMJ = 3 };          /* ALGORITHM_TYPE */
enum { SJBG_EAGER = 0, SJBG_LAZY = 1 };                                /* PROGRESSIVENESS_TYPE */
enum {                                                                 /* RESULT_WRITING_METHOD */
    SJBG_RESULT_NO_OUTPUT = 0,             /* count + checksums only */
    SJBG_RESULT_COUNT_KERNEL = 1,          /* count pass, then exact pair write pass */
    SJBG_RESULT_ESTIMATED_SELECTIVITY = 2, /* single pass into the caller's buffer */
    SJBG_RESULT_BITMAP = 3,                /* NLJ: single pass, match masks decoded on device */
    SJBG_RESULT_ATOMIC = 4                 /* single pass, atomic range reservation */
};

/* Hash-join partitioning (no reference counterpart). */
enum {
    SJBG_PART_AUTO = 0,    /* library picks (autotuner when SJBG_F_AUTOTUNE) */
    SJBG_PART_NONE = 1,    /* one open-addressing table per window in HBM */
    SJBG_PART_RADIX = 2,   /* radix partitioning on key bits, shared-memory tables */
    SJBG_PART_LEARNED = 3  /* learned key-CDF partitioning, radix fallback */
};

/* Memory kind of caller buffers. */
enum { SJBG_MEM_HOST = 0, SJBG_MEM_DEVICE = 1 };

/* sjbg_config.flags */
#define SJBG_F_XOR      0x1u  /* enumerate pairs to compute xor_checksum */
#define SJBG_F_PROFILE  0x2u  /* time every kernel launch with CUDA events */
#define SJBG_F_AUTOTUNE 0x4u  /* pick buckets / tiles / fan-out by measurement */
#define SJBG_F_VERIFY   0x8u  /* learned partitioning: also run radix and compare */
#define SJBG_F_GRAPH    0x10u /* capture batched lazy calls on device inputs in a CUDA graph, replay repeats */
#define SJBG_F_PERSISTENT 0x20u /* eager: one resident kernel takes batches from a queue (the reference's usePK) */

/* sjbg_window_result.flags */
#define SJBG_WR_XOR             0x1u /* xor_checksum is valid */
#define SJBG_WR_PAIRS_TRUNCATED 0x2u /* more pairs than pairs_capacity; n_pairs = capacity */
#define SJBG_WR_FALLBACK        0x4u /* learned model overflowed; radix was used */
#define SJBG_WR_RADIX_BY_COST   0x8u /* learned partitioner chose radix: balanced on the sample, few heavy tuples */

/* Executor configuration.  Field meanings follow the reference's
 * AlgorithmConfig / DataConfig / QueryConfig / EngineConfig
 * (include/experiment/Config.hpp:17-52). */
typedef struct sjbg_config {
    uint32_t algorithm;             /* SJBG_ALG_*         (AlgorithmConfig::underlyingAlgorithm) */
    uint32_t progressiveness;       /* SJBG_LAZY/EAGER    (AlgorithmConfig::progressiveness) */
    uint32_t result_mode;           /* SJBG_RESULT_*      (AlgorithmConfig::resultWritingMethod) */
    uint32_t partitioner;           /* SJBG_PART_*        (hash join only) */
    uint64_t batch_size;            /* tuples per batch   (DataConfig::batchSize) */
    uint64_t max_tuples_per_window; /* per side           (EngineConfig::maxTupleInWindow) */
    uint64_t window_size;           /* eager window length per side (QueryConfig::windowSize) */
    uint64_t num_distinct_keys;     /* key-domain hint    (DataConfig::numDistinctKey); 0 = unknown */
    uint32_t flags;                 /* SJBG_F_* */
    uint32_t radix_bits;            /* partition fan-out log2 (<= 14); 0 = about 4096 left tuples per bucket */
    uint32_t learned_leaves;        /* leaf segments of the CDF model, 0 = 256 */
    float sample_rate;              /* learned: fraction of tuples sampled, 0 = 0.01 */
    float overflow_bound;           /* learned: worst partition / mean partition allowed, 0 = 8 */
    int32_t device;                 /* CUDA device ordinal */
    uint64_t hbm_budget_bytes;      /* streaming admission budget, 0 = no limit */
    uint32_t idle_timeout_ms;       /* SJBG_F_PERSISTENT: longest wait of the kernel for the next batch, 0 = 1000 */
    uint32_t reserved;              /* 0 */
} sjbg_config;

typedef struct sjbg_window_result {
    uint64_t count;
    uint64_t xor_checksum;
    uint64_t prod_checksum;
    uint64_t n_pairs;          /* pairs written to the caller's buffer */
    uint32_t status;           /* SJBG_OK or SJBG_E_* for this window */
    uint32_t flags;            /* SJBG_WR_* */
    uint32_t partitioner_used; /* SJBG_PART_* actually used */
    float ms;                  /* device time of the call that produced it */
} sjbg_window_result;

/* One window of a batched call: spans into the left / right arrays and into
 * the shared pair buffer. */
typedef struct sjbg_window_desc {
    uint64_t left_offset;
    uint64_t n_left;
    uint64_t right_offset;
    uint64_t n_right;
    uint64_t pairs_offset;   /* first pair slot of this window */
    uint64_t pairs_capacity; /* 0 = do not write pairs for this window */
} sjbg_window_desc;

typedef struct sjbg_handle sjbg_handle;

/* ---- lifetime --------------------------------------------------------------
 * Replaces the executor constructors that allocate device buffers sized by
 * maxTupleInWindow (e.g. src/sjb/windowing/lazy/executor/GPU/GPU_HJ.cu:266-287)
 * and the selection in WindowingFactory::create (WindowingFactory.cpp:52-298). */
SJBG_API int sjbg_create(const sjbg_config *cfg, sjbg_handle **out);
/* Replaces the executor destructors (GPU_HJ.cu:289-309). */
SJBG_API int sjbg_destroy(sjbg_handle *h);
/* Text of the last error on this handle (or of the last failed create when h is NULL). */
SJBG_API const char *sjbg_last_error(const sjbg_handle *h);
/* Run subsequent work on this CUDA stream (cudaStream_t passed as void*); NULL = the handle's own. */
SJBG_API int sjbg_set_stream(sjbg_handle *h, void *cuda_stream);
/* Library / ABI version. */
SJBG_API int sjbg_version(void);

/* ---- lazy windows ------------------------------------------------------------
 * One window: all left tuples against all right tuples.  Replaces
 * BaseLazyExecutor::execute (BaseLazyExecutor.hpp:26-30) once the caller has
 * the window's batches as contiguous spans.  pairs may be NULL. */
SJBG_API int sjbg_lazy_execute(sjbg_handle *h,
                      const sjbg_tuple *left, uint64_t n_left,
                      const sjbg_tuple *right, uint64_t n_right,
                      uint32_t mem,
                      sjbg_pair *pairs, uint64_t pairs_capacity,
                      sjbg_window_result *out);

/* The reference's exact argument form: ring buffers plus the tuple offsets of
 * the window's batches (each batch_size tuples long), as CountBased::execute
 * pops them (include/sjb/windowing/lazy/CountBased.cuh:112-138).  Host rings. */
SJBG_API int sjbg_lazy_execute_ring(sjbg_handle *h,
                           const sjbg_tuple *left_ring, const uint64_t *left_batch_offsets, uint64_t n_left_batches,
                           const sjbg_tuple *right_ring, const uint64_t *right_batch_offsets, uint64_t n_right_batches,
                           sjbg_pair *pairs, uint64_t pairs_capacity,
                           sjbg_window_result *out);

/* Many windows in one call (no reference counterpart: the reference runs one
 * window per executor call).  `windows` and `out` are host arrays; `left`,
 * `right` and `pairs` are in memory of kind `mem`. */
SJBG_API int sjbg_lazy_execute_batch(sjbg_handle *h,
                            const sjbg_tuple *left, const sjbg_tuple *right, uint32_t mem,
                            const sjbg_window_desc *windows, uint32_t n_windows,
                            sjbg_pair *pairs,
                            sjbg_window_result *out);

/* ---- eager windows -----------------------------------------------------------
 * One incoming batch: join it against the other side's state of the current
 * window, then add it to its own side's state.  Returns the batch's new
 * matches in *match_count.  Replaces BaseEagerExecutor::execute
 * (BaseEagerExecutor.hpp:16; e.g. eager CPU_HJ::execute,
 * src/sjb/windowing/eager/executor/CPU/CPU_HJ.cpp:35-48). */
SJBG_API int sjbg_eager_execute(sjbg_handle *h, const sjbg_tuple *batch, uint64_t n, int is_left,
                       uint32_t mem, uint64_t *match_count);
/* Close the current window and reset both sides' state.  Replaces
 * BaseEagerExecutor::clearStates (BaseEagerExecutor.hpp:18). */
SJBG_API int sjbg_eager_clear_states(sjbg_handle *h);
/* Totals of the current (not yet cleared) window, including checksums and
 * pairs written so far by sjbg_eager_execute. */
SJBG_API int sjbg_eager_window_result(sjbg_handle *h, sjbg_pair *pairs, uint64_t pairs_capacity,
                             sjbg_window_result *out);
/* Replaces BaseEagerExecutor::onEndOfStream (BaseEagerExecutor.hpp:20). */
SJBG_API int sjbg_eager_end_of_stream(sjbg_handle *h);

/* A whole recorded eager stream in one call: n_batches left batches and
 * n_batches right batches of batch_size tuples, with the results of feeding
 * them in the reference's order L0, R0, L1, R1, ...
 * (src/sjb/source/Source.cpp:20-28) with a window closed whenever either side
 * has received window_size tuples
 * (include/sjb/windowing/eager/CountBased.cuh:38-46).  All windows are joined
 * together on the device (nested-loop: one grid over every batch pair; hash
 * and sort-merge: one stable sort per window for the batch counts plus the
 * lazy join of the windows).  batch_counts (host, 2*n_batches entries, may be
 * NULL) receives each batch's new matches in arrival order; out (host, one
 * entry per window) receives the window totals, and entries past the last
 * window get status SJBG_E_INVALID. */
SJBG_API int sjbg_eager_run(sjbg_handle *h, const sjbg_tuple *left, const sjbg_tuple *right,
                   uint64_t n_batches, uint32_t mem,
                   uint64_t *batch_counts, sjbg_window_result *out, uint32_t n_windows_out);

/* ---- persistent eager joins (SJBG_F_PERSISTENT) ----------------------------------
 * Replaces the reference's persistent-kernel executor GPU_HJ_PK
 * (src/sjb/windowing/eager/executor/GPU/GPU_HJ_PK.cu:10-89,101-180; chosen by
 * EagerJoinConfig::usePK, include/experiment/Config.hpp:15).  On an eager
 * handle created with SJBG_F_PERSISTENT, one cooperative kernel stays resident
 * on the device and takes tickets (batches, and the clear / report / stop
 * commands behind sjbg_eager_clear_states, sjbg_eager_window_result and
 * sjbg_eager_end_of_stream) from a queue in mapped host memory, in order.
 * sjbg_eager_execute then posts its batch and reads the count from a mapped
 * result slot: no launch, copy-engine transfer or stream synchronisation per
 * batch.  Pinned host batches are read by the kernel in place; pageable ones
 * are copied into the queue.  Hash join (HJ) takes up to 32 SMs; nested-loop
 * and sort-merge joins take the whole GPU while the kernel runs, so other
 * work on the device waits until sjbg_eager_end_of_stream stops it or its
 * wait for the next batch runs out (idle_timeout_ms).  The window state stays
 * in device memory when the kernel returns; the next batch relaunches it. */

/* Post one batch without waiting; *ticket names it for sjbg_eager_wait.  A host
 * batch is copied before the call returns; a device batch (16-byte aligned)
 * is read in place and must stay unchanged until its ticket completes. */
SJBG_API int sjbg_eager_post(sjbg_handle *h, const sjbg_tuple *batch, uint64_t n, int is_left, uint32_t mem,
                             uint64_t *ticket);
/* Wait for a posted batch (one of the last 64 posted) and return its new
 * matches.  SJBG_E_TIMEOUT when the kernel does not answer within
 * idle_timeout_ms + 2 s or one of its bounded device-side waits gave up (the
 * handle then refuses batches until sjbg_eager_clear_states). */
SJBG_API int sjbg_eager_wait(sjbg_handle *h, uint64_t ticket, uint64_t *match_count);
/* Whether the kernel is resident, and how often it was launched.  Returns
 * SJBG_E_TIMEOUT once after the kernel returned because its wait for the next
 * batch ran out (its device status word then holds the timeout bit); SJBG_OK
 * otherwise. */
SJBG_API int sjbg_eager_pk_status(sjbg_handle *h, int *running, uint64_t *launches);

/* ---- streaming loop (no reference counterpart) --------------------------------
 * Event-time tumbling windows of window_ns, admitted under hbm_budget_bytes. */
typedef struct sjbg_stream_stats {
    uint64_t windows_closed;
    uint64_t tuples_joined;
    uint64_t windows_rejected;
    uint64_t fallbacks;
    double p50_ms;
    double p99_ms;
    double busy_ms;
} sjbg_stream_stats;

/* One closed event-time window: its result (n_pairs is 0: the loop writes
 * no pairs), the window's id (tuples with floor(ts / window_ns) == window_id)
 * and how many tuples each side contributed. */
typedef struct sjbg_stream_window {
    sjbg_window_result result;
    uint64_t window_id;
    uint64_t n_left;
    uint64_t n_right;
} sjbg_stream_window;

SJBG_API int sjbg_stream_open(sjbg_handle *h, uint64_t window_ns);
/* Push one batch (ts = event time in ns, non-decreasing per side). */
SJBG_API int sjbg_stream_push(sjbg_handle *h, const sjbg_tuple *batch, uint64_t n, int is_left, uint32_t mem);
/* Retrieve closed windows' results in window-id order; *n_out receives how many were written. */
SJBG_API int sjbg_stream_poll(sjbg_handle *h, sjbg_stream_window *out, uint32_t max_out, uint32_t *n_out);
SJBG_API int sjbg_stream_close(sjbg_handle *h, sjbg_stream_stats *stats);

/* ---- device-resident ingest ring (count-based lazy windows) ----------------------
 * Replaces the pinned host ring of Windowing::Lazy::CountBased
 * (include/sjb/windowing/lazy/CountBased.cuh:45-101: incoming batches are
 * memmoved into a pinned ring, and a joiner copies each full window to the
 * device per call).  The ring lives in HBM: `depth` slots of window_tuples
 * tuples per side; tuples [kW, (k+1)W) of each side in arrival order form
 * window k (the reference's tumbling count window).  sjbg_ring_push copies a
 * batch straight into its slot on a copy stream (split where it crosses a
 * window boundary); once both sides have filled window k its join (the
 * handle's lazy algorithm, count and checksums, no pairs) is enqueued behind
 * those copies only, so ingest of window k + 1 overlaps the join of window k.
 * A pinned host batch is read asynchronously: keep it unchanged until
 * sjbg_ring_poll has reported every window it contributes to, or
 * sjbg_ring_close has returned.  A side that gets `depth` windows ahead of the
 * other makes the push fail with SJBG_E_CAPACITY ("Ring buffer is full", where
 * the reference exits).  Partial windows at close are not joined, as in the
 * reference. */
SJBG_API int sjbg_ring_open(sjbg_handle *h, uint64_t window_tuples, uint32_t depth);
SJBG_API int sjbg_ring_push(sjbg_handle *h, const sjbg_tuple *batch, uint64_t n, int is_left, uint32_t mem);
/* Finished windows in window order (window_id = k; ms = device time from the
 * window's last copy to the end of its join). */
SJBG_API int sjbg_ring_poll(sjbg_handle *h, sjbg_stream_window *out, uint32_t max_out, uint32_t *n_out);
/* Wait for every enqueued join; stats: windows joined, tuples, p50/p99 of ms. */
SJBG_API int sjbg_ring_close(sjbg_handle *h, sjbg_stream_stats *stats);

/* ---- synthetic inputs on the device ---------------------------------------------
 * Fill n tuples of a stream (global indices first..first+n-1) in device memory:
 * key uniform in [0, domain) when zipf_table is NULL, else Zipf rank from the
 * table (device memory, `domain` entries, see sjbg_gen.h) mapped through the
 * seeded permutation; val = (u32)index, ts = index. */
SJBG_API int sjbg_generate(sjbg_handle *h, sjbg_tuple *dev_out, uint64_t first, uint64_t n,
                  uint64_t seed, uint64_t domain, const uint64_t *zipf_table, uint64_t perm_seed);

/* Host-only helper of sjbg_generate: fill table[0..n) with the Zipf(z) CDF over
 * ranks 0..n-1 in 64-bit fixed point (the layout sjbg_generate expects). */
SJBG_API int sjbg_zipf_table(uint64_t *table, uint64_t n, double z);

/* ---- allocation-free lazy hash join ------------------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory (a host framework that owns every device allocation, or a
 * steady-state loop that must not allocate): the lazy hash join of one window
 * (count and prod_checksum; radix partitioning) that allocates nothing and
 * copies nothing from the host.  left/right (n_left, n_right <= 2^20 tuples,
 * else SJBG_E_CAPACITY) and out are DEVICE memory; the work is enqueued on
 * cuda_stream (NULL = the legacy default stream) and out is written when it
 * completes, with out->status carrying what the kernels reported on the
 * device (SJBG_OK, or SJBG_E_TIMEOUT / SJBG_E_CAPACITY).  The return value
 * covers the argument checks and the launches.  Needs no handle.  Its scratch is a fixed 17 MiB device array
 * that every GPU loading the library holds until exit; the first call on a
 * device looks up that array's address and should come before any stream
 * capture.  Calls share the array: calls that overlap on the GPU race and
 * must be serialised by the caller. */
SJBG_API int sjbg_lazy_hj_noalloc(const sjbg_tuple *left, uint64_t n_left, const sjbg_tuple *right,
                                  uint64_t n_right, sjbg_window_result *out, void *cuda_stream);

/* ---- kernel profile (SJBG_F_PROFILE) ---------------------------------------------
 * Per kernel name: launches and summed CUDA-event time since the last reset. */
SJBG_API int sjbg_kernel_stats(sjbg_handle *h, uint32_t index, char *name, size_t name_len,
                      uint64_t *launches, double *total_ms);
SJBG_API int sjbg_kernel_stats_reset(sjbg_handle *h);

/* Kernel launches issued by this handle since creation (a replayed graph
 * counts each kernel it runs). */
SJBG_API uint64_t sjbg_launch_count(const sjbg_handle *h);

#ifdef __cplusplus
}
#endif

#endif /* SJBG_H */
