// runtime.h - host-side runtime shared by the library's translation units:
// the handle, its device workspace, kernel launch bookkeeping and profiling.
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "../../include/sjbg.h"
#include "common.cuh"

namespace sjbg {

// Named device workspace slots (contents are scratch unless noted).
enum WsSlot : int {
    WS_IN_LEFT, WS_IN_RIGHT,         // staging copies of host inputs
    WS_PART_LEFT, WS_PART_RIGHT,     // partitioned (key,val) arrays
    WS_BUCKET_CNT, WS_BUCKET_START, WS_BUCKET_CURSOR, WS_BUCKET_WIN,
    WS_WIN_PLAN, WS_TILE_PREFIX, WS_WIN_ACC, WS_PAIRS, WS_STATUS,
    WS_MODEL, WS_SAMPLE, WS_SAMPLE_KEYS, WS_HEAVY, WS_AUX0, WS_AUX1, WS_AUX2, WS_AUX3,
    WS_SORT_K0, WS_SORT_K1, WS_SORT_V0, WS_SORT_V1, WS_SORT_HIST, WS_SORT_MAP, WS_SORT_VIEW,
    WS_GEN_TABLE,
    WS_COMPACT, WS_COMPACT_CNT,      // light tuples written by the counting pass
    WS_COARSE_ROWS,                  // per tile: coarse-partition offsets of its light tuples
    WS_EAGER_META, WS_EAGER_K0, WS_EAGER_K1, WS_EAGER_V0, WS_EAGER_V1, WS_EAGER_TILES,   // recorded eager streams
    WS_COUNT
};

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
};

struct EagerState;
struct StreamState;
struct RingState;   // device-resident ingest ring (ring.cu)
struct RingDeleter {
    void operator()(RingState *p) const;
};

}  // namespace sjbg

struct sjbg_handle {
    sjbg_config cfg{};
    int device = 0;
    int num_sms = 0;
    size_t max_smem_optin = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    cudaStream_t copy_stream = nullptr;   // host-input copies overlapped with joins (created on first use)
    std::string err;

    sjbg::DevBuf ws[sjbg::WS_COUNT];
    sjbg::DevBuf pinned[6];   // 0 plan upload, 1 learned, 2 ring gather, 3 results, 4 count pass, 5 eager

    // profiling (SJBG_F_PROFILE)
    struct Pending { int kid; cudaEvent_t a, b; };
    std::vector<Pending> pending;
    std::vector<cudaEvent_t> event_pool;
    std::vector<std::string> knames;
    std::vector<uint64_t> klaunches;
    std::vector<double> kms;
    uint64_t launches = 0;
    bool capturing = false;

    // tunables (the autotuner picks them per workload shape)
    struct Tune {
        uint32_t bucket_target = 4096;   // left tuples per hash-join bucket
        bool persistent_join = true;     // bucket join drains a device work queue
        uint32_t partitioner = 0;        // SJBG_PART_AUTO handles: the tuned choice (0 = by window size)
        float ms = 0.0f;                 // measured time of the chosen setting (autotuner)
    } tune;

    // captured batched calls (SJBG_F_GRAPH)
    struct GraphEntry {
        std::vector<uint64_t> key;
        cudaGraphExec_t exec = nullptr;
        sjbg::DevBuf pinned[6];
        uint32_t part_used = 0;
        uint64_t kernels = 0;   // kernel launches captured: counted again on every replay
    };
    std::vector<std::unique_ptr<GraphEntry>> graphs;
    std::map<std::string, Tune> tuned;   // autotuner decisions by workload shape
    bool tune_loaded = false;

    std::unique_ptr<sjbg::EagerState> eager;
    std::unique_ptr<sjbg::StreamState> streaming;
    std::unique_ptr<sjbg::RingState, sjbg::RingDeleter> ring;

    ~sjbg_handle();
};

namespace sjbg {

int fail(sjbg_handle *h, int code, const std::string &msg);
int cuda_fail(sjbg_handle *h, cudaError_t e, const char *what);

#define SJBG_CK(h, call)                                              \
    do {                                                              \
        cudaError_t _e = (call);                                      \
        if (_e != cudaSuccess) return ::sjbg::cuda_fail((h), _e, #call); \
    } while (0)

// Copy between pinned host staging and device memory with a kernel, in
// stream order on the handle's stream (no copy engine involved).
int stage_copy(sjbg_handle *h, void *dst, const void *src, size_t bytes);
// Zero a ws_get buffer with SM stores (16-byte aligned, whole words): the
// zeros stay in L2 for the kernels that use the buffer next, where a memset
// may write them past L2.
int zero_fill(sjbg_handle *h, void *dst, size_t bytes);
// stage_copy and zero_fill in one launch (a call's plan upload and its table
// clear: one kernel boundary less on the call's critical path).
int stage_copy_zero(sjbg_handle *h, void *dst, const void *src, size_t bytes, void *zdst, size_t zbytes);

// Device buffer of at least `bytes` in slot s (contents not preserved on growth).
void *ws_get(sjbg_handle *h, WsSlot s, size_t bytes);
// Pinned host staging buffer i of at least `bytes`.
void *pinned_get(sjbg_handle *h, int i, size_t bytes);

int kernel_id(sjbg_handle *h, const char *name);
cudaEvent_t event_get(sjbg_handle *h);
// Fold finished profiling events into the per-kernel totals (after a stream sync).
void profile_collect(sjbg_handle *h);

// Launch a kernel on the handle's stream, counting it and (when profiling)
// bracketing it with CUDA events.
template <typename... KArgs, typename... Args>
cudaError_t launch(sjbg_handle *h, const char *name, void (*kernel)(KArgs...), dim3 grid, dim3 block,
                   size_t smem, Args &&...args) {
    const bool prof = (h->cfg.flags & SJBG_F_PROFILE) && !h->capturing;
    cudaEvent_t a = nullptr, b = nullptr;
    if (prof) {
        a = event_get(h);
        cudaEventRecord(a, h->stream);
    }
    kernel<<<grid, block, smem, h->stream>>>(std::forward<Args>(args)...);
    cudaError_t e = cudaGetLastError();
    h->launches++;
    if (prof) {
        b = event_get(h);
        cudaEventRecord(b, h->stream);
        h->pending.push_back({kernel_id(h, name), a, b});
    }
    return e;
}

// Raise a kernel's dynamic shared-memory limit on the current device to at
// least `bytes`.  The limit is process-wide state of the kernel, shared by
// every handle and thread, so it is only ever raised: a call asking for less
// than a concurrent caller's launch needs leaves that launch's limit alone.
cudaError_t raise_smem_limit(const void *kernel, size_t bytes);

template <typename K>
void allow_big_smem(K kernel, size_t bytes) {
    raise_smem_limit(reinterpret_cast<const void *>(kernel), bytes);
}

// ---- host-side window description used by the join modules -------------
struct WinHost {
    uint64_t left_off, n_left, right_off, n_right;
    uint64_t pairs_off, pairs_cap;
};

// Lazy batch drivers (device-resident inputs; pairs may be null).  They
// accumulate into acc[0..n) (device, zeroed by the caller), OR kErr* bits into
// acc[n].info, and leave the stream unsynchronised.
int hj_lazy_batch(sjbg_handle *h, const sjbg_tuple *dL, const sjbg_tuple *dR, const WinHost *wins, uint32_t n,
                  sjbg_pair *dPairs, WinAcc *acc, bool enumerate, uint32_t *part_used);
uint32_t choose_partitioner(const sjbg_handle *h, const WinHost *wins, uint32_t n);
int hj_global_batch(sjbg_handle *h, const sjbg_tuple *dL, const sjbg_tuple *dR, const WinHost *wins, uint32_t n,
                    sjbg_pair *dPairs, WinAcc *acc, bool enumerate);
int nlj_lazy_batch(sjbg_handle *h, const sjbg_tuple *dL, const sjbg_tuple *dR, const WinHost *wins, uint32_t n,
                   sjbg_pair *dPairs, WinAcc *acc, bool enumerate);
int smj_lazy_batch(sjbg_handle *h, const sjbg_tuple *dL, const sjbg_tuple *dR, const WinHost *wins, uint32_t n,
                   sjbg_pair *dPairs, WinAcc *acc, bool enumerate);

int generate_device(sjbg_handle *h, sjbg_tuple *out, uint64_t first, uint64_t n, uint64_t seed, uint64_t domain,
                    const uint64_t *table, uint64_t perm_seed);

// Autotuner (tune.cu): choose h->tune for this batch shape, measuring the
// candidates on the batch itself the first time a shape is seen.
int autotune_lazy(sjbg_handle *h, const sjbg_tuple *dL, const sjbg_tuple *dR, const WinHost *wins, uint32_t n,
                  bool enumerate);
// One device-side lazy batch (no host synchronisation), used by the runtime and
// the tuner.  hAcc (pinned) receives n + 1 entries: the windows' accumulators,
// then the call's device status word in hAcc[n].info (kErr* bits).
int run_lazy_device(sjbg_handle *h, const sjbg_tuple *dL, const sjbg_tuple *dR, const WinHost *wins, uint32_t n,
                    sjbg_pair *dPairs, WinAcc *hAcc, uint32_t *part_used);
// SJBG_OK, or the error a device status word reports (recorded on the handle).
int device_status_error(sjbg_handle *h, unsigned long long bits);

}  // namespace sjbg
