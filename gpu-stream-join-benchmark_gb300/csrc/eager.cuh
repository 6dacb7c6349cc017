// eager.cuh - eager (per-batch) executors: state layout.
#pragma once
#include "runtime.h"

namespace sjbg {

constexpr uint32_t kEagerMaxSortBatch = 8192;   // eager sort-merge batches are sorted by one CTA

// One side's state of the current eager window (device memory).
struct EagerSide {
    sjbg_tuple *tuples = nullptr;   // arrival order, cap tuples
    uint64_t n = 0;                 // tuples so far in this window
    // hash join: open-addressing table keyed by key, with per-key chains
    uint32_t *tkeys = nullptr;      // slots + 1 (last slot: key 0xFFFFFFFF)
    uint32_t *tcnt = nullptr;
    unsigned long long *tsum = nullptr;   // sum of this side's pair hash (left: fr, right: gs)
    uint32_t *thead = nullptr;
    uint32_t *next = nullptr;       // chain link per tuple (index into tuples)
    // sort-merge join: the side's tuples sorted by key, plus prefix sums of its pair hash
    uint32_t *skeys = nullptr, *svals = nullptr;
    uint32_t *skeys2 = nullptr, *svals2 = nullptr;
    unsigned long long *F = nullptr;   // n + 1 entries
};

struct PkState;   // persistent eager kernel (eager_pk.cu)
struct PkDeleter {
    void operator()(PkState *p) const;
};

struct EagerState {
    EagerSide side[2];
    uint64_t cap = 0;          // tuples per side
    uint32_t table_bits = 0;
    WinAcc *acc = nullptr;     // current window totals (device)
    unsigned long long *batch_count = nullptr;   // device slot for the last batch's matches
    sjbg_pair *pairs = nullptr;   // current window's pairs (device), pairs_cap entries
    uint64_t pairs_cap = 0;
    uint32_t *sort_tmp = nullptr;  // sorted incoming batch: keys then vals (2 * kEagerMaxSortBatch)
    std::vector<void *> allocs;
    std::unique_ptr<PkState, PkDeleter> pk;   // SJBG_F_PERSISTENT: created by the first ticket
    ~EagerState();
};

// One CTA of a recorded eager stream's nested-loop join (nlj.cu): left batch
// lb against right batch rb of window `win`, left tuples [l0, l0 + tile).
struct ERunItem {
    uint32_t win;    // window accumulator
    uint32_t lb;     // left batch
    uint32_t rb;     // right batch
    uint32_t dest;   // counter of the later batch: 2 * batch + side
    uint32_t l0;     // first left tuple of this CTA inside the batch
    uint32_t pad[3];
};
int eager_nlj_blocks(sjbg_handle *h, const sjbg_tuple *dl, const sjbg_tuple *dr, uint64_t B, const ERunItem *items,
                     uint32_t n_items, WinAcc *acc, unsigned long long *counts, bool enumerate);
uint32_t nlj_left_tile();   // left tuples per nested-loop CTA

// A whole recorded eager stream (eager_run.cu): batch counts into dCounts
// (2 * n_batches), window totals into dWin (then the status word).
int eager_run_batched(sjbg_handle *h, const sjbg_tuple *dl, const sjbg_tuple *dr, uint64_t n_batches, bool enumerate,
                      unsigned long long *dCounts, WinAcc *dWin, uint32_t *n_windows);

int eager_init(sjbg_handle *h);
int eager_init_and_clear(sjbg_handle *h);

// Persistent eager kernel (eager_pk.cu), used by the eager entry points of
// SJBG_F_PERSISTENT handles.
int pk_execute(sjbg_handle *h, const sjbg_tuple *batch, uint64_t n, int side, bool from_host, uint64_t *match);
int pk_post_batch(sjbg_handle *h, const sjbg_tuple *batch, uint64_t n, int side, bool from_host, uint64_t *ticket);
int pk_wait_batch(sjbg_handle *h, uint64_t ticket, uint64_t *match);
int pk_clear_states(sjbg_handle *h);
int pk_report(sjbg_handle *h, WinAcc *totals);
int pk_stop(sjbg_handle *h, bool reset);
int pk_status(sjbg_handle *h, int *running, uint64_t *launches);
// Stop a handle's persistent kernel before the handle goes.
int eager_shutdown(sjbg_handle *h);

}  // namespace sjbg
