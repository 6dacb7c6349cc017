// eager_pk.cu - persistent eager joins (sm_103a).
//
// The reference's persistent executor GPU_HJ_PK
// (src/sjb/windowing/eager/executor/GPU/GPU_HJ_PK.cu:10-89,101-180; switched
// on by EagerJoinConfig::usePK, include/experiment/Config.hpp:15) keeps build
// and probe kernels resident with one thread per tuple; every thread spins,
// without a bound, on its own signal byte in mapped host memory, which the
// host sets per thread and then spins on until the thread clears it.
//
// Here, with SJBG_F_PERSISTENT, one cooperative kernel per eager handle stays
// resident and takes TICKETS from a queue in mapped host memory:
//
//   host                                          device (G CTAs)
//   copy the batch into the ticket's payload      CTA 0 waits for ticket t's
//   slot, fill the descriptor, release-store      descriptor (acquire, system
//   seq = t + 1                                   scope), adds the window state
//                                                 the ticket needs and
//                                                 broadcasts it (L2) to the
//                                                 other CTAs; every CTA does its
//                                                 share and arrives; CTA 0, once
//   acquire-load result seq == t + 1, read   <--  all have, writes the result
//   the batch's new matches                       and release-stores its seq
//
// so a batch costs no kernel launch, no copy-engine transfer and no stream
// synchronisation.  Tickets run strictly in order, one at a time (a batch
// must see every earlier batch of the other side, and only those); inside a
// ticket the CTAs split the batch.  Per algorithm:
//   HJ   per tuple: copy it into its side's store, probe the other side's
//        table, insert into its own (eager_hj_step, shared with the per-batch
//        kernel);
//   NLJ  copy the batch into its side's store; grid barrier; the batch against
//        the other side's store in (left tile, right split) blocks (nlj_block,
//        coherent loads);
//   SMJ  the batch into device memory; grid barrier; one warp per batch
//        element: its stable rank in the batch by counting
//        over the batch's keys in shared memory, with the exclusive prefix of
//        the side's pair hash in the same pass, and the probe of the other
//        side's sorted run by a 32-way warp search; grid barrier; the side's
//        run and the sorted batch are merged into the other buffer of a
//        ping-pong pair, each element's prefix sum formed from the two inputs'
//        prefix sums, so no separate scan runs.
// Other tickets: clear (close the window: snapshot the totals, reset the
// state), report (snapshot the totals), stop (exit).
//
// Every wait is bounded by %globaltimer:
//   * CTA 0 waits at most idle_timeout_ms for the next ticket.  When the wait
//     runs out it stores kErrTimeout and the ticket it was waiting for in the
//     control block, and every CTA returns.  The window state stays in device
//     memory: the next post relaunches the kernel from that ticket, and
//     sjbg_eager_pk_status reports the expiry once as SJBG_E_TIMEOUT.
//   * waits for the other CTAs inside a ticket (the broadcast, the arrivals,
//     the grid barrier) give up after kSyncNs: the kernel stores kErrTimeout,
//     the ticket's result carries it, every CTA returns, and the handle
//     refuses further batches until its window is cleared.
//   * the host waits for a ticket's result at most idle_timeout_ms + 2 s.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <thread>

#include "eager_dev.cuh"
#include "nlj.cuh"

namespace sjbg {

namespace {

enum : uint32_t { kPkSkip = 0, kPkBatch = 1, kPkClear = 2, kPkReport = 3, kPkStop = 4 };
enum : unsigned long long { kPkNotRunning = 0, kPkRunning = 1, kPkStopped = 2, kPkIdleExit = 3, kPkFailed = 4 };
constexpr unsigned long long kQuitSeq = ~0ull;         // broadcast value: every CTA returns
constexpr unsigned long long kSyncNs = 2000000000ull;  // longest wait for the other CTAs inside a ticket
constexpr int kPkThreads = kNljThreads;                // nlj_block's CTA size
constexpr uint32_t kPkQueueMax = 64;

// One queue entry, written by the host (mapped host memory).
struct __align__(64) PkDesc {
    unsigned long long seq;   // ticket + 1 once the entry is complete (stored last, with release)
    unsigned long long src;   // device-visible address of the batch's tuples
    uint32_t cmd, side, n, pad;
    unsigned long long pad2[4];
};
// One result per queue entry, written by the device (mapped host memory).
struct __align__(64) PkResult {
    unsigned long long seq;   // ticket + 1 once the result is complete (stored last, with release)
    unsigned long long count;   // the batch's new matches
    unsigned long long win_count, win_xor, win_prod, win_pairs;   // window totals before a clear / report
    unsigned long long status;   // kErr* bits raised while the ticket ran
    unsigned long long pad;
};
// Why and where the kernel last returned (mapped host memory, written by the device).
struct __align__(64) PkCtl {
    unsigned long long state;    // kPk*
    unsigned long long ticket;   // the ticket the kernel would have taken next
    unsigned long long err;      // kErr* bits of that exit
    unsigned long long pad[5];
};
static_assert(sizeof(PkDesc) == 64 && sizeof(PkResult) == 64 && sizeof(PkCtl) == 64, "one 64-byte line each");

// The ticket in flight, as CTA 0 broadcasts it.
struct PkWork {
    unsigned long long src;
    uint32_t cmd, side, n, base, oth_n, par_own, par_oth, pad;
};
// Synchronisation words, reset before every launch.
struct __align__(64) PkSync {
    unsigned long long bseq;     // ticket + 1 whose work is in `work`; kQuitSeq = return
    unsigned long long tcount;   // matches of the ticket in flight
    uint32_t arrive;             // CTAs done with the ticket in flight
    uint32_t err;                // kErr* bits of the ticket in flight
    uint32_t bar_count, bar_gen;   // grid barrier inside a ticket
    PkWork work;
};
// Window state that lives across launches (device memory).
struct __align__(64) PkDev {
    unsigned long long side_n[2];   // tuples of each side in the current window
    uint32_t parity[2];             // sort-merge: which buffer of the side's pair holds its run
    PkSync sync;
};

struct PkArgs {
    const PkDesc *desc;
    PkResult *res;
    PkCtl *ctl;
    PkDev *dev;
    unsigned long long first_ticket;
    unsigned long long idle_ns;
    unsigned long long cap;   // tuples per side
    uint32_t Q;
    uint32_t batch_cap;
    sjbg_tuple *tuples[2];
    ETab tab[2];
    uint32_t *skeys[2][2];
    uint32_t *svals[2][2];
    unsigned long long *F[2][2];
    uint32_t *bkeys, *bvals;
    unsigned long long *bF;
    uint2 *stage;   // sort-merge: the batch's (key, val) in arrival order, in device memory
    WinAcc *acc;
    sjbg_pair *pairs;
    unsigned long long pairs_cap;
};

// ---------------------------------------------------------------- memory-order primitives
__device__ __forceinline__ unsigned long long ld_acq_sys(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long ld_acq_gpu(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint32_t ld_acq_gpu(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_rel_sys(unsigned long long *p, unsigned long long v) {
    asm volatile("st.release.sys.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void st_rel_gpu(unsigned long long *p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
// Loads of data the host (or an earlier ticket's payload in the same slot)
// wrote: fetched again, never from a cached line.
__device__ __forceinline__ uint4 ld_cv4(const void *p) {
    uint4 v;
    asm volatile("ld.global.cv.v4.u32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p));
    return v;
}
__device__ __forceinline__ unsigned long long ld_cv64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.global.cv.u64 %0, [%1];" : "=l"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ uint32_t ld_cv32(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.global.cv.u32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}

// ---------------------------------------------------------------- ticket protocol
// CTA 0, thread 0: wait for ticket t from the host and broadcast it.  Returns 1
// when the kernel must return (the wait for the host ran out).
__device__ int pk_take(const PkArgs &a, unsigned long long t, PkWork *w) {
    PkDev *d = a.dev;
    const PkDesc *e = a.desc + (t % a.Q);
    const unsigned long long t0 = global_ns();
    uint32_t spins = 0;
    while (ld_acq_sys(&e->seq) != t + 1) {
        if (global_ns() - t0 > a.idle_ns) {
            a.ctl->ticket = t;
            a.ctl->err = kErrTimeout;
            st_rel_sys(&a.ctl->state, kPkIdleExit);
            st_rel_gpu(&d->sync.bseq, kQuitSeq);
            return 1;
        }
        __nanosleep(spins < 1024 ? 32 : 1024);
        spins++;
    }
    PkWork x;
    x.cmd = ld_cv32(&e->cmd);
    x.side = ld_cv32(&e->side) & 1u;
    x.n = ld_cv32(&e->n);
    x.src = ld_cv64(&e->src);
    x.base = (uint32_t)d->side_n[x.side];
    x.oth_n = (uint32_t)d->side_n[x.side ^ 1u];
    x.par_own = d->parity[x.side];
    x.par_oth = d->parity[x.side ^ 1u];
    x.pad = 0;
    // the host checked these; nothing reaches past the buffers if it did not
    if (x.cmd < kPkBatch || x.cmd > kPkStop ||
        (x.cmd == kPkBatch && (x.n > a.batch_cap || (unsigned long long)x.base + x.n > a.cap || (x.src & 15ull)))) {
        x.cmd = kPkSkip;
        atomicOr(&d->sync.err, kErrBadWindow);
    }
    if (x.cmd == kPkClear || x.cmd == kPkReport) {   // every earlier ticket is complete here
        PkResult *r = a.res + (t % a.Q);
        const volatile WinAcc *acc = a.acc;
        r->win_count = acc->count;
        r->win_xor = acc->xr;
        r->win_prod = acc->prod;
        r->win_pairs = acc->npairs;
    }
    d->sync.work = x;
    st_rel_gpu(&d->sync.bseq, t + 1);
    *w = x;
    return 0;
}

// Other CTAs, thread 0: wait for CTA 0's broadcast of ticket t.
__device__ int pk_follow(const PkArgs &a, unsigned long long t, PkWork *w) {
    PkSync *s = &a.dev->sync;
    const unsigned long long t0 = global_ns();
    for (;;) {
        const unsigned long long q = ld_acq_gpu(&s->bseq);
        if (q == t + 1) break;
        if (q == kQuitSeq) return 1;
        if (global_ns() - t0 > a.idle_ns + kSyncNs) {
            atomicOr(&s->err, kErrTimeout);
            return 1;
        }
        __nanosleep(32);
    }
    __threadfence();
    const volatile PkWork *v = &s->work;
    w->src = v->src;
    w->cmd = v->cmd;
    w->side = v->side;
    w->n = v->n;
    w->base = v->base;
    w->oth_n = v->oth_n;
    w->par_own = v->par_own;
    w->par_oth = v->par_oth;
    w->pad = 0;
    return 0;
}

// Grid barrier inside a ticket (all CTAs; bounded).  False when it gave up.
__device__ bool pk_grid_sync(PkDev *d) {
    __shared__ int ok;
    SJBG_BARRIER();
    if (threadIdx.x == 0) {
        ok = 1;
        PkSync *s = &d->sync;
        const uint32_t gen = ld_acq_gpu(&s->bar_gen);
        __threadfence();
        if (atomicAdd(&s->bar_count, 1u) == gridDim.x - 1) {
            s->bar_count = 0;
            __threadfence();
            atomicAdd(&s->bar_gen, 1u);
        } else {
            const unsigned long long t0 = global_ns();
            while (ld_acq_gpu(&s->bar_gen) == gen) {
                if (global_ns() - t0 > kSyncNs) {
                    atomicOr(&s->err, kErrTimeout);
                    ok = 0;
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
    }
    SJBG_BARRIER();
    return ok != 0;
}

// Every CTA after its share of ticket t.  CTA 0 waits for all, publishes the
// result and advances the window state.  Returns 1 when the kernel must return.
template <int kAlg>
__device__ int pk_arrive(const PkArgs &a, unsigned long long t, const PkWork &w) {
    __shared__ int quit;
    SJBG_BARRIER();
    if (threadIdx.x == 0) {
        quit = w.cmd == kPkStop;
        PkDev *d = a.dev;
        PkSync *s = &d->sync;
        __threadfence();
        atomicAdd(&s->arrive, 1u);
        if (blockIdx.x == 0) {
            const unsigned long long t0 = global_ns();
            bool ok = true;
            while (ld_acq_gpu(&s->arrive) < gridDim.x) {
                if (global_ns() - t0 > kSyncNs) {
                    ok = false;
                    break;
                }
                __nanosleep(32);
            }
            __threadfence();
            uint32_t err = atomicExch(&s->err, 0u);
            if (!ok) err |= kErrTimeout;
            PkResult *r = a.res + (t % a.Q);
            r->count = atomicExch(&s->tcount, 0ull);
            r->status = err;
            if (!(err & kErrTimeout)) {
                if (w.cmd == kPkBatch) {
                    d->side_n[w.side] += w.n;
                    if (kAlg == SJBG_ALG_SMJ) d->parity[w.side] ^= 1u;
                } else if (w.cmd == kPkClear) {
                    d->side_n[0] = d->side_n[1] = 0;
                    d->parity[0] = d->parity[1] = 0;
                }
            }
            s->arrive = 0;
            if (err & kErrTimeout) {   // the window state is in doubt: return and let the host refuse batches
                a.ctl->ticket = t + 1;
                a.ctl->err = err;
                st_rel_sys(&a.ctl->state, kPkFailed);
                st_rel_gpu(&s->bseq, kQuitSeq);
                quit = 1;
            } else if (w.cmd == kPkStop) {
                a.ctl->ticket = t + 1;
                a.ctl->err = 0;
                st_rel_sys(&a.ctl->state, kPkStopped);
            }
            __threadfence_system();
            st_rel_sys(&r->seq, t + 1);
        }
    }
    SJBG_BARRIER();
    return quit;
}

// ---------------------------------------------------------------- ticket work
template <bool kEnum, bool kPairs>
__device__ void pk_hj_batch(const PkArgs &a, const PkWork &w) {
    const int side = (int)w.side;
    const sjbg_tuple *src = reinterpret_cast<const sjbg_tuple *>(w.src);
    sjbg_tuple *store = a.tuples[side] + w.base;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < w.n; i0 += stride) {   // CTA-uniform: whole warps step
        const uint32_t i = i0 + threadIdx.x;
        const bool valid = i < w.n;
        uint32_t key = 0, val = 0;
        if (valid) {
            const uint4 t = ld_cv4(src + i);
            *reinterpret_cast<uint4 *>(store + i) = t;
            key = t.x;
            val = t.y;
        }
        eager_hj_step<kEnum, kPairs>(valid, key, val, w.base + i, side, a.tab[side], a.tab[side ^ 1],
                                     a.tuples[side ^ 1], w.oth_n, a.acc, &a.dev->sync.tcount, a.pairs,
                                     a.pairs_cap);
    }
}

template <bool kEnum, bool kPairs>
__device__ void pk_nlj_batch(const PkArgs &a, const PkWork &w) {
    const int side = (int)w.side;
    const sjbg_tuple *src = reinterpret_cast<const sjbg_tuple *>(w.src);
    sjbg_tuple *store = a.tuples[side] + w.base;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < w.n; i += gridDim.x * blockDim.x)
        *reinterpret_cast<uint4 *>(store + i) = ld_cv4(src + i);
    if (!pk_grid_sync(a.dev)) return;
    const sjbg_tuple *Lw = side == 0 ? store : a.tuples[0];
    const sjbg_tuple *Rw = side == 0 ? a.tuples[1] : store;
    const uint32_t nL = side == 0 ? w.n : w.oth_n;
    const uint32_t nR = side == 0 ? w.oth_n : w.n;
    if (nL == 0 || nR == 0) return;
    // right splits fine enough that the blocks cover the grid
    const uint32_t lt = (nL + kLTile - 1) / kLTile;
    uint32_t rsplit = kRSplit;
    while (rsplit > 256 && lt * ((nR + rsplit - 1) / rsplit) < gridDim.x) rsplit >>= 1;
    const uint32_t items = lt * ((nR + rsplit - 1) / rsplit);
    for (uint32_t it = blockIdx.x; it < items; it += gridDim.x)
        nlj_block<kEnum, kPairs, true>(Lw, nL, Rw, nR, (it % lt) * kLTile, (it / lt) * rsplit, a.acc,
                                       &a.dev->sync.tcount, a.pairs, a.pairs_cap, rsplit);
}

// First position p in sorted a[0, n) with a[p] >= key (kUpper: a[p] > key),
// by the whole warp: 32 probes per round, so about log32(n) dependent loads.
template <bool kUpper>
__device__ __forceinline__ uint32_t warp_search(const uint32_t *a, uint32_t n, uint32_t key) {
    uint32_t lo = 0, hi = n;   // the answer lies in [lo, hi]
    const uint32_t lane = lane_id();
    while (hi - lo > 32) {
        const uint32_t step = (hi - lo + 31) / 32;
        const uint32_t p = lo + lane * step;
        const bool before = p < hi && (kUpper ? a[p] <= key : a[p] < key);
        const uint32_t c = __popc(__ballot_sync(0xFFFFFFFFu, before));
        const uint32_t nlo = c ? lo + (c - 1) * step + 1 : lo;
        hi = min(hi, lo + c * step);
        lo = nlo;
    }
    const uint32_t p = lo + lane;
    const bool before = p < hi && (kUpper ? a[p] <= key : a[p] < key);
    return lo + __popc(__ballot_sync(0xFFFFFFFFu, before));
}

// Upper bound of key in sorted a[lo, n) when a[lo] starts key's run (lo is its
// lower bound): one round of 32 probes when the run is shorter than 32 (the
// common case), the full search past them otherwise.
__device__ __forceinline__ uint32_t warp_upper_from(const uint32_t *a, uint32_t n, uint32_t lo, uint32_t key) {
    const uint32_t p = lo + lane_id();
    const unsigned le = __ballot_sync(0xFFFFFFFFu, p < n && a[p] <= key);
    if (le != 0xFFFFFFFFu) return lo + __popc(le);
    return lo + 32 + warp_search<true>(a + lo + 32, n - lo - 32, key);
}

// Phase 0: the batch's (key, val) into device memory, once (every CTA reads
// all of it next; from the host link that would be once per CTA).
// Phase 1: rank each batch element in (key, arrival) order with the exclusive
// prefix of the side's pair hash, and probe the other side's run.
// Phase 2: merge the side's run with the sorted batch into the other buffer.
template <bool kEnum, bool kPairs>
__device__ void pk_smj_batch(const PkArgs &a, const PkWork &w, uint8_t *smem) {
    const int side = (int)w.side;
    const uint32_t n = w.n;
    const sjbg_tuple *src = reinterpret_cast<const sjbg_tuple *>(w.src);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint4 t = ld_cv4(src + i);
        a.stage[i] = make_uint2(t.x, t.y);
    }
    if (!pk_grid_sync(a.dev)) return;
    uint32_t *sk = reinterpret_cast<uint32_t *>(smem);                                      // n keys
    unsigned long long *sh = reinterpret_cast<unsigned long long *>(smem + 4 * ((n + 1) & ~1u));   // n hashes
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const uint2 t = a.stage[i];
        sk[i] = t.x;
        sh[i] = own_hash(side, t.y);
    }
    SJBG_BARRIER();
    const uint32_t lane = lane_id();
    const uint32_t warps = gridDim.x * (blockDim.x / 32);
    const uint32_t gw = blockIdx.x * (blockDim.x / 32) + warp_id();
    const uint32_t *okeys = a.skeys[side ^ 1][w.par_oth];
    const uint32_t *ovals = a.svals[side ^ 1][w.par_oth];
    const unsigned long long *oF = a.F[side ^ 1][w.par_oth];
    unsigned long long count = 0, xr = 0, prod = 0;
    for (uint32_t j = gw; j < n; j += warps) {   // warp-uniform
        const uint32_t kj = sk[j];
        uint32_t below = 0;
        unsigned long long hsum = 0;
        for (uint32_t i = lane; i < n; i += 32) {
            const uint32_t ki = sk[i];
            if (ki < kj || (ki == kj && i < j)) {
                below++;
                hsum += sh[i];
            }
        }
        below = (uint32_t)warp_sum_u64(below);
        hsum = warp_sum_u64(hsum);
        const uint32_t vj = a.stage[j].y;
        if (lane == 0) {
            a.bkeys[below] = kj;
            a.bvals[below] = vj;
            a.bF[below] = hsum;
        }
        // the probe
        const uint32_t lo = warp_search<false>(okeys, w.oth_n, kj);
        const uint32_t hi = (lo < w.oth_n && okeys[lo] == kj) ? warp_upper_from(okeys, w.oth_n, lo, kj) : lo;
        if (lane == 0) {
            count += hi - lo;
            prod += sh[j] * (oF[hi] - oF[lo]);
        }
        if (kEnum)
            for (uint32_t q = lo + lane; q < hi; q += 32)
                xr ^= side == 0 ? sjbg_pair_hash(vj, ovals[q]) : sjbg_pair_hash(ovals[q], vj);
        if (kPairs && hi > lo) {
            unsigned long long b = 0;
            if (lane == 0) b = atomicAdd(&a.acc->npairs, (unsigned long long)(hi - lo));
            b = __shfl_sync(0xFFFFFFFFu, b, 0);
            for (uint32_t q = lo + lane; q < hi; q += 32)
                if (b + (q - lo) < a.pairs_cap)
                    a.pairs[b + (q - lo)] = side == 0 ? sjbg_pair{vj, ovals[q]} : sjbg_pair{ovals[q], vj};
        }
    }
    if (blockIdx.x == 0) {   // the batch's total hash, for the merged run's last prefix
        __shared__ unsigned long long wtot[kPkThreads / 32];
        unsigned long long part = 0;
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) part += sh[i];
        part = warp_sum_u64(part);
        if (lane == 0) wtot[warp_id()] = part;
        SJBG_BARRIER();
        if (threadIdx.x == 0) {
            unsigned long long tot = 0;
            for (int q = 0; q < kPkThreads / 32; q++) tot += wtot[q];
            a.bF[n] = tot;
        }
    }
    flush_acc(a.acc, count, xr, prod);
    {
        const unsigned long long c = warp_sum_u64(count);
        if (lane == 0 && c) atomicAdd(&a.dev->sync.tcount, c);
    }
    if (!pk_grid_sync(a.dev)) return;
    // phase 2: the sorted batch's keys and prefix sums into shared memory
    uint32_t *bk = sk;
    unsigned long long *bF = sh;
    for (uint32_t i = threadIdx.x; i <= n; i += blockDim.x) {
        if (i < n) bk[i] = a.bkeys[i];
        bF[i] = a.bF[i];
    }
    SJBG_BARRIER();
    const uint32_t na = w.base;
    const uint32_t *rk = a.skeys[side][w.par_own];
    const uint32_t *rv = a.svals[side][w.par_own];
    const unsigned long long *rF = a.F[side][w.par_own];
    uint32_t *ok = a.skeys[side][w.par_own ^ 1];
    uint32_t *ov = a.svals[side][w.par_own ^ 1];
    unsigned long long *oFn = a.F[side][w.par_own ^ 1];
    // run elements: output rank = own index + batch elements with a smaller key
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < na; i += gridDim.x * blockDim.x) {
        const uint32_t k = rk[i];
        uint32_t lo = 0, hi = n;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (bk[mid] < k) lo = mid + 1; else hi = mid;
        }
        const uint32_t p = i + lo;
        ok[p] = k;
        ov[p] = rv[i];
        oFn[p] = rF[i] + bF[lo];
    }
    // batch elements: output rank = own rank + run elements with a key not larger
    for (uint32_t j = gw; j < n; j += warps) {
        const uint32_t k = bk[j];
        const uint32_t ub = warp_search<true>(rk, na, k);
        if (lane == 0) {
            const uint32_t p = j + ub;
            ok[p] = k;
            ov[p] = a.bvals[j];
            oFn[p] = bF[j] + rF[ub];
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) oFn[na + n] = rF[na] + bF[n];
}

// Close the window: reset the tables / runs and the totals.
template <int kAlg>
__device__ void pk_clear(const PkArgs &a) {
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x, nt = gridDim.x * blockDim.x;
    if (kAlg == SJBG_ALG_HJ) {
        for (int s = 0; s < 2; s++) {
            const ETab &t = a.tab[s];
            const uint32_t C = 1u << t.bits;   // C + 1 entries; C is a multiple of 4
            for (uint32_t i = tid; i < C / 4; i += nt) {
                reinterpret_cast<uint4 *>(t.keys)[i] = make_uint4(kEmptyKey, kEmptyKey, kEmptyKey, kEmptyKey);
                reinterpret_cast<uint4 *>(t.head)[i] = make_uint4(kNilIdx, kNilIdx, kNilIdx, kNilIdx);
                reinterpret_cast<uint4 *>(t.cnt)[i] = make_uint4(0, 0, 0, 0);
                reinterpret_cast<uint4 *>(t.sum)[2 * i] = make_uint4(0, 0, 0, 0);
                reinterpret_cast<uint4 *>(t.sum)[2 * i + 1] = make_uint4(0, 0, 0, 0);
            }
            if (tid == 0) {
                t.keys[C] = kEmptyKey;
                t.head[C] = kNilIdx;
                t.cnt[C] = 0;
                t.sum[C] = 0;
            }
        }
    }
    if (tid == 0) {
        if (kAlg == SJBG_ALG_SMJ)
            for (int s = 0; s < 2; s++) a.F[s][0][0] = a.F[s][1][0] = 0;
        *a.acc = WinAcc{0, 0, 0, 0, 0};
    }
}

template <int kAlg, bool kEnum, bool kPairs>
__global__ void __launch_bounds__(kPkThreads) eager_pk_kernel(PkArgs a) {
    extern __shared__ __align__(16) uint8_t pk_smem[];
    __shared__ PkWork w;
    __shared__ int quit;
    unsigned long long t = a.first_ticket;
    for (;;) {
        if (threadIdx.x == 0) quit = blockIdx.x == 0 ? pk_take(a, t, &w) : pk_follow(a, t, &w);
        SJBG_BARRIER();
        if (quit) return;
        if (w.cmd == kPkBatch) {
            if (kAlg == SJBG_ALG_HJ) pk_hj_batch<kEnum, kPairs>(a, w);
            else if (kAlg == SJBG_ALG_NLJ) pk_nlj_batch<kEnum, kPairs>(a, w);
            else pk_smj_batch<kEnum, kPairs>(a, w, pk_smem);
        } else if (w.cmd == kPkClear) {
            pk_clear<kAlg>(a);
        }
        if (pk_arrive<kAlg>(a, t, w)) return;
        t++;
    }
}

using PkKernel = void (*)(PkArgs);

template <int kAlg>
PkKernel pk_kernel_for(bool en, bool pairs) {
    if (pairs) return eager_pk_kernel<kAlg, true, true>;
    if (en) return eager_pk_kernel<kAlg, true, false>;
    return eager_pk_kernel<kAlg, false, false>;
}

inline unsigned long long host_acquire(const unsigned long long *p) { return __atomic_load_n(p, __ATOMIC_ACQUIRE); }
inline void host_release(unsigned long long *p, unsigned long long v) { __atomic_store_n(p, v, __ATOMIC_RELEASE); }

}  // namespace

// ---------------------------------------------------------------- host runtime
struct PkState {
    cudaStream_t stream = nullptr;   // non-blocking; the kernel lives on it
    uint8_t *hmem = nullptr;         // mapped host block: control, queue, results, payload slots
    uint8_t *dmem = nullptr;         // its device view
    PkCtl *hctl = nullptr, *dctl = nullptr;
    PkDesc *hdesc = nullptr, *ddesc = nullptr;
    PkResult *hres = nullptr, *dres = nullptr;
    sjbg_tuple *hpay = nullptr, *dpay = nullptr;
    PkDev *dev = nullptr;
    uint32_t *bkeys = nullptr, *bvals = nullptr;
    unsigned long long *bF = nullptr;
    uint2 *stage = nullptr;
    unsigned long long *F2[2] = {nullptr, nullptr};
    std::vector<void *> dallocs;
    uint32_t Q = 0;
    uint64_t slot = 0;   // tuples per payload slot
    uint64_t next = 0;   // next ticket to post
    uint64_t done = 0;   // tickets whose results were read (every ticket < done)
    std::vector<unsigned long long> count, status;   // results of the last Q tickets, by ticket % Q
    std::vector<WinAcc> snap;                         // window totals of clear / report tickets
    uint64_t side_posted[2] = {0, 0};
    PkKernel kernel = nullptr;
    int grid = 0;
    size_t smem = 0;
    bool running = false;
    bool host_direct = false;   // the GPU reads pageable host memory coherently (address translation services)
    bool broken = false;        // a ticket failed on the device: batches refused until the window is cleared
    bool reset_state = true;    // clear the device window state before the next launch
    uint64_t launches = 0;
    uint64_t idle_exits = 0, idle_reported = 0;
    ~PkState();
};

static int pk_sync_stream(PkState &pk) {
    return cudaStreamSynchronize(pk.stream) == cudaSuccess ? SJBG_OK : SJBG_E_CUDA;
}

PkState::~PkState() {
    if (stream) {
        // a kernel still running (the handle could not stop it) returns by
        // itself within idle_timeout_ms
        if (running) cudaStreamSynchronize(stream);
        cudaStreamDestroy(stream);
    }
    for (void *p : dallocs) cudaFree(p);
    if (hmem) cudaFreeHost(hmem);
}

static uint64_t pk_idle_ms(const sjbg_handle *h) { return h->cfg.idle_timeout_ms ? h->cfg.idle_timeout_ms : 1000; }

static int pk_init(sjbg_handle *h) {
    EagerState &st = *h->eager;
    auto pk = std::make_unique<PkState>();
    const uint64_t B = h->cfg.batch_size;
    if (B > 0x7FFFFFFFull) return fail(h, SJBG_E_UNSUPPORTED, "persistent eager batches are limited to 2^31 tuples");
    pk->slot = B;
    pk->Q = (uint32_t)std::max<uint64_t>(4, std::min<uint64_t>(kPkQueueMax, (64ull << 20) / (16 * B + 1)));
    const size_t head = sizeof(PkCtl) + (sizeof(PkDesc) + sizeof(PkResult)) * pk->Q;
    const size_t bytes = head + sizeof(sjbg_tuple) * B * pk->Q;
    if (cudaStreamCreateWithFlags(&pk->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaHostAlloc(&pk->hmem, bytes, cudaHostAllocMapped | cudaHostAllocPortable) != cudaSuccess ||
        cudaHostGetDevicePointer(reinterpret_cast<void **>(&pk->dmem), pk->hmem, 0) != cudaSuccess) {
        cudaGetLastError();
        return fail(h, SJBG_E_NOMEM, "persistent eager queue (mapped host memory)");
    }
    std::memset(pk->hmem, 0, head);
    pk->hctl = reinterpret_cast<PkCtl *>(pk->hmem);
    pk->hdesc = reinterpret_cast<PkDesc *>(pk->hmem + sizeof(PkCtl));
    pk->hres = reinterpret_cast<PkResult *>(pk->hmem + sizeof(PkCtl) + sizeof(PkDesc) * pk->Q);
    pk->hpay = reinterpret_cast<sjbg_tuple *>(pk->hmem + head);
    pk->dctl = reinterpret_cast<PkCtl *>(pk->dmem);
    pk->ddesc = reinterpret_cast<PkDesc *>(pk->dmem + sizeof(PkCtl));
    pk->dres = reinterpret_cast<PkResult *>(pk->dmem + sizeof(PkCtl) + sizeof(PkDesc) * pk->Q);
    pk->dpay = reinterpret_cast<sjbg_tuple *>(pk->dmem + head);
    auto dalloc = [&](size_t b) -> void * {
        void *p = nullptr;
        if (cudaMalloc(&p, b ? b : 16) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        pk->dallocs.push_back(p);
        return p;
    };
    pk->dev = static_cast<PkDev *>(dalloc(sizeof(PkDev)));
    if (!pk->dev) return fail(h, SJBG_E_NOMEM, "persistent eager state");
    const bool en = h->cfg.result_mode != SJBG_RESULT_NO_OUTPUT || (h->cfg.flags & SJBG_F_XOR);
    const bool pairs = st.pairs != nullptr;
    switch (h->cfg.algorithm) {
        case SJBG_ALG_HJ: pk->kernel = pk_kernel_for<SJBG_ALG_HJ>(en, pairs); break;
        case SJBG_ALG_NLJ: pk->kernel = pk_kernel_for<SJBG_ALG_NLJ>(en, pairs); break;
        default: {
            pk->kernel = pk_kernel_for<SJBG_ALG_SMJ>(en, pairs);
            pk->bkeys = static_cast<uint32_t *>(dalloc(4 * B));
            pk->bvals = static_cast<uint32_t *>(dalloc(4 * B));
            pk->bF = static_cast<unsigned long long *>(dalloc(8 * (B + 1)));
            pk->stage = static_cast<uint2 *>(dalloc(8 * B));
            for (int s = 0; s < 2; s++)
                pk->F2[s] = static_cast<unsigned long long *>(dalloc(8 * (st.cap + 1)));
            if (!pk->bkeys || !pk->bvals || !pk->bF || !pk->stage || !pk->F2[0] || !pk->F2[1])
                return fail(h, SJBG_E_NOMEM, "persistent sort-merge buffers");
            pk->smem = 4 * ((B + 1) & ~1ull) + 8 * (B + 1);   // keys, then hashes (phase 2: sorted keys and prefixes)
            break;
        }
    }
    if (pk->smem > 48 * 1024) {
        if (cudaFuncSetAttribute(pk->kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pk->smem) !=
            cudaSuccess) {
            cudaGetLastError();
            return fail(h, SJBG_E_UNSUPPORTED, "persistent sort-merge batch does not fit shared memory");
        }
    }
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, pk->kernel, kPkThreads, pk->smem) != cudaSuccess ||
        occ < 1) {
        cudaGetLastError();
        return fail(h, SJBG_E_UNSUPPORTED, "persistent eager kernel does not fit an SM");
    }
    // HJ: one tuple per thread of a 4,096-tuple batch (fewer CTAs, fewer arrivals per
    // ticket), the rest of the GPU stays free; NLJ and SMJ: the whole GPU (their
    // tickets are compare- or bandwidth-heavy).  Measured per ticket: the SMJ at
    // W = 2^20 takes 52 us with 2 CTAs per SM and 45 us with 4; the NLJ at
    // W = 65,536 takes 26 us with 2 and 37 us with 4 (its blocks are fewer than
    // the slots of 4 per SM, and every CTA joins each grid barrier)
    const int per_sm = h->cfg.algorithm == SJBG_ALG_SMJ ? 4 : 2;
    pk->grid = h->cfg.algorithm == SJBG_ALG_HJ ? std::min(16, h->num_sms) : std::min(occ, per_sm) * h->num_sms;
    int pageable = 0;
    if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, h->device) != cudaSuccess) {
        cudaGetLastError();
        pageable = 0;
    }
    pk->host_direct = pageable != 0;
    pk->count.assign(pk->Q, 0);
    pk->status.assign(pk->Q, 0);
    pk->snap.assign(pk->Q, WinAcc{0, 0, 0, 0, 0});
    st.pk.reset(pk.release());
    return SJBG_OK;
}

static int pk_launch(sjbg_handle *h) {
    EagerState &st = *h->eager;
    PkState &pk = *st.pk;
    if (pk.reset_state) {
        SJBG_CK(h, cudaMemsetAsync(pk.dev, 0, sizeof(PkDev), pk.stream));
        pk.reset_state = false;
    } else {
        SJBG_CK(h, cudaMemsetAsync(&pk.dev->sync, 0, sizeof(PkSync), pk.stream));
    }
    PkArgs a;
    std::memset(&a, 0, sizeof(a));
    a.desc = pk.ddesc;
    a.res = pk.dres;
    a.ctl = pk.dctl;
    a.dev = pk.dev;
    a.first_ticket = pk.done;   // every ticket before it is complete; later ones are in the queue or to come
    a.idle_ns = pk_idle_ms(h) * 1000000ull;
    a.cap = st.cap;
    a.Q = pk.Q;
    a.batch_cap = (uint32_t)pk.slot;
    const uint32_t bits = st.table_bits;
    for (int s = 0; s < 2; s++) {
        EagerSide &S = st.side[s];
        a.tuples[s] = S.tuples;
        a.tab[s] = ETab{S.tkeys, S.tcnt, S.thead, S.next, S.tsum, bits};
        a.skeys[s][0] = S.skeys;
        a.skeys[s][1] = S.skeys2;
        a.svals[s][0] = S.svals;
        a.svals[s][1] = S.svals2;
        a.F[s][0] = S.F;
        a.F[s][1] = pk.F2[s];
    }
    a.bkeys = pk.bkeys;
    a.bvals = pk.bvals;
    a.bF = pk.bF;
    a.stage = pk.stage;
    a.acc = st.acc;
    a.pairs = st.pairs;
    a.pairs_cap = st.pairs_cap;
    host_release(&pk.hctl->state, kPkRunning);
    void *args[] = {&a};
    const cudaError_t e = cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(pk.kernel), dim3(pk.grid),
                                                      dim3(kPkThreads), args, pk.smem, pk.stream);
    if (e != cudaSuccess) {
        host_release(&pk.hctl->state, kPkNotRunning);
        return cuda_fail(h, e, "persistent eager kernel launch");
    }
    pk.running = true;
    pk.launches++;
    h->launches++;
    return SJBG_OK;
}

// Read finished results in ticket order.
static void pk_harvest(PkState &pk) {
    while (pk.done < pk.next) {
        const PkResult &r = pk.hres[pk.done % pk.Q];
        if (host_acquire(&r.seq) != pk.done + 1) break;
        const uint32_t i = (uint32_t)(pk.done % pk.Q);
        pk.count[i] = r.count;
        pk.status[i] = r.status;
        pk.snap[i] = WinAcc{r.win_count, r.win_xor, r.win_prod, r.win_pairs, 0};
        if (r.status & kErrTimeout) pk.broken = true;
        pk.done++;
    }
}

// When the kernel has returned: find out why and, after an idle expiry,
// relaunch it if tickets are waiting.  Called between polls.
static int pk_check(sjbg_handle *h, bool relaunch) {
    PkState &pk = *h->eager->pk;
    if (!pk.running) return relaunch && pk.done < pk.next ? pk_launch(h) : SJBG_OK;
    const unsigned long long state = host_acquire(&pk.hctl->state);
    if (state == kPkRunning) return SJBG_OK;
    if (pk_sync_stream(pk) != SJBG_OK) return fail(h, SJBG_E_CUDA, "persistent eager kernel failed");
    pk.running = false;
    pk_harvest(pk);
    if (state == kPkIdleExit) pk.idle_exits++;
    if (state == kPkFailed) {
        pk.broken = true;
        return fail(h, SJBG_E_TIMEOUT, "a bounded wait of the persistent eager kernel gave up");
    }
    return relaunch && pk.done < pk.next ? pk_launch(h) : SJBG_OK;
}

// Wait for every ticket < upto to be read; bounded.
static int pk_drain_to(sjbg_handle *h, uint64_t upto) {
    PkState &pk = *h->eager->pk;
    const auto deadline = std::chrono::steady_clock::now() + std::chrono::milliseconds(pk_idle_ms(h) + 2000);
    uint32_t spins = 0;
    for (;;) {
        pk_harvest(pk);
        if (pk.done >= upto) return SJBG_OK;
        if (int rc = pk_check(h, true)) return rc;
        if (++spins > 64) {
            if (std::chrono::steady_clock::now() > deadline)
                return fail(h, SJBG_E_TIMEOUT, "the persistent eager kernel did not answer in time");
            std::this_thread::yield();
        }
    }
}

// Post one ticket.  For a batch, `src` is a device-visible address that stays
// valid until the ticket completes, or null to copy `host` into the slot.
static int pk_post(sjbg_handle *h, uint32_t cmd, int side, const sjbg_tuple *host, const sjbg_tuple *src,
                   uint64_t n, uint64_t *ticket) {
    EagerState &st = *h->eager;
    if (!st.pk) {
        if (int rc = pk_init(h)) return rc;
    }
    PkState &pk = *st.pk;
    if (cmd == kPkBatch) {
        if (pk.broken) return fail(h, SJBG_E_STATE, "a ticket failed on the device: clear the window first");
        if (pk.side_posted[side] + n > st.cap)
            return fail(h, SJBG_E_CAPACITY, "eager window exceeds its capacity (window_size + batch_size)");
        if (n > pk.slot) return fail(h, SJBG_E_INVALID, "a batch larger than batch_size");
    }
    const uint64_t t = pk.next;
    if (t >= pk.Q)
        if (int rc = pk_drain_to(h, t - pk.Q + 1)) return rc;   // the slot's previous ticket is read
    PkDesc &d = pk.hdesc[t % pk.Q];
    unsigned long long addr = 0;
    if (cmd == kPkBatch) {
        if (src && (reinterpret_cast<uintptr_t>(src) & 15) == 0) {
            addr = reinterpret_cast<unsigned long long>(src);
        } else if (host) {
            sjbg_tuple *slot = pk.hpay + (t % pk.Q) * pk.slot;
            if (n) std::memcpy(slot, host, sizeof(sjbg_tuple) * n);
            addr = reinterpret_cast<unsigned long long>(pk.dpay + (t % pk.Q) * pk.slot);
        } else {
            return fail(h, SJBG_E_INVALID, "device batches of a persistent handle must be 16-byte aligned");
        }
        pk.side_posted[side] += n;
    }
    if (cmd == kPkClear) {
        pk.side_posted[0] = pk.side_posted[1] = 0;
        pk.broken = false;
    }
    d.src = addr;
    d.cmd = cmd;
    d.side = (uint32_t)side;
    d.n = (uint32_t)n;
    host_release(&d.seq, t + 1);
    pk.next = t + 1;
    if (ticket) *ticket = t;
    return pk_check(h, true);
}

static int pk_wait(sjbg_handle *h, uint64_t t, unsigned long long *count, WinAcc *snap) {
    PkState &pk = *h->eager->pk;
    if (t >= pk.next || pk.next - t > pk.Q) return fail(h, SJBG_E_INVALID, "no such ticket (or its result was overwritten)");
    if (int rc = pk_drain_to(h, t + 1)) return rc;
    const uint32_t i = (uint32_t)(t % pk.Q);
    if (count) *count = pk.count[i];
    if (snap) *snap = pk.snap[i];
    const unsigned long long bits = pk.status[i];
    if (bits & kErrTimeout) return fail(h, SJBG_E_TIMEOUT, "a bounded wait of the persistent eager kernel gave up");
    if (bits) return fail(h, SJBG_E_CAPACITY, "the persistent eager kernel refused a ticket outside its buffers");
    return SJBG_OK;
}

// ---- entry points used by eager.cu on SJBG_F_PERSISTENT handles
int pk_execute(sjbg_handle *h, const sjbg_tuple *batch, uint64_t n, int side, bool from_host, uint64_t *match) {
    const sjbg_tuple *src = nullptr;
    if (!h->eager->pk)
        if (int rc = pk_init(h)) return rc;
    if (!from_host) {
        src = batch;
    } else if (h->eager->pk->host_direct) {
        // the device reads host memory coherently through the host's page tables:
        // the kernel takes the caller's batch in place (the call waits for the result)
        src = batch;
    } else {
        // pinned caller memory is read by the kernel in place (the call waits for the result)
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, batch) == cudaSuccess && at.type == cudaMemoryTypeHost && at.devicePointer)
            src = static_cast<const sjbg_tuple *>(at.devicePointer);
        else
            cudaGetLastError();
    }
    uint64_t t = 0;
    if (int rc = pk_post(h, kPkBatch, side, batch, src, n, &t)) return rc;
    unsigned long long c = 0;
    if (int rc = pk_wait(h, t, &c, nullptr)) return rc;
    if (match) *match = c;
    return SJBG_OK;
}

int pk_post_batch(sjbg_handle *h, const sjbg_tuple *batch, uint64_t n, int side, bool from_host, uint64_t *ticket) {
    return pk_post(h, kPkBatch, side, batch, from_host ? nullptr : batch, n, ticket);
}

int pk_wait_batch(sjbg_handle *h, uint64_t ticket, uint64_t *match) {
    if (!h->eager->pk) return fail(h, SJBG_E_INVALID, "no ticket was posted");
    unsigned long long c = 0;
    if (int rc = pk_wait(h, ticket, &c, nullptr)) return rc;
    if (match) *match = c;
    return SJBG_OK;
}

int pk_clear_states(sjbg_handle *h) {
    uint64_t t = 0;
    if (int rc = pk_post(h, kPkClear, 0, nullptr, nullptr, 0, &t)) return rc;
    return pk_wait(h, t, nullptr, nullptr);
}

int pk_report(sjbg_handle *h, WinAcc *totals) {
    uint64_t t = 0;
    if (int rc = pk_post(h, kPkReport, 0, nullptr, nullptr, 0, &t)) return rc;
    return pk_wait(h, t, nullptr, totals);
}

// Stop the kernel (it is relaunched by the next post).  `reset` also clears
// the device window state at the next launch (another path changed it).
int pk_stop(sjbg_handle *h, bool reset) {
    EagerState &st = *h->eager;
    if (!st.pk) return SJBG_OK;
    PkState &pk = *st.pk;
    if (int rc = pk_check(h, false)) return rc;
    if (pk.running) {
        uint64_t t = 0;
        if (int rc = pk_post(h, kPkStop, 0, nullptr, nullptr, 0, &t)) return rc;
        if (int rc = pk_drain_to(h, t + 1)) return rc;
        if (pk_sync_stream(pk) != SJBG_OK) return fail(h, SJBG_E_CUDA, "persistent eager kernel failed");
        pk.running = false;
    }
    if (reset) {
        pk.reset_state = true;
        pk.side_posted[0] = pk.side_posted[1] = 0;
        pk.broken = false;
    }
    return SJBG_OK;
}

int pk_status(sjbg_handle *h, int *running, uint64_t *launches) {
    EagerState &st = *h->eager;
    if (!st.pk) {
        if (running) *running = 0;
        if (launches) *launches = 0;
        return SJBG_OK;
    }
    PkState &pk = *st.pk;
    if (int rc = pk_check(h, false)) return rc;
    if (running) *running = pk.running ? 1 : 0;
    if (launches) *launches = pk.launches;
    if (pk.idle_exits > pk.idle_reported) {
        pk.idle_reported = pk.idle_exits;
        return fail(h, SJBG_E_TIMEOUT,
                    "the persistent eager kernel's wait for the next batch ran out; it returned and is relaunched "
                    "by the next batch");
    }
    return SJBG_OK;
}

void PkDeleter::operator()(PkState *p) const { delete p; }

}  // namespace sjbg
