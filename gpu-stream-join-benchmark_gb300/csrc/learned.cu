// learned.cu - learned key-CDF partitioner: sampling, least-squares fit and
// model check (no reference counterpart).
//
// Per window, on the device:
//   1. sample      rate * (|L|+|R|) keys at jittered strided positions of both
//                  sides, gathered once into a packed key array; per-window
//                  min/max key.
//   2. count       equal-width histogram of the sample over kBins key bins and
//                  exact per-key sample counts in a per-window hash table; the
//                  keys reaching the candidate threshold are listed and the
//                  listed keys are counted per count class as they grow.
//   3. heavy       listed keys whose sample count exceeds one bucket's fair
//                  share become candidates.
//   4. fit         (one CTA per window) the top kMaxHeavy candidates are made
//                  heavy and removed from the histogram; the light CDF at the
//                  bin edges is fitted by least squares: a root line routes
//                  points to `leaves` leaves, each leaf gets its own line
//                  (centred sums, two passes); lo/hi clamps make it monotone.
//   5. check       (inference) the model buckets the light sample; if the
//                  largest predicted bucket exceeds overflow_bound times the
//                  mean, the window falls back to radix partitioning.  It also
//                  keeps radix (by cost) when heavy keys hold little of the
//                  sample and radix buckets the whole sample evenly.
#include <algorithm>
#include <cstring>
#include <vector>

#include "learned.cuh"
#include "runtime.h"

namespace sjbg {

constexpr uint32_t kBins = 1u << 14;     // histogram bins of the fit (held in shared memory)
constexpr uint32_t kCandMax = 2048;       // heavy candidates kept per window
constexpr uint32_t kSampleThreads = 256;
constexpr uint32_t kPredStride = 1u << 14;  // predicted-bucket counters per window (max buckets)
// A window keeps radix partitioning (by cost) when heavy keys hold less than
// this share of its sample and radix's largest sampled bucket is at most this
// many times the mean: measured at z = 0.5 over 2^24 keys, the learned
// classification then costs more per tuple than its buckets save.
constexpr float kCostHeavyShare = 0.10f;
constexpr float kCostRadixBalance = 2.0f;

struct SampleWin {
    uint64_t left_off, n_left, right_off, n_right;
    uint32_t m;            // samples (even)
    uint32_t table_log2;   // per-window sample count table
    uint64_t table_off;    // first slot of this window's table
    uint32_t thresh;       // heavy candidate threshold (sample count)
    uint32_t log2_buckets;
    uint32_t run_log2;     // samples are runs of 2^run_log2 consecutive tuples (3, or 0 for tiny windows)
    uint32_t pad0;
    uint64_t key_off;      // first sampled key of this window in the packed key array
    uint64_t list_off;     // first entry of this window's list of keys at or above thresh
    uint32_t list_cap;     // m / thresh + 1: every listed key has at least thresh samples
    uint32_t pad;
    uint64_t stride[2];    // tuples between run starts, left and right side: n / (runs per side)
};

struct SampleScratch {
    uint32_t kmin, kmax;   // sample key range
    uint32_t n_cand;
    uint32_t cut;          // candidates have a sample count >= cut
    uint32_t cls[32];      // listed keys per count class floor(log2(count))
    uint32_t n_list;       // keys that reached thresh (table slots in the list)
    uint32_t pad[3];
};

// Sample i of a window: the samples come in runs of 2^run_log2 consecutive
// tuples (one 128-byte line for runs of 8), even runs from the left side, odd
// from the right; the j-th run of a side lies in the j-th of its equal strides,
// at a hashed offset inside it (the high half of hash * room: no division),
// moved to the nearest line start.
__device__ __forceinline__ uint32_t sample_key(const SampleWin &s, const sjbg_tuple *L, const sjbg_tuple *R, uint32_t i) {
    const uint32_t run = 1u << s.run_log2;
    const uint32_t r = i >> s.run_log2, q = i & (run - 1u);
    const bool right = r & 1u;
    const uint64_t n = right ? s.n_right : s.n_left;
    const uint64_t j = r >> 1;
    const uint64_t stride = right ? s.stride[1] : s.stride[0];   // >= run by construction of m, < 2^32 for n < 2^36
    const uint64_t room = stride - run + 1;
    const uint64_t jit = ((uint64_t)(uint32_t)sjbg_mix64(0x5A17ull + r) * (room & 0xFFFFFFFFull)) >> 32;
    const sjbg_tuple *side = right ? R + s.right_off : L + s.left_off;
    uint64_t idx = j * stride + jit;
    if (run == 8) {
        // a run of 8 tuples starts on a 128-byte line: one line per run, not two.
        // Rounded down, or up when down would leave the run's stride.
        const uint64_t a = ((uintptr_t)(side + idx) >> 4) & 7u;
        idx = idx - a >= j * stride && idx >= a ? idx - a : idx + ((8u - a) & 7u);
    }
    idx += q;
    if (idx >= n) idx = n - 1;
    return side[idx].key;
}

// Gathers each window's sample into the packed key array (four independent
// loads per thread in flight) and its min/max key.
__global__ void __launch_bounds__(kSampleThreads)
sample_minmax_kernel(const sjbg_tuple *L, const sjbg_tuple *R, const SampleWin *wins, SampleScratch *scr,
                     uint32_t *keys) {
    const uint32_t w = blockIdx.y;
    const SampleWin s = wins[w];
    uint32_t *kw = keys + s.key_off;
    uint32_t lo = 0xFFFFFFFFu, hi = 0;
    const uint32_t step = gridDim.x * blockDim.x;
    for (uint32_t i0 = blockIdx.x * blockDim.x + threadIdx.x; i0 < s.m; i0 += 4 * step) {
        uint32_t k[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const uint32_t i = i0 + q * step;
            k[q] = i < s.m ? sample_key(s, L, R, i) : 0u;
        }
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const uint32_t i = i0 + q * step;
            if (i < s.m) {
                kw[i] = k[q];
                lo = min(lo, k[q]);
                hi = max(hi, k[q]);
            }
        }
    }
    // one pair of global atomics per CTA (every CTA of a window updates the same two words)
    __shared__ uint32_t lo_s, hi_s;
    if (threadIdx.x == 0) {
        lo_s = 0xFFFFFFFFu;
        hi_s = 0;
    }
    lo = __reduce_min_sync(0xFFFFFFFFu, lo);
    hi = __reduce_max_sync(0xFFFFFFFFu, hi);
    SJBG_BARRIER();
    if (lane_id() == 0) {
        atomicMin(&lo_s, lo);
        atomicMax(&hi_s, hi);
    }
    SJBG_BARRIER();
    if (threadIdx.x == 0) {
        atomicMin(&scr[w].kmin, lo_s);
        atomicMax(&scr[w].kmax, hi_s);
    }
}

__device__ __forceinline__ float key_x(uint32_t key, float kmin, float inv) {
    return fminf(fmaxf(((float)key - kmin) * inv, 0.0f), 1.0f);
}
__device__ __forceinline__ void model_range(const SampleScratch &sc, float *kmin, float *inv) {
    *kmin = (float)sc.kmin;
    float range = (float)sc.kmax - (float)sc.kmin;
    *inv = range > 0.0f ? 1.0f / range : 0.0f;
}
__device__ __forceinline__ uint32_t bin_of(float x) {
    uint32_t b = (uint32_t)(x * (float)kBins);
    return b < kBins ? b : kBins - 1;
}

// Sample histogram + exact sample counts (table slot = key << 32 | count).
// A CTA aggregates kCountChunk sampled keys at a time in a shared table, then
// adds each distinct key's count once to the window's histogram and table.
// Each table update moves its key between count classes; a key's updates are
// ordered by the atomics, so every class change is counted exactly once, and
// the update that lifts a key to thresh lists its slot.
constexpr uint32_t kCountChunk = 2048;
constexpr uint32_t kCountSlotsLog2 = 12;   // 2 * kCountChunk slots: a free slot always exists
constexpr uint32_t kCountSlots = 1u << kCountSlotsLog2;
constexpr uint32_t kNoKey = 0xFFFFFFFFu;   // empty shared slot (the key itself counts in slot kCountSlots)
constexpr uint32_t kCountPer = kCountChunk / kSampleThreads;   // keys per thread and chunk
static_assert(kCountChunk % kSampleThreads == 0 && kCountSlots + 1 <= 0xFFFFu, "chunk layout");

// The count-class changes and the newly listed slots of a CTA's chunk are
// gathered in shared memory and added to the window's counters once per chunk
// (cls_d: per class, the change; list_s / n_list_s: the slots that reached
// thresh): every CTA of a window updates the same few class counters, and one
// global atomic per change serialised there.
__device__ __forceinline__ void count_update(const SampleWin &s, uint32_t *hw, unsigned long long *tw, int *cls_d,
                                             uint32_t *list_s, uint32_t *n_list_s, float kmin, float inv, uint32_t k,
                                             uint32_t c) {
    const uint32_t mask = (1u << s.table_log2) - 1;
    atomicAdd(&hw[bin_of(key_x(k, kmin, inv))], c);
    uint32_t slot = slot_hash(k, s.table_log2);
    uint32_t before = 0xFFFFFFFFu;   // the key's count before this update
    // the compare-and-swap claims an empty slot or returns the slot's key (a
    // count is at least 1, so a taken slot is never 0): one round trip for a
    // key new to the table, two for a key already in it
    for (uint32_t p = 0; p <= mask; p++) {
        const unsigned long long prev = atomicCAS(&tw[slot], 0ull, ((unsigned long long)k << 32) | c);
        if (prev == 0ull) {
            before = 0;
            break;
        }
        if ((uint32_t)(prev >> 32) == k) {
            before = (uint32_t)atomicAdd(&tw[slot], (unsigned long long)c);
            break;
        }
        slot = (slot + 1) & mask;
    }
    const uint32_t after = before + c;
    if (before == 0xFFFFFFFFu || after < s.thresh) return;   // (a full table drops the key)
    const int cn = 31 - __clz(after);
    if (before < s.thresh) {
        atomicAdd(&cls_d[cn], 1);
        list_s[atomicAdd(n_list_s, 1u)] = slot;   // at most one per distinct key of the chunk
    } else {
        const int co = 31 - __clz(before);
        if (co != cn) {
            atomicAdd(&cls_d[cn], 1);
            atomicSub(&cls_d[co], 1);
        }
    }
}

__global__ void __launch_bounds__(kSampleThreads)
sample_count_kernel(const uint32_t *keys, const SampleWin *wins, SampleScratch *scr, uint32_t *hist,
                    unsigned long long *table, uint32_t *lists) {
    __shared__ uint32_t skey[kCountSlots], scnt[kCountSlots + 1];
    __shared__ uint16_t used[kCountChunk + 1];   // slots taken by the chunk's distinct keys
    __shared__ uint32_t n_used;
    __shared__ int cls_d[32];                     // the chunk's count-class changes
    __shared__ uint32_t list_s[kCountChunk + 1];  // the chunk's newly listed table slots
    __shared__ uint32_t n_list_s, list_base;
    const uint32_t w = blockIdx.y;
    const SampleWin s = wins[w];
    float kmin, inv;
    model_range(scr[w], &kmin, &inv);
    const uint32_t *kw = keys + s.key_off;
    uint32_t *hw = hist + (uint64_t)w * kBins;
    uint32_t *lw = lists + s.list_off;
    SampleScratch &sc = scr[w];
    unsigned long long *tw = table + s.table_off;
    for (uint32_t j = threadIdx.x; j <= kCountSlots; j += blockDim.x) {
        if (j < kCountSlots) skey[j] = kNoKey;
        scnt[j] = 0;
    }
    if (threadIdx.x == 0) {
        n_used = 0;
        n_list_s = 0;
    }
    if (threadIdx.x < 32) cls_d[threadIdx.x] = 0;
    SJBG_BARRIER();
    for (uint32_t base = blockIdx.x * kCountChunk; base < s.m; base += gridDim.x * kCountChunk) {
        const uint32_t end = min(base + kCountChunk, s.m);
        // all of a thread's keys of the chunk are loaded at once (one memory latency)
        uint32_t k[kCountPer];
#pragma unroll
        for (uint32_t q = 0; q < kCountPer; q++) {
            const uint32_t i = base + q * kSampleThreads + threadIdx.x;
            k[q] = i < end ? kw[i] : kNoKey;
        }
        // lanes holding the same key are counted once, by the lowest of them,
        // so a skewed chunk's heaviest keys cost one shared atomic per warp;
        // a slot taken for the first time is listed for the flush
#pragma unroll
        for (uint32_t q = 0; q < kCountPer; q++) {
            const bool has = base + q * kSampleThreads + threadIdx.x < end;
            const uint32_t same = __match_any_sync(0xFFFFFFFFu, k[q]) & __ballot_sync(0xFFFFFFFFu, has);
            if (has && lane_id() == (uint32_t)(__ffs(same) - 1)) {
                const uint32_t c = __popc(same);
                if (k[q] == kNoKey) {
                    if (atomicAdd(&scnt[kCountSlots], c) == 0u) used[atomicAdd(&n_used, 1u)] = (uint16_t)kCountSlots;
                } else {
                    uint32_t slot = slot_hash(k[q], kCountSlotsLog2);
                    for (uint32_t p = 0; p < kCountSlots; p++) {
                        const uint32_t prev = atomicCAS(&skey[slot], kNoKey, k[q]);
                        if (prev == kNoKey || prev == k[q]) {
                            if (prev == kNoKey) used[atomicAdd(&n_used, 1u)] = (uint16_t)slot;
                            atomicAdd(&scnt[slot], c);
                            break;
                        }
                        slot = (slot + 1) & (kCountSlots - 1);
                    }
                }
            }
        }
        SJBG_BARRIER();
        // one global update per distinct key of the chunk, from the list of taken slots
        const uint32_t nu = n_used;
        for (uint32_t u = threadIdx.x; u < nu; u += blockDim.x) {
            const uint32_t j = used[u];
            count_update(s, hw, tw, cls_d, list_s, &n_list_s, kmin, inv, j < kCountSlots ? skey[j] : kNoKey,
                         scnt[j]);
            if (j < kCountSlots) skey[j] = kNoKey;
            scnt[j] = 0;
        }
        SJBG_BARRIER();
        // the chunk's class changes and listed slots into the window's counters and list
        if (threadIdx.x < 32 && cls_d[threadIdx.x] != 0) {
            atomicAdd(&sc.cls[threadIdx.x], (uint32_t)cls_d[threadIdx.x]);   // (a negative change wraps)
            cls_d[threadIdx.x] = 0;
        }
        const uint32_t nl = n_list_s;
        if (threadIdx.x == 0) {
            list_base = nl ? atomicAdd(&sc.n_list, nl) : 0u;
            n_used = 0;
        }
        SJBG_BARRIER();
        for (uint32_t i = threadIdx.x; i < nl; i += blockDim.x)
            if (list_base + i < s.list_cap) lw[list_base + i] = list_s[i];
        SJBG_BARRIER();
        if (threadIdx.x == 0) n_list_s = 0;
    }
}

// The smallest count class boundary 2^k (>= thresh) above which at most
// kCandMax keys lie: every key counted more often than any dropped key is kept.
__device__ __forceinline__ uint32_t candidate_cut(const SampleScratch &sc, uint32_t thresh) {
    uint32_t acc = 0;
    for (int k = 31; k >= 0; k--) {
        acc += sc.cls[k];
        if (acc > kCandMax) return max(thresh, k == 31 ? 0xFFFFFFFFu : (1u << (k + 1)));
    }
    return thresh;
}

// The listed keys (those that reached thresh) at or above the cut.
__global__ void __launch_bounds__(kSampleThreads)
heavy_candidates_kernel(const SampleWin *wins, const unsigned long long *table, SampleScratch *scr,
                        const uint32_t *lists, unsigned long long *cand) {
    const uint32_t w = blockIdx.y;
    const SampleWin s = wins[w];
    const unsigned long long *tw = table + s.table_off;
    const uint32_t *lw = lists + s.list_off;
    const uint32_t nl = min(scr[w].n_list, s.list_cap);
    const uint32_t cut = candidate_cut(scr[w], s.thresh);
    if (blockIdx.x == 0 && threadIdx.x == 0) scr[w].cut = cut;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nl; i += gridDim.x * blockDim.x) {
        const unsigned long long v = tw[lw[i]];
        const uint32_t c = (uint32_t)v;
        if (v && c >= cut) {
            uint32_t pos = atomicAdd(&scr[w].n_cand, 1u);
            // candidates sort by count descending, then key: (count << 32 | ~key)
            if (pos < kCandMax) cand[(uint64_t)w * kCandMax + pos] = ((unsigned long long)c << 32) | (~(uint32_t)(v >> 32));
        }
    }
}

// Exclusive scan of two 64-bit values over the CTA (all threads; ends with a
// barrier, so ws may be reused): returns the prefix of v1, stores the prefix
// of v2 in *ex2 (when given) and both totals.
__device__ __forceinline__ unsigned long long cta_excl_scan2(unsigned long long v1, unsigned long long v2,
                                                             unsigned long long *tot1, unsigned long long *tot2,
                                                             unsigned long long (*ws)[2],
                                                             unsigned long long *ex2 = nullptr) {
    const uint32_t lane = lane_id(), wid = warp_id(), nw = blockDim.x >> 5;
    unsigned long long x1 = v1, x2 = v2;
    for (uint32_t o = 1; o < 32; o <<= 1) {
        const unsigned long long y1 = __shfl_up_sync(0xFFFFFFFFu, x1, o), y2 = __shfl_up_sync(0xFFFFFFFFu, x2, o);
        if (lane >= o) {
            x1 += y1;
            x2 += y2;
        }
    }
    if (lane == 31) {
        ws[wid][0] = x1;
        ws[wid][1] = x2;
    }
    SJBG_BARRIER();
    if (wid == 0) {
        unsigned long long t1 = lane < nw ? ws[lane][0] : 0ull, t2 = lane < nw ? ws[lane][1] : 0ull;
        for (uint32_t o = 1; o < 32; o <<= 1) {
            const unsigned long long y1 = __shfl_up_sync(0xFFFFFFFFu, t1, o), y2 = __shfl_up_sync(0xFFFFFFFFu, t2, o);
            if (lane >= o) {
                t1 += y1;
                t2 += y2;
            }
        }
        __syncwarp();
        ws[lane][0] = t1;   // inclusive over warps
        ws[lane][1] = t2;
    }
    SJBG_BARRIER();
    const unsigned long long b1 = wid ? ws[wid - 1][0] : 0ull, b2 = wid ? ws[wid - 1][1] : 0ull;
    *tot1 = ws[nw - 1][0];
    *tot2 = ws[nw - 1][1];
    SJBG_BARRIER();
    if (ex2) *ex2 = b2 + x2 - v2;
    return b1 + x1 - v1;
}

// One CTA (1024 threads) per window.
__global__ void __launch_bounds__(1024)
learned_fit_kernel(const SampleWin *wins, SampleScratch *scr, uint32_t *hist, unsigned long long *cand,
                   LearnedModel *models, uint32_t leaves, uint32_t max_heavy, float bound) {
    extern __shared__ uint32_t fit_smem[];         // kBins histogram counters (dynamic)
    __shared__ unsigned long long sc[kCandMax];
    __shared__ float lfit[kMaxLeaves][5];          // per leaf: n, mean x, mean y, slope, largest y
    __shared__ uint32_t lstart[kMaxLeaves + 1];     // first bin of each leaf
    __shared__ uint32_t warp_tot[32];
    __shared__ unsigned long long wsum[32][2];
    __shared__ unsigned long long bsum[kMaxLeaves + 1][2];   // S1 and S2 at each leaf's first bin
    __shared__ float root_s[2];
    __shared__ uint32_t n_heavy_s, light_total_s, log2_eff_s, compact_s, cost_s;
    __shared__ uint32_t cpre[kCandMax + 1];        // exclusive prefix of the sorted candidates' counts
    const uint32_t w = blockIdx.x;
    const SampleWin s = wins[w];
    LearnedModel &M = models[w];
    uint32_t *hw = hist + (uint64_t)w * kBins;
    float kmin, inv;
    model_range(scr[w], &kmin, &inv);

    // ---- heavy keys: bitonic sort of the candidates (descending), keep the top
    const uint32_t nc = min(scr[w].n_cand, kCandMax);
    for (uint32_t i = threadIdx.x; i < kCandMax; i += blockDim.x) sc[i] = i < nc ? cand[(uint64_t)w * kCandMax + i] : 0ull;
    SJBG_BARRIER();
    // Thread t holds elements t and t + 1024 in registers.  Stages up to
    // ncap (the candidates rounded up to a power of two: the zeros beyond it
    // only meet zeros); partners j < 32 apart are exchanged by warp shuffles,
    // j = 1024 inside the thread, the others through shared memory.
    {
        static_assert(kCandMax == 2048, "two sort elements per thread of 1024");
        uint32_t ncap = 2;
        while (ncap < nc) ncap <<= 1;
        const uint32_t t = threadIdx.x;
        unsigned long long v0 = sc[t], v1 = sc[t + 1024];
        // element i with partner value pv: the lower index of a descending
        // pair (and the upper of an ascending one) keeps the larger value
        // (values are distinct keys' entries, or equal zeros of the padding)
        auto cx = [](unsigned long long v, unsigned long long pv, uint32_t i, uint32_t j, uint32_t k) {
            const bool keep_larger = ((i & j) == 0) == ((i & k) == 0);
            return (v > pv) == keep_larger ? v : pv;
        };
        // up to 1,024 candidates the second elements are all padding (zeros
        // meet only zeros): the whole CTA skips them
        const bool two = ncap > 1024;
        for (uint32_t k = 2; k <= ncap; k <<= 1) {
            for (uint32_t j = k >> 1; j > 0; j >>= 1) {
                if (j == 1024) {   // k = 2048: descending, element t is the lower one
                    const unsigned long long hi = v0 > v1 ? v0 : v1, lo = v0 > v1 ? v1 : v0;
                    v0 = hi;
                    v1 = lo;
                } else if (j >= 32) {
                    sc[t] = v0;
                    if (two) sc[t + 1024] = v1;
                    SJBG_BARRIER();
                    const unsigned long long p0 = sc[t ^ j];
                    const unsigned long long p1 = two ? sc[(t ^ j) + 1024] : 0ull;
                    SJBG_BARRIER();
                    v0 = cx(v0, p0, t, j, k);
                    if (two) v1 = cx(v1, p1, t + 1024, j, k);
                } else {
                    v0 = cx(v0, __shfl_xor_sync(0xFFFFFFFFu, v0, j), t, j, k);
                    if (two) v1 = cx(v1, __shfl_xor_sync(0xFFFFFFFFu, v1, j), t + 1024, j, k);
                }
            }
        }
        sc[t] = v0;
        sc[t + 1024] = v1;
        SJBG_BARRIER();
    }
    // largest first, a candidate is heavy while its sampled count exceeds an
    // eighth of one bucket's share of the mass that is still light: the first
    // h with c_h * 8P <= m - (c_0 + .. + c_{h-1}) ends the heavy keys
    const uint64_t P = 1ull << s.log2_buckets;
    const uint32_t lim = min(nc, max_heavy);
    {
        const uint32_t per = kCandMax / blockDim.x, h0 = threadIdx.x * per;   // 2 candidates per thread
        uint32_t sum = 0;
        for (uint32_t q = 0; q < per; q++) sum += (uint32_t)(sc[h0 + q] >> 32);
        uint32_t tot;
        const uint32_t ex = warp_excl_scan(sum, &tot);
        if (lane_id() == 31) warp_tot[warp_id()] = ex + sum;
        if (threadIdx.x == 0) n_heavy_s = lim;
        SJBG_BARRIER();
        if (warp_id() == 0) {
            const uint32_t x = lane_id() < (blockDim.x >> 5) ? warp_tot[lane_id()] : 0u;
            uint32_t tt;
            warp_tot[lane_id()] = warp_excl_scan(x, &tt);
            if (lane_id() == 0) cpre[kCandMax] = tt;
        }
        SJBG_BARRIER();
        uint32_t run = warp_tot[warp_id()] + ex;
        for (uint32_t q = 0; q < per; q++) {
            const uint32_t h = h0 + q;
            const uint32_t c = (uint32_t)(sc[h] >> 32);
            cpre[h] = run;
            if (h < lim && (uint64_t)c * 8 * P <= (uint64_t)s.m - run) atomicMin(&n_heavy_s, h);
            run += c;
        }
        SJBG_BARRIER();
    }
    if (threadIdx.x == 0) {
        const uint32_t h = n_heavy_s;
        const uint64_t light = (uint64_t)s.m - cpre[h];
        // fan-out for the light keys only: about as many light tuples per
        // bucket as the window's plan has tuples per bucket
        uint32_t lg = s.log2_buckets;
        while (lg > 0 && ((uint64_t)s.m << (lg - 1)) >= (light << s.log2_buckets)) lg--;
        // the largest light key must stay well inside the overflow bound
        const uint64_t c1 = h < nc ? (sc[h] >> 32) : (uint64_t)scr[w].cut;
        while (lg > 0 && 2.0 * (double)c1 * (double)(1ull << lg) > (double)bound * (double)light) lg--;
        log2_eff_s = lg;
        // when at most half of the sample is light, the counting pass also
        // writes the light tuples out compacted, and only those are re-read
        compact_s = (h > 0 && 2 * light <= s.m) ? 1u : 0u;
        cost_s = ((float)(s.m - light) < kCostHeavyShare * (float)s.m) ? 1u : 0u;
    }
    SJBG_BARRIER();
    const uint32_t nh = n_heavy_s;
    for (uint32_t h = threadIdx.x; h < nh; h += blockDim.x) M.heavy_keys[h] = ~(uint32_t)sc[h];
    SJBG_BARRIER();
    // the set's claim scratch is the histogram's space, free until the histogram is loaded
    static_assert(2u << kHeavyBucketsLog2 <= kBins, "claim scratch fits the histogram's space");
    heavy_set_build(M.heavy_set, M.heavy_keys, nh, fit_smem);   // ends with a barrier
    __shared__ uint8_t placed_s[kMaxHeavy];   // keys that found no slot stay light
    for (uint32_t h = threadIdx.x; h < nh; h += blockDim.x) placed_s[h] = heavy_placed(M.heavy_keys, h, fit_smem) ? 1 : 0;
    SJBG_BARRIER();

    // ---- the window's light histogram, in shared memory from here on
    uint32_t *hb = fit_smem;   // kBins counters, later the inclusive CDF counts
    for (uint32_t i = threadIdx.x; i < kBins; i += blockDim.x) hb[i] = hw[i];
    SJBG_BARRIER();
    for (uint32_t h = threadIdx.x; h < nh; h += blockDim.x)
        if (placed_s[h]) atomicSub(&hb[bin_of(key_x(M.heavy_keys[h], kmin, inv))], (uint32_t)(sc[h] >> 32));
    SJBG_BARRIER();

    // ---- the light CDF at the bin edges, and its running sums, in integers.
    // Thread t owns bins [t * pt, (t + 1) * pt).  With cdf_j the inclusive
    // count of bin j, S1(j) = sum_{i<j} cdf_i and S2(j) = sum_{i<j} i * cdf_i
    // are exact; every least-squares sum below is a difference of them or a
    // closed form in the bin index, so no sum is formed in floating point.
    const uint32_t nwarps = blockDim.x >> 5;
    const uint32_t wid = warp_id(), lane = lane_id();
    const uint32_t pt = kBins / blockDim.x, jb = threadIdx.x * pt;
    uint32_t cnt = 0;
    unsigned long long a1 = 0, a2 = 0;   // the chunk's own inclusive counts: their sum, and sum j * them
    for (uint32_t q = 0; q < pt; q++) {
        cnt += hb[jb + q];
        a1 += cnt;
        a2 += (unsigned long long)(jb + q) * cnt;
    }
    unsigned long long tot_cnt, dummy;
    const unsigned long long before = cta_excl_scan2(cnt, 0ull, &tot_cnt, &dummy, wsum);   // counts ahead of the chunk
    // the chunk's share of S1 and S2: every inclusive count is `before` higher than its local one
    const unsigned long long sj = (unsigned long long)pt * jb + (unsigned long long)pt * (pt - 1) / 2;
    unsigned long long s1k, s2k;
    unsigned long long e1 = 0, e2 = 0;
    e1 = cta_excl_scan2(pt * before + a1, before * sj + a2, &s1k, &s2k, wsum, &e2);
    if (threadIdx.x == 0) light_total_s = (uint32_t)tot_cnt;
    for (uint32_t l = threadIdx.x; l <= leaves; l += blockDim.x) {
        lstart[l] = kBins;
        bsum[l][0] = s1k;
        bsum[l][1] = s2k;
    }
    SJBG_BARRIER();
    const uint32_t total = light_total_s;
    const float invt = total ? 1.0f / (float)total : 0.0f;

    // ---- root line y = a x + b over the bin points x_j = (j + 1) / kBins, y_j = cdf_j / total:
    // sum x and sum x^2 are closed forms, sum y = S1(K) / total, sum x y = (S2(K) + S1(K)) / (K total)
    if (threadIdx.x == 0) {
        const double nn = kBins, it = total ? 1.0 / (double)total : 0.0;
        const double sy = (double)s1k * it, sxy = ((double)s2k + (double)s1k) * it / nn;
        const double sx = (nn + 1.0) / 2.0, sxx = (nn + 1.0) * (2.0 * nn + 1.0) / (6.0 * nn);
        const double den = nn * sxx - sx * sx;
        double ra = den != 0.0 ? (nn * sxy - sx * sy) / den : 1.0;
        if (!(ra > 0.0)) ra = 1.0;   // the root must increase with the key
        root_s[0] = (float)ra;
        root_s[1] = (float)((sy - ra * sx) / nn);
    }
    SJBG_BARRIER();
    const float root_a = root_s[0], root_b = root_s[1];
    auto leaf_of = [&](uint32_t j) {
        const float x = (float)(j + 1) / (float)kBins;
        int l = (int)floorf((root_a * x + root_b) * (float)leaves);
        return min(max(l, 0), (int)leaves - 1);
    };
    // leaf_of is non-decreasing in j, so every leaf owns a contiguous run of
    // bins: the first bin of leaf l is where leaf_of first reaches l.  The
    // owner of that bin records it with S1 and S2 there, and stores its CDF.
    {
        unsigned long long s1 = e1, s2 = e2;
        uint32_t run = before;
        int lp = jb ? leaf_of(jb - 1) : -1;
        for (uint32_t q = 0; q < pt; q++) {
            const uint32_t j = jb + q;
            const int lj = leaf_of(j);
            for (int l = lp + 1; l <= lj; l++) {
                lstart[l] = j;
                bsum[l][0] = s1;
                bsum[l][1] = s2;
            }
            lp = lj;
            run += hb[j];
            hb[j] = run;
            s1 += run;
            s2 += (unsigned long long)j * run;
        }
    }
    SJBG_BARRIER();

    // ---- one thread per leaf: least-squares line over the leaf's bins [j0, j1),
    // centred at the leaf's mean x.  With c = j1 - j0 bins:
    //   mean x = (j0 + j1 + 1) / 2K,  sum dx^2 = c (c^2 - 1) / 12K^2,
    //   sum dx dy = sum dx y = (2 S2 - (j0 + j1 - 1) S1) / (2K total)  (S1, S2 over the leaf)
    for (uint32_t l = threadIdx.x; l < leaves; l += blockDim.x) {
        const uint32_t j0 = lstart[l], j1 = lstart[l + 1];
        const uint32_t c = j1 > j0 ? j1 - j0 : 0u;
        float mx = 0.f, my = 0.f, slope = 0.f, mxv = -1.f;
        if (c) {
            const unsigned long long s1 = bsum[l + 1][0] - bsum[l][0];
            const long long s2 = (long long)(bsum[l + 1][1] - bsum[l][1]);
            const long long t = 2 * s2 - (long long)(j0 + j1 - 1) * (long long)s1;
            mx = (float)(j0 + j1 + 1) / (2.0f * (float)kBins);
            my = (float)s1 * invt / (float)c;
            mxv = (float)hb[j1 - 1] * invt;   // the CDF does not decrease: its value at the last bin
            if (c > 1) {
                const float fc = (float)c;
                slope = 6.0f * (float)kBins * invt * (float)t / (fc * (fc * fc - 1.0f));
                if (!(slope >= 0.f)) slope = 0.f;
            }
        }
        lfit[l][0] = (float)c;
        lfit[l][1] = mx;
        lfit[l][2] = my;
        lfit[l][3] = slope;
        lfit[l][4] = mxv;   // largest CDF value routed to the leaf (-1 when empty)
    }
    SJBG_BARRIER();
    // ---- monotone clamps: a leaf owns the CDF range from the largest value of
    // the leaves before it to its own largest value (prefix maximum over leaves);
    // empty leaves inherit the previous upper bound
    if (wid == 0) {
        const uint32_t chunk = (leaves + 31) / 32;
        const uint32_t l0 = lane * chunk, l1 = min(leaves, l0 + chunk);
        float m = 0.f;
        for (uint32_t l = l0; l < l1; l++) m = fmaxf(m, lfit[l][4]);
        float incl = m;
        for (int o = 1; o < 32; o <<= 1) {
            const float y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= (uint32_t)o) incl = fmaxf(incl, y);
        }
        float prev = __shfl_up_sync(0xFFFFFFFFu, incl, 1);
        if (lane == 0) prev = 0.f;
        for (uint32_t l = l0; l < l1; l++) {
            float lo, hi, slope, mx, my;
            if (lfit[l][0] < 1.f) {
                lo = hi = prev; slope = 0.f; mx = 0.f; my = prev;
            } else {
                mx = lfit[l][1]; my = lfit[l][2]; slope = lfit[l][3];
                lo = prev;
                hi = fmaxf(lfit[l][4], lo);
            }
            M.leaf[l] = make_float4(slope, my - slope * mx, lo, hi);
            prev = hi;
        }
        if (lane == 0) {
            M.kmin = kmin; M.inv_range = inv; M.root_a = root_a; M.root_b = root_b;
            M.leaves = leaves; M.log2_buckets = log2_eff_s; M.fallback = (total == 0 && nh == 0) ? 1u : 0u;
            M.n_heavy = nh;
            M.compact = compact_s;
            M.cost_check = cost_s;
        }
    }
}

// Inference on the sample: predicted bucket sizes of the light keys.
__global__ void __launch_bounds__(kSampleThreads)
learned_check_kernel(const uint32_t *keys, const SampleWin *wins, const LearnedModel *models, uint32_t *pred,
                     uint32_t *prad) {
    __shared__ HeavySet hs;
    __shared__ LearnedCore core;
    const uint32_t w = blockIdx.y;
    const SampleWin s = wins[w];
    const LearnedModel *m = &models[w];
    if (m->fallback) return;   // whole CTA
    heavy_set_load(hs, m);
    copy_to_smem(&core, m, sizeof(LearnedCore));
    uint32_t *pw = pred + (uint64_t)w * kPredStride;
    uint32_t *rw = prad + (uint64_t)w * kPredStride;
    const uint32_t *kw = keys + s.key_off;
    const uint32_t rmask = (1u << s.log2_buckets) - 1u;   // radix on the plan's fan-out, every key
    // four keys per thread loaded at once (one memory latency per four keys)
    const uint32_t step = gridDim.x * blockDim.x;
    for (uint32_t i0 = blockIdx.x * blockDim.x + threadIdx.x; i0 < s.m; i0 += 4 * step) {
        uint32_t k[4];
#pragma unroll
        for (int q = 0; q < 4; q++) k[q] = i0 + q * step < s.m ? kw[i0 + q * step] : 0u;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            if (i0 + q * step >= s.m) continue;
            if (core.cost_check) atomicAdd(&rw[k[q] & rmask], 1u);
            if (heavy_find(hs, k[q]) == kHeavyBucket) atomicAdd(&pw[learned_bucket(core, k[q])], 1u);
        }
    }
}

// One CTA per window: worst predicted bucket vs the mean -> fallback flag;
// the window's plan is pointed at its model slot.
__global__ void __launch_bounds__(1024)
learned_overflow_kernel(const SampleWin *wins, LearnedModel *models, const uint32_t *pred, const uint32_t *prad,
                        float bound, WinPlan *plan) {
    __shared__ uint32_t mx_s, sum_s, rmx_s;
    const uint32_t w = blockIdx.x;
    LearnedModel &M = models[w];
    if (threadIdx.x == 0) plan[w].model = w;
    if (M.fallback) return;
    if (threadIdx.x == 0) { mx_s = 0; sum_s = 0; rmx_s = 0; }
    SJBG_BARRIER();
    const uint32_t P = 1u << M.log2_buckets;
    const uint32_t *pw = pred + (uint64_t)w * kPredStride;
    uint32_t mx = 0, sm = 0;
    for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) { mx = max(mx, pw[i]); sm += pw[i]; }
    atomicMax(&mx_s, mx);
    atomicAdd(&sum_s, sm);
    // radix on the plan's fan-out, all sampled keys
    const SampleWin s = wins[w];
    const uint32_t PR = 1u << s.log2_buckets;
    const uint32_t *rw = prad + (uint64_t)w * kPredStride;
    uint32_t rmx = 0;
    for (uint32_t i = threadIdx.x; i < PR; i += blockDim.x) rmx = max(rmx, rw[i]);
    atomicMax(&rmx_s, rmx);
    SJBG_BARRIER();
    if (threadIdx.x == 0) {
        const float mean = (float)sum_s / (float)P;
        // a window whose light sample is too small to judge keeps its model
        if (sum_s >= 4 * P && (float)mx_s > bound * mean) {
            M.fallback = 1u;
        } else if (M.cost_check && s.m >= 4 * PR && (float)(s.m - sum_s) < kCostHeavyShare * (float)s.m &&
                   (float)rmx_s * (float)PR <= kCostRadixBalance * (float)s.m) {
            // heavy keys hold little of the sample and radix is balanced on it:
            // the model's per-tuple work (set lookup, leaf line) costs more than it saves
            M.fallback = 2u;
        }
    }
}

uint32_t learned_log2_buckets(sjbg_handle *h, uint64_t n_left) {
    if (h->cfg.radix_bits) return h->cfg.radix_bits;
    uint32_t b = 0;
    while (((uint64_t)h->tune.bucket_target << b) < n_left) b++;
    return b;
}

size_t learned_stage_bytes(uint32_t n) { return (sizeof(SampleWin) + sizeof(SampleScratch)) * (size_t)n; }

LearnedStage learned_stage(sjbg_handle *h, const WinPlan *plan, uint32_t n, uint8_t *hst) {
    const float rate = h->cfg.sample_rate > 0.0f ? h->cfg.sample_rate : 0.01f;
    LearnedStage st{};
    SampleWin *sw = reinterpret_cast<SampleWin *>(hst);
    for (uint32_t w = 0; w < n; w++) {
        const WinPlan &p = plan[w];
        SampleWin s;
        std::memset(&s, 0, sizeof(s));
        s.left_off = p.left_off; s.n_left = p.n_left; s.right_off = p.right_off; s.n_right = p.n_right;
        const uint64_t nmin = std::min(p.n_left, p.n_right);
        uint64_t m = (uint64_t)((double)rate * (double)(p.n_left + p.n_right));
        m = std::max<uint64_t>(m, 64);
        m = std::min<uint64_t>(m, 2 * nmin);   // at most one sample per tuple
        // runs of 8 tuples (whole 128-byte lines) once each side has room for
        // 8 runs: m a multiple of 16 samples, at most one per tuple
        s.run_log2 = (m >= 128 && nmin >= 64) ? 3u : 0u;
        m &= ~((2ull << s.run_log2) - 1);
        if (nmin == 0) m = 0;
        s.m = (uint32_t)m;
        uint32_t lg = 6;
        while (((uint64_t)1 << lg) < 2 * m) lg++;
        s.table_log2 = lg;
        s.table_off = st.table_total;
        st.table_total += (uint64_t)1 << lg;
        s.log2_buckets = p.log2_buckets;
        const uint64_t P = (uint64_t)1 << p.log2_buckets;
        // heavy candidates: keys sampled at least max(4, m / 64P) times; the fit
        // keeps those that exceed an eighth of a bucket of the remaining light mass
        s.thresh = (uint32_t)std::max<uint64_t>(4, m / (64 * P));
        s.key_off = st.keys_total;
        st.keys_total += m;
        s.list_cap = (uint32_t)(m / s.thresh + 1);
        s.list_off = st.list_total;
        st.list_total += s.list_cap;
        const uint64_t runs = m >> (s.run_log2 + 1);   // runs per side
        s.stride[0] = runs ? p.n_left / runs : 0;
        s.stride[1] = runs ? p.n_right / runs : 0;
        st.max_m = std::max(st.max_m, s.m);
        st.max_list = std::max(st.max_list, s.list_cap);
        std::memcpy(&sw[w], &s, sizeof(s));
    }
    SampleScratch init;
    std::memset(&init, 0, sizeof(init));
    init.kmin = 0xFFFFFFFFu;
    for (uint32_t w = 0; w < n; w++) std::memcpy(hst + sizeof(SampleWin) * n + sizeof(SampleScratch) * w, &init, sizeof(init));
    return st;
}

int learned_prepare(sjbg_handle *h, const sjbg_tuple *dL, const sjbg_tuple *dR, const LearnedStage &st,
                    uint8_t *dstage, uint32_t n, WinPlan *dPlan, const LearnedModel **dModels, bool allow_heavy) {
    const float bound = h->cfg.overflow_bound > 0.0f ? h->cfg.overflow_bound : 8.0f;
    const uint32_t leaves = h->cfg.learned_leaves ? std::min(h->cfg.learned_leaves, kMaxLeaves) : kMaxLeaves;
    const uint64_t table_total = st.table_total, keys_total = st.keys_total, list_total = st.list_total;
    const uint32_t max_m = st.max_m, max_list = st.max_list;
    const size_t swB = sizeof(SampleWin) * n;
    uint8_t *dsmall = dstage;
    const size_t histB = sizeof(uint32_t) * (size_t)kBins * n, tabB = sizeof(unsigned long long) * table_total;
    const size_t candB = sizeof(unsigned long long) * (size_t)kCandMax * n, predB = sizeof(uint32_t) * (size_t)n * kPredStride;
    // sample histograms, then the model's and radix's predicted bucket counts
    uint32_t *dHist = static_cast<uint32_t *>(ws_get(h, WS_AUX0, histB + 2 * predB));
    unsigned long long *dTab = static_cast<unsigned long long *>(ws_get(h, WS_AUX1, tabB));
    unsigned long long *dCand = static_cast<unsigned long long *>(ws_get(h, WS_AUX2, candB));
    LearnedModel *dM = static_cast<LearnedModel *>(ws_get(h, WS_MODEL, sizeof(LearnedModel) * n));
    // the packed sample keys of every window, then the windows' lists of keys at or above thresh
    uint32_t *dKeys = static_cast<uint32_t *>(ws_get(h, WS_SAMPLE_KEYS, sizeof(uint32_t) * (keys_total + list_total + 1)));
    if (!dHist || !dTab || !dCand || !dM || !dKeys)
        return fail(h, SJBG_E_NOMEM, "learned partitioner buffers");
    uint32_t *dLists = dKeys + keys_total;
    uint32_t *dPred = dHist + (size_t)kBins * n;
    uint32_t *dPrad = dPred + (size_t)n * kPredStride;
    SJBG_CK(h, cudaMemsetAsync(dHist, 0, histB + 2 * predB, h->stream));
    SJBG_CK(h, cudaMemsetAsync(dTab, 0, tabB, h->stream));
    const SampleWin *dSw = reinterpret_cast<const SampleWin *>(dsmall);
    SampleScratch *dScr = reinterpret_cast<SampleScratch *>(dsmall + swB);

    // one pass of four loads per thread: all of a window's sample in flight at once
    const uint32_t bs = std::max<uint32_t>(1, std::min<uint32_t>(256, (max_m + 1023) / 1024));
    SJBG_CK(h, launch(h, "learned_sample", sample_minmax_kernel, dim3(bs, n), dim3(kSampleThreads), 0, dL, dR, dSw,
                      dScr, dKeys));
    // one chunk per CTA, unless the CTAs of all windows would take more than
    // one wave: then each CTA takes several chunks in turn (a second wave
    // costs a whole CTA's latency, a second chunk less)
    int count_per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&count_per_sm, sample_count_kernel, kSampleThreads, 0) != cudaSuccess) {
        cudaGetLastError();
        count_per_sm = 1;
    }
    const uint32_t wave = (uint32_t)std::max(count_per_sm, 1) * (uint32_t)std::max(h->num_sms, 1);
    const uint32_t bn = std::max<uint32_t>(1, std::min<uint32_t>({256u, (max_m + kCountChunk - 1) / kCountChunk,
                                                                  std::max<uint32_t>(1, wave / std::max<uint32_t>(n, 1))}));
    SJBG_CK(h, launch(h, "learned_count", sample_count_kernel, dim3(bn, n), dim3(kSampleThreads), 0,
                      (const uint32_t *)dKeys, dSw, dScr, dHist, dTab, dLists));
    const uint32_t tx = std::max<uint32_t>(1, std::min<uint32_t>(16, (max_list + 4095) / 4096));
    SJBG_CK(h, launch(h, "learned_heavy", heavy_candidates_kernel, dim3(tx, n), dim3(kSampleThreads), 0, dSw,
                      (const unsigned long long *)dTab, dScr, (const uint32_t *)dLists, dCand));
    allow_big_smem(learned_fit_kernel, sizeof(uint32_t) * kBins);
    SJBG_CK(h, launch(h, "learned_fit", learned_fit_kernel, dim3(n), dim3(1024), sizeof(uint32_t) * kBins, dSw, dScr,
                      dHist, dCand, dM, leaves, allow_heavy ? kMaxHeavy : 0u, bound));
    const uint32_t bc = std::max<uint32_t>(1, std::min<uint32_t>(64, (max_m + 4095) / 4096));
    SJBG_CK(h, launch(h, "learned_check", learned_check_kernel, dim3(bc, n), dim3(kSampleThreads), 0,
                      (const uint32_t *)dKeys, dSw, (const LearnedModel *)dM, dPred, dPrad));
    SJBG_CK(h, launch(h, "learned_overflow", learned_overflow_kernel, dim3(n), dim3(1024), 0, dSw, dM,
                      (const uint32_t *)dPred, (const uint32_t *)dPrad, bound, dPlan));
    *dModels = dM;
    return SJBG_OK;
}

}  // namespace sjbg
