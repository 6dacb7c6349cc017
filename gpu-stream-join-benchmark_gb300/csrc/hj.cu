// hj.cu - lazy hash join (sm_103a).
//
// Replaces the reference's lazy GPU hash-join family
// (src/sjb/windowing/lazy/executor/GPU/GPU_HJ.cu:9-309 and its NoOutput /
// CountKernel / EstimatedSelectivity / Atomic variants), whose matching rule
// is the lazy CPU_HJ's (src/sjb/windowing/lazy/executor/CPU/CPU_HJ.cpp:30-136):
// every left tuple joins every right tuple of the window with an equal key.
//
// Design (many windows per call, one launch per pass):
//   1. part_hist     per 4096-tuple tile: bucket of each tuple -> shared histogram
//                    -> one atomicAdd per non-empty bucket into the global counts.
//   2. part_scan     per window, exclusive scan of its counts on both sides ->
//                    bucket starts; buckets with tuples on both sides form the
//                    join list (item records), the only buckets step 4 visits.
//   3. part_scatter  per tile: local counting sort by bucket in shared memory,
//                    one atomicAdd per bucket to reserve a range, then the tile
//                    is written as contiguous per-bucket runs of (key,val) words
//                    (windows of many buckets: a coarse pass inside part_hist,
//                    then part_fine).
//   4. bucket_join   per join item (persistent CTAs, one item ahead): a radix
//                    window's bucket through a direct table indexed by
//                    key >> radix bits when its indices allow it, else an
//                    open-addressing table in shared memory from the left run,
//                    probed with the right run.
//        count mode: table slot = {key, count, sum fr(val)}, updated with
//                    32-bit shared atomics (the sum as two words with carry);
//                    keys that do not fit go back into the left run (compacted
//                    in place) and are joined in a further pass, so any bucket,
//                    however skewed, finishes.
//        enum mode:  table slot = {key, chain head}, chains over a staged chunk
//                    of left vals; every pair is visited for the xor checksum
//                    and, when asked, written with one atomic per warp.
// The bucket of a key is its low radix bits (plain radix partitioning) or the
// learned partitioner's prediction (learned.cu).
#include <algorithm>
#include <cstring>
#include <type_traits>
#include <vector>

#include "learned.cuh"
#include "runtime.h"

namespace sjbg {

constexpr int kTile = 4096;          // tuples per partitioning tile
constexpr uint32_t kHistTiles = 16;  // tiles per counting CTA at least (amortises its set-up)
constexpr int kPartThreads = 512;
constexpr int kJoinThreads = 512;
constexpr uint32_t kMaxBucketsLog2 = 14;
// Two-level partitioning: a window of 2^lg buckets is split into 2^ceil(lg/2)
// coarse partitions of 2^floor(lg/2) fine buckets each (at most 128 of each).
constexpr uint32_t kCoarseMax = 128;
constexpr uint32_t kRow = kCoarseMax + 1;   // per tile: exclusive coarse offsets, then its total
constexpr uint32_t kGroupTiles = 64;        // tiles whose runs of one coarse partition a fine CTA gathers
constexpr uint32_t kFineChunk = 2048;       // tuples a fine CTA sorts at a time
constexpr int kFineThreads = 256;

__host__ __device__ __forceinline__ uint32_t coarse_bits(uint32_t lg) { return (lg + 1) / 2; }
// Windows of at least this many buckets are partitioned in two passes: with
// fewer, a 4,096-tuple tile still writes runs of several tuples per bucket.
constexpr uint32_t kTwoLevelMinLog2 = 11;
// Heavy keys whose counting-pass accumulators are replicated per lane.
constexpr uint32_t kHotHeavy = 32;

__device__ __forceinline__ uint32_t find_window(const uint32_t *prefix, uint32_t n, uint32_t t) {
    // largest w with prefix[w] <= t  (prefix has n+1 entries, prefix[0] = 0)
    uint32_t lo = 0, hi = n;  // answer in [lo, hi)
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (prefix[mid] <= t) lo = mid; else hi = mid;
    }
    return lo;
}

// Partitioning model of the CTA's window: learned (when it has a model that
// did not fall back) or plain radix on the key's low bits.
// The CTA's copy of the model lives in shared memory (`core`).
struct Classifier {
    const LearnedCore *m;   // null: radix
    uint32_t mask;
    __device__ __forceinline__ uint32_t bucket(uint32_t key) const {
        return m ? learned_bucket(*m, key) : (key & mask);
    }
};

// The window's model in global memory, or null for radix partitioning.
__device__ __forceinline__ const LearnedModel *model_of(const WinPlan &wp, const LearnedModel *models) {
    return (wp.model != 0xFFFFFFFFu && !models[wp.model].fallback) ? &models[wp.model] : nullptr;
}

// All threads of the CTA; ends with a barrier when the window has a model.
__device__ __forceinline__ Classifier make_classifier(const WinPlan &wp, const LearnedModel *gm, LearnedCore &core) {
    Classifier c;
    c.m = nullptr;
    c.mask = (1u << wp.log2_buckets) - 1u;
    if (gm) {
        copy_to_smem(&core, gm, sizeof(LearnedCore));
        c.m = &core;
    }
    return c;
}

// ------------------------------------------------------------------ 1. histogram
// Also aggregates heavy keys of learned windows: per heavy key, count and
// sum of fr (left) / gs (right); heavy tuples are not partitioned.
__global__ void __launch_bounds__(kPartThreads, 2)
part_hist_kernel(const sjbg_tuple *__restrict__ L, const sjbg_tuple *__restrict__ R, const WinPlan *__restrict__ wins,
                 uint32_t nwin, const uint32_t *__restrict__ tileL, const uint32_t *__restrict__ tileR,
                 const uint32_t *__restrict__ hgroupL, const uint32_t *__restrict__ hgroupR,
                 uint32_t *__restrict__ cnt, uint32_t B, const LearnedModel *__restrict__ models,
                 HeavyAcc *__restrict__ hacc, uint64_t *__restrict__ compL, uint64_t *__restrict__ compR,
                 uint32_t *__restrict__ ccnt, uint32_t *__restrict__ rows) {
    extern __shared__ __align__(16) uint32_t hist[];   // P counters, then (coarse output) the tile stage
    __shared__ HeavySet hs;
    // heavy-key sums as two 32-bit words: native 32-bit shared atomics, with
    // the low word's carry (seen in its returned old value) added to the high
    // word.  The kHotHeavy heaviest keys (ids 0 .. kHotHeavy-1, heaviest first)
    // have one copy per lane after the kMaxHeavy shared ones: copy kMaxHeavy +
    // 32 * id + lane sits in the lane's own bank, so the many lanes of a warp
    // that hold the same hot key update it without bank conflicts.
    constexpr uint32_t kHeavySlotsAcc = kMaxHeavy + 32 * kHotHeavy;
    __shared__ uint32_t hcnt[kHeavySlotsAcc], hsum_lo[kHeavySlotsAcc], hsum_hi[kHeavySlotsAcc];
    // this CTA covers an equal share of one window side's tiles: the side has
    // hgroup[w + 1] - hgroup[w] counting CTAs ("hist groups")
    const bool right = blockIdx.x >= hgroupL[nwin];
    const uint32_t g = right ? blockIdx.x - hgroupL[nwin] : blockIdx.x;
    const uint32_t *hp = right ? hgroupR : hgroupL;
    const uint32_t *tp = right ? tileR : tileL;
    const uint32_t w = find_window(hp, nwin, g);
    const WinPlan wp = wins[w];
    __shared__ LearnedCore core;
    const LearnedModel *gm = model_of(wp, models);
    const Classifier cls = make_classifier(wp, gm, core);
    const bool heavy = cls.m && cls.m->n_heavy;
    const bool compact = heavy && cls.m->compact;
    // compact arrays: window w's side starts at its first tile * kTile
    uint64_t *cdst = compact ? (right ? compR : compL) + (uint64_t)tp[w] * kTile : nullptr;
    // coarse output (every window that is not compacted, when rows is given):
    // each tile's light tuples, sorted by coarse partition, go to the same
    // tile-sized region of the output; the tile's row holds the coarse offsets
    const bool coarse = rows != nullptr && !compact && wp.two_level;
    const uint32_t lgC = coarse_bits(wp.log2_buckets), cshift = wp.log2_buckets - lgC, ncoarse = 1u << lgC;
    __shared__ uint32_t ccnt_s[kCoarseMax], cpre_s[kCoarseMax + 1];
    uint64_t *stage = reinterpret_cast<uint64_t *>(hist + ((1u << wp.log2_buckets) + 1) / 2 * 2);
    uint64_t *coarse_out = coarse ? (right ? compR : compL) + (uint64_t)tp[w] * kTile : nullptr;
    uint32_t *rows_side = coarse ? rows + (right ? tileL[nwin] : 0) * kRow : nullptr;
    if (coarse)
        for (uint32_t i = threadIdx.x; i < ncoarse; i += blockDim.x) ccnt_s[i] = 0;
    const uint64_t nside = right ? wp.n_right : wp.n_left;
    const uint32_t side_tiles = tp[w + 1] - tp[w], ncta = hp[w + 1] - hp[w], j = g - hp[w];
    const uint32_t t_first = (uint32_t)((uint64_t)j * side_tiles / ncta);   // tile indices inside the window side
    const uint32_t t_end = (uint32_t)((uint64_t)(j + 1) * side_tiles / ncta);
    // counters of the buckets in use: the model's own fan-out when there is one
    const uint32_t P = 1u << (cls.m ? cls.m->log2_buckets : wp.log2_buckets);
    for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) hist[i] = 0;
    if (heavy) {
        for (uint32_t i = threadIdx.x; i < kHeavySlotsAcc; i += blockDim.x) { hcnt[i] = 0; hsum_lo[i] = 0; hsum_hi[i] = 0; }
        heavy_set_load(hs, gm);   // ends with a barrier
    }
    SJBG_BARRIER();
    // heavy keys are summed with shared atomics only: measured, that beats
    // keeping the hottest keys' sums in registers (fewer instructions per tuple
    // outweigh the atomics' serialisation on the hottest keys)
    constexpr int kPer = kTile / kPartThreads;
    const sjbg_tuple *base = right ? R + wp.right_off : L + wp.left_off;
    // key and val of the thread's tuples of tile tt (the sectors read are those
    // of whole tuples, the registers half)
    auto load_tile = [&](uint32_t tt, uint2 (&v)[kPer]) {
        const uint64_t start = (uint64_t)tt * kTile;
        const uint32_t n = (uint32_t)(nside - start < (uint64_t)kTile ? nside - start : (uint64_t)kTile);
        const uint2 *src = reinterpret_cast<const uint2 *>(base + start);
#pragma unroll
        for (int k = 0; k < kPer; k++) {
            const uint32_t i = threadIdx.x + k * kPartThreads;
            v[k] = i < n ? __ldg(src + 2 * i) : make_uint2(0u, 0u);
        }
    };
    // compacted windows: each warp buffers its light tuples in its share of the
    // stage (which only coarse output uses otherwise); wn is warp-uniform
    constexpr uint32_t kWarpBuf = kTile / (kPartThreads / 32);   // a warp's tile fits an empty buffer
    uint64_t *wbuf = stage + warp_id() * kWarpBuf;
    uint32_t wn = 0;
    auto flush_light = [&]() {
        uint32_t base = 0;
        if (lane_id() == 0) base = atomicAdd(&ccnt[2 * w + (right ? 1 : 0)], wn);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        __syncwarp();   // the buffer's writes are visible to every lane
        for (uint32_t j = lane_id(); j < wn; j += 32) cdst[base + j] = wbuf[j];
        __syncwarp();   // read before it is refilled
        wn = 0;
    };
    // The counting loop, compiled once per kind of window (heavy keys, compacted
    // light tuples, coarse output, learned or radix buckets), so that none of
    // the mode tests runs per tuple.
    auto count_tiles = [&](auto heavy_t, auto compact_t, auto coarse_t, auto learned_t) {
        constexpr bool kHeavy = decltype(heavy_t)::value, kCompact = decltype(compact_t)::value;
        constexpr bool kCoarse = decltype(coarse_t)::value, kLearned = decltype(learned_t)::value;
        auto bucket_of = [&](uint32_t key) -> uint32_t {
            if constexpr (kLearned) return learned_bucket(*cls.m, key);
            else return key & cls.mask;
        };
        // software pipeline: tile tt+1 is in flight while tile tt is counted
        uint2 nv[kPer];
        if (t_first < t_end) load_tile(t_first, nv);
        for (uint32_t tt = t_first; tt < t_end; tt++) {
            const uint64_t start = (uint64_t)tt * kTile;
            const uint32_t n = (uint32_t)(nside - start < (uint64_t)kTile ? nside - start : (uint64_t)kTile);
            uint2 v[kPer];
#pragma unroll
            for (int k = 0; k < kPer; k++) v[k] = nv[k];
            if (tt + 1 < t_end) load_tile(tt + 1, nv);
            uint32_t lightmask = 0;
            uint32_t pk[kPer];   // coarse output: coarse << 16 | rank inside the tile's coarse run, or ~0u
            // the tuples of a tile, compiled apart for full tiles (no bounds test)
            auto count_tuples = [&](auto full_t) {
            constexpr bool kFull = decltype(full_t)::value;
#pragma unroll
            for (int k = 0; k < kPer; k++) {
                const uint32_t i = threadIdx.x + k * kPartThreads;
                const bool valid = kFull || i < n;
                const uint32_t key = v[k].x, val = v[k].y;
                pk[k] = 0xFFFFFFFFu;
                if constexpr (kHeavy) {
                    const uint32_t hid = valid ? heavy_find(hs, key) : kHeavyBucket;
                    if (hid != kHeavyBucket) {
                        const unsigned long long f = sjbg_fside(val, right ? 1u : 0u);   // one mix, either side
                        const uint32_t a = hid < kHotHeavy ? kMaxHeavy + 32u * hid + lane_id() : hid;
                        atomicAdd(&hcnt[a], 1u);
                        const uint32_t flo = (uint32_t)f;
                        const uint32_t old = atomicAdd(&hsum_lo[a], flo);
                        atomicAdd(&hsum_hi[a], add_carry((uint32_t)(f >> 32), old, flo));
                    } else if (valid) {
                        // light keys: compacted windows count them in part_hist_light
                        if constexpr (kCompact) {
                            lightmask |= 1u << k;
                        } else {
                            const uint32_t b = bucket_of(key);
                            atomicAdd(&hist[b], 1u);
                            if constexpr (kCoarse) pk[k] = ((b >> cshift) << 16) | atomicAdd(&ccnt_s[b >> cshift], 1u);
                        }
                    }
                } else {
                    // plain partitioning: one shared atomic per tuple (measured faster
                    // than combining a warp's equal buckets first, skewed keys included)
                    const uint32_t b = valid ? bucket_of(key) : 0u;
                    if (valid) atomicAdd(&hist[b], 1u);
                    if constexpr (kCoarse)
                        if (valid) pk[k] = ((b >> cshift) << 16) | atomicAdd(&ccnt_s[b >> cshift], 1u);
                }
            }
            };
            if (n == (uint32_t)kTile) count_tuples(std::true_type{});
            else count_tuples(std::false_type{});
            if constexpr (kCoarse) {
                SJBG_BARRIER();   // every rank of the tile is assigned
                uint32_t *row = rows_side + (uint64_t)(tp[w] + tt) * kRow;
                if (warp_id() == 0) {
                    // exclusive offsets of the (at most 128) coarse runs; counters reset for the next tile
                    uint32_t a[kCoarseMax / 32], sum = 0;
#pragma unroll
                    for (int q = 0; q < (int)(kCoarseMax / 32); q++) {
                        const uint32_t c = lane_id() * (kCoarseMax / 32) + q;
                        a[q] = c < ncoarse ? ccnt_s[c] : 0u;
                        sum += a[q];
                    }
                    uint32_t tot;
                    uint32_t run = warp_excl_scan(sum, &tot);
#pragma unroll
                    for (int q = 0; q < (int)(kCoarseMax / 32); q++) {
                        const uint32_t c = lane_id() * (kCoarseMax / 32) + q;
                        if (c < ncoarse) {
                            cpre_s[c] = run;
                            row[c] = run;
                            ccnt_s[c] = 0;
                        }
                        run += a[q];
                    }
                    if (lane_id() == 0) {
                        cpre_s[ncoarse] = tot;
                        row[ncoarse] = tot;
                    }
                }
                SJBG_BARRIER();
#pragma unroll
                for (int k = 0; k < kPer; k++)
                    if (pk[k] != 0xFFFFFFFFu)
                        stage[cpre_s[pk[k] >> 16] + (pk[k] & 0xFFFFu)] = ((uint64_t)v[k].y << 32) | v[k].x;
                SJBG_BARRIER();
                // the tile's light tuples, contiguous per coarse run, written out whole
                const uint32_t nl = cpre_s[ncoarse];
                uint64_t *dst = coarse_out + (uint64_t)tt * kTile;
                for (uint32_t i = threadIdx.x; i < nl; i += blockDim.x) dst[i] = stage[i];
            }
            if constexpr (kCompact) {
                // the tile's light tuples go to the warp's buffer as (key,val) words
                // (warp scan, no block barrier); a full buffer is written out to the
                // window side's compact array with one global reservation
                const uint32_t nl = __popc(lightmask);
                uint32_t wt;
                const uint32_t ex = warp_excl_scan(nl, &wt);
                if (wn + wt > kWarpBuf) flush_light();
                uint32_t pos = wn + ex;
#pragma unroll
                for (int k = 0; k < kPer; k++)
                    if ((lightmask >> k) & 1u) wbuf[pos++] = ((uint64_t)v[k].y << 32) | v[k].x;
                wn += wt;
            }
        }
        if constexpr (kCompact)
            if (wn) flush_light();
    };
    using T = std::true_type;
    using F = std::false_type;
    if (compact) count_tiles(T{}, T{}, F{}, T{});
    else if (heavy && coarse) count_tiles(T{}, F{}, T{}, T{});
    else if (heavy) count_tiles(T{}, F{}, F{}, T{});
    else if (cls.m && coarse) count_tiles(F{}, F{}, T{}, T{});
    else if (cls.m) count_tiles(F{}, F{}, F{}, T{});
    else if (coarse) count_tiles(F{}, F{}, T{}, F{});
    else count_tiles(F{}, F{}, F{}, F{});
    SJBG_BARRIER();
    uint32_t *dst = cnt + (right ? B : 0) + wp.bucket_base;
    for (uint32_t i = threadIdx.x; i < P; i += blockDim.x)
        if (hist[i]) atomicAdd(&dst[i], hist[i]);
    if (heavy) {
        // fold the hot keys' per-lane copies into their shared slots: warp q sums key q's
        for (uint32_t q = warp_id(); q < kHotHeavy; q += blockDim.x >> 5) {
            const uint32_t a = kMaxHeavy + 32u * q + lane_id();
            uint32_t c = hcnt[a];
            unsigned long long sm = ((unsigned long long)hsum_hi[a] << 32) | hsum_lo[a];
            sm = warp_sum_u64(sm);
            for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xFFFFFFFFu, c, o);
            if (lane_id() == 0) {
                // slot q itself is never updated by the counting loop
                hcnt[q] = c;
                hsum_lo[q] = (uint32_t)sm;
                hsum_hi[q] = (uint32_t)(sm >> 32);
            }
        }
        SJBG_BARRIER();
        HeavyAcc *ha = hacc + (uint64_t)w * kMaxHeavy;
        for (uint32_t i = threadIdx.x; i < cls.m->n_heavy; i += blockDim.x) {
            if (!hcnt[i]) continue;
            const unsigned long long sm = ((unsigned long long)hsum_hi[i] << 32) | hsum_lo[i];
            if (right) {
                atomicAdd(&ha[i].cnt_r, (unsigned long long)hcnt[i]);
                atomicAdd(&ha[i].sum_r, sm);
            } else {
                atomicAdd(&ha[i].cnt_l, (unsigned long long)hcnt[i]);
                atomicAdd(&ha[i].sum_l, sm);
            }
        }
    }
}

// Bucket counts of the compacted light tuples of compacted learned windows
// (part_hist only wrote them out).  Persistent CTAs stride over the tiles of
// all window sides; tiles past a side's compacted count are skipped.
// Per window side, the tiles (or fine items) that each later pass has work
// for, as exclusive prefixes over the windows, written once the counting pass
// is done: kind 0 part_hist_light (the compacted windows' light tiles), kind 1
// part_scatter (those, plus every tile of a single-level window that was not
// compacted), kind 2 part_fine (two-level windows that were not compacted).
// Array 2 * kind + side (left 0, right 1) of n + 1 entries.  One warp per array.
enum : uint32_t { kWorkLight = 0, kWorkScatter = 1, kWorkFine = 2 };
__global__ void part_work_kernel(const WinPlan *__restrict__ wins, uint32_t nwin, const uint32_t *__restrict__ tileL,
                                 const uint32_t *__restrict__ tileR, const uint32_t *__restrict__ itemL,
                                 const uint32_t *__restrict__ itemR, const LearnedModel *__restrict__ models,
                                 const uint32_t *__restrict__ ccnt, uint32_t *__restrict__ work) {
    const uint32_t a = warp_id();
    if (a >= 6) return;   // whole warp
    const uint32_t kind = a >> 1, right = a & 1u;
    const uint32_t *tp = right ? tileR : tileL, *ip = right ? itemR : itemL;
    uint32_t *out = work + a * (nwin + 1);
    uint32_t carry = 0;
    for (uint32_t base = 0; base < nwin; base += 32) {
        const uint32_t w = base + lane_id();
        uint32_t c = 0;
        if (w < nwin) {
            const WinPlan wp = wins[w];
            const LearnedModel *gm = model_of(wp, models);
            const bool compact = gm && gm->n_heavy && gm->compact;
            const uint32_t light = (ccnt[2 * w + right] + kTile - 1) / kTile;
            if (kind == kWorkLight) c = compact ? light : 0u;
            else if (kind == kWorkScatter) c = compact ? light : (wp.two_level ? 0u : tp[w + 1] - tp[w]);
            else c = (wp.two_level && !compact) ? ip[w + 1] - ip[w] : 0u;
        }
        uint32_t tot;
        const uint32_t ex = warp_excl_scan(c, &tot);
        if (w < nwin) out[w] = carry + ex;
        carry += tot;
    }
    if (lane_id() == 0) out[nwin] = carry;
}

// Work item t of a persistent pass over prefix arrays pl (left) / pr (right):
// its window side and the index of the item inside the window side.
struct WorkItem {
    uint32_t w, local;
    bool right;
};
__device__ __forceinline__ WorkItem work_item(const uint32_t *pl, const uint32_t *pr, uint32_t nwin, uint32_t t) {
    WorkItem it;
    it.right = t >= pl[nwin];
    const uint32_t *p = it.right ? pr : pl;
    const uint32_t x = it.right ? t - pl[nwin] : t;
    it.w = find_window(p, nwin, x);
    it.local = x - p[it.w];
    return it;
}

__global__ void __launch_bounds__(kPartThreads)
part_hist_light_kernel(const WinPlan *__restrict__ wins, uint32_t nwin, const uint32_t *__restrict__ tileL,
                       const uint32_t *__restrict__ tileR, const uint32_t *__restrict__ work,
                       uint32_t *__restrict__ cnt, uint32_t B, const LearnedModel *__restrict__ models,
                       const uint64_t *__restrict__ compL, const uint64_t *__restrict__ compR,
                       const uint32_t *__restrict__ ccnt) {
    extern __shared__ uint32_t hist[];
    __shared__ LearnedCore core;
    const uint32_t *pl = work + 2 * kWorkLight * (nwin + 1), *pr = pl + (nwin + 1);
    const uint32_t items = pl[nwin] + pr[nwin];
    for (uint32_t bt = blockIdx.x; bt < items; bt += gridDim.x) {
        const WorkItem it = work_item(pl, pr, nwin, bt);
        const bool right = it.right;
        const uint32_t w = it.w;
        const uint32_t *tp = right ? tileR : tileL;
        const WinPlan wp = wins[w];
        const LearnedModel *gm = model_of(wp, models);   // a compacted window's model
        const uint64_t nside = ccnt[2 * w + (right ? 1 : 0)];
        const uint64_t start = (uint64_t)it.local * kTile;
        const uint32_t n = (uint32_t)(nside - start < (uint64_t)kTile ? nside - start : (uint64_t)kTile);
        SJBG_BARRIER();   // the previous tile's readers of hist and core are done
        const Classifier cls = make_classifier(wp, gm, core);   // ends with a barrier
        const uint32_t P = 1u << core.log2_buckets;
        for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) hist[i] = 0;
        SJBG_BARRIER();
        const uint64_t *src = (right ? compR : compL) + (uint64_t)tp[w] * kTile + start;
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) atomicAdd(&hist[cls.bucket((uint32_t)__ldg(src + i))], 1u);
        SJBG_BARRIER();
        uint32_t *dst = cnt + (right ? B : 0) + wp.bucket_base;
        for (uint32_t i = threadIdx.x; i < P; i += blockDim.x)
            if (hist[i]) atomicAdd(&dst[i], hist[i]);
    }
}

// Heavy keys' contribution per window: count += |L_k||R_k|, prod += (sum fr)(sum gs).
__global__ void heavy_finish_kernel(const WinPlan *__restrict__ wins, uint32_t nwin,
                                    const LearnedModel *__restrict__ models, const HeavyAcc *__restrict__ hacc,
                                    WinAcc *__restrict__ acc) {
    const uint32_t w = blockIdx.x;
    const WinPlan wp = wins[w];
    if (wp.model == 0xFFFFFFFFu) return;
    if (models[wp.model].fallback) {   // 1: the model overflowed; 2: radix chosen by cost
        if (threadIdx.x == 0) acc[w].info = models[wp.model].fallback == 2u ? kInfoRadixByCost : kInfoFallback;
        return;
    }
    const uint32_t nh = models[wp.model].n_heavy;
    if (threadIdx.x == 0) acc[w].info = kInfoLearned | ((unsigned long long)nh << 32);
    unsigned long long c = 0, p = 0;
    for (uint32_t i = threadIdx.x; i < nh; i += blockDim.x) {
        const HeavyAcc a = hacc[(uint64_t)w * kMaxHeavy + i];
        c += a.cnt_l * a.cnt_r;
        p += a.sum_l * a.sum_r;
    }
    flush_acc(&acc[w], c, 0, p);
}

// ------------------------------------------------------------------ 2. scan
// Single-CTA exclusive scan of the bucket counts -> start and cursor.  The
// left side (counts [0, B)) and the right side (counts [B, 2B)) are scanned
// separately: each side's offsets index its own partitioned array.
__global__ void __launch_bounds__(1024) part_scan_kernel(const uint32_t *__restrict__ cnt, uint32_t *__restrict__ start,
                                                         uint32_t *__restrict__ cursor, uint32_t B) {
    __shared__ uint32_t warp_tot[32];
    __shared__ uint32_t carry_s;
    constexpr uint32_t kItems = 4;
    const uint32_t chunk = blockDim.x * kItems;
    for (uint32_t side = 0; side < 2; side++) {
        const uint32_t lo = side * B, hi = lo + B;
        if (threadIdx.x == 0) carry_s = 0;
        SJBG_BARRIER();
        for (uint32_t base = lo; base < hi; base += chunk) {
            uint32_t v[kItems], s = 0;
#pragma unroll
            for (uint32_t k = 0; k < kItems; k++) {
                const uint32_t i = base + threadIdx.x * kItems + k;
                v[k] = i < hi ? cnt[i] : 0;
                s += v[k];
            }
            uint32_t wt;
            const uint32_t ex = warp_excl_scan(s, &wt);
            if (lane_id() == 31) warp_tot[warp_id()] = ex + s;
            SJBG_BARRIER();
            if (warp_id() == 0) {
                const uint32_t x = lane_id() < (blockDim.x >> 5) ? warp_tot[lane_id()] : 0;
                uint32_t tt;
                warp_tot[lane_id()] = warp_excl_scan(x, &tt);
            }
            SJBG_BARRIER();
            uint32_t run = carry_s + warp_tot[warp_id()] + ex;
#pragma unroll
            for (uint32_t k = 0; k < kItems; k++) {
                const uint32_t i = base + threadIdx.x * kItems + k;
                if (i < hi) {
                    start[i] = run;
                    cursor[i] = run;
                }
                run += v[k];
            }
            SJBG_BARRIER();
            if (threadIdx.x == blockDim.x - 1) carry_s = run;
            SJBG_BARRIER();
        }
    }
}

// One bucket of the join list with what its join reads before the tuples:
// both sides' counts and run starts, the window, the window's radix bits, and
// whether the window is radix-partitioned (its buckets may use a direct table).
struct __align__(16) JoinItem {
    uint32_t b, nR, nS, sR, sS, w, lg, direct;
};
static_assert(sizeof(JoinItem) == 32, "two 16-byte words per join item");

// Per window, one CTA: exclusive scan of the window's bucket counts on each
// side, starting at the window's base in that side's partitioned array (the
// tuples of the windows before it: baseL / baseR), giving the bucket starts
// and scatter cursors; then every bucket with tuples on both sides is appended
// to the join list (items, length *jn: nothing else can match).
__global__ void __launch_bounds__(1024)
part_scan_win_kernel(const WinPlan *__restrict__ wins, const uint32_t *__restrict__ baseL,
                     const uint32_t *__restrict__ baseR, const uint32_t *__restrict__ cnt,
                     uint32_t *__restrict__ start, uint32_t *__restrict__ cursor, uint32_t B,
                     const LearnedModel *__restrict__ models, JoinItem *__restrict__ items,
                     uint32_t *__restrict__ jn) {
    __shared__ uint32_t warp_tot[32];
    __shared__ uint32_t carry_s;
    const uint32_t w = blockIdx.x;
    const WinPlan wp = wins[w];
    const uint32_t P = 1u << wp.log2_buckets, b0 = wp.bucket_base;
    constexpr uint32_t kItems = 4;
    const uint32_t chunk = blockDim.x * kItems;
    for (uint32_t side = 0; side < 2; side++) {
        const uint32_t lo = side * B + b0, hi = lo + P;
        if (threadIdx.x == 0) carry_s = side ? baseR[w] : baseL[w];
        SJBG_BARRIER();
        for (uint32_t base = lo; base < hi; base += chunk) {
            uint32_t v[kItems], s = 0;
#pragma unroll
            for (uint32_t k = 0; k < kItems; k++) {
                const uint32_t i = base + threadIdx.x * kItems + k;
                v[k] = i < hi ? cnt[i] : 0;
                s += v[k];
            }
            uint32_t wt;
            const uint32_t ex = warp_excl_scan(s, &wt);
            if (lane_id() == 31) warp_tot[warp_id()] = ex + s;
            SJBG_BARRIER();
            if (warp_id() == 0) {
                const uint32_t x = lane_id() < (blockDim.x >> 5) ? warp_tot[lane_id()] : 0;
                uint32_t tt;
                warp_tot[lane_id()] = warp_excl_scan(x, &tt);
            }
            SJBG_BARRIER();
            uint32_t run = carry_s + warp_tot[warp_id()] + ex;
#pragma unroll
            for (uint32_t k = 0; k < kItems; k++) {
                const uint32_t i = base + threadIdx.x * kItems + k;
                if (i < hi) {
                    start[i] = run;
                    cursor[i] = run;
                }
                run += v[k];
            }
            SJBG_BARRIER();
            if (threadIdx.x == blockDim.x - 1) carry_s = run;
            SJBG_BARRIER();
        }
    }
    // join list: one reservation per warp of joinable buckets (the starts were
    // written by this CTA, before the scan's last barrier)
    const uint32_t direct = (models ? model_of(wp, models) : nullptr) == nullptr ? 1u : 0u;
    for (uint32_t i0 = 0; i0 < P; i0 += blockDim.x) {
        const uint32_t i = i0 + threadIdx.x, b = b0 + i;
        const uint32_t nR = i < P ? cnt[b] : 0u, nS = i < P ? cnt[B + b] : 0u;
        const bool ok = nR != 0u && nS != 0u;
        const unsigned m = __ballot_sync(0xFFFFFFFFu, ok);
        uint32_t wbase = 0;
        if (lane_id() == 0 && m) wbase = atomicAdd(jn, (uint32_t)__popc(m));
        wbase = __shfl_sync(0xFFFFFFFFu, wbase, 0);
        if (ok) {
            JoinItem ji;
            ji.b = b; ji.nR = nR; ji.nS = nS; ji.sR = start[b]; ji.sS = start[B + b];
            ji.w = w; ji.lg = wp.log2_buckets; ji.direct = direct;
            items[wbase + __popc(m & ((1u << lane_id()) - 1u))] = ji;
        }
    }
}

// Block-wide exclusive scan of P (<= 16384) shared counters in place.
__device__ void block_scan_smem(uint32_t *a, uint32_t P, uint32_t *warp_tot) {
    const uint32_t per = (P + blockDim.x - 1) / blockDim.x;
    const uint32_t b0 = min(P, threadIdx.x * per), b1 = min(P, b0 + per);
    uint32_t s = 0;
    for (uint32_t i = b0; i < b1; i++) s += a[i];
    uint32_t tot;
    uint32_t ex = warp_excl_scan(s, &tot);
    if (lane_id() == 31) warp_tot[warp_id()] = ex + s;
    SJBG_BARRIER();
    if (warp_id() == 0) {
        uint32_t x = lane_id() < (blockDim.x >> 5) ? warp_tot[lane_id()] : 0, tt;
        warp_tot[lane_id()] = warp_excl_scan(x, &tt);
    }
    SJBG_BARRIER();
    uint32_t run = warp_tot[warp_id()] + ex;
    for (uint32_t i = b0; i < b1; i++) {
        uint32_t c = a[i];
        a[i] = run;
        run += c;
    }
    SJBG_BARRIER();
}

// ------------------------------------------------------------------ 3. scatter
constexpr int kScatterPer = kTile / kPartThreads;   // tuples per thread per tile

// Where a scatter work item's tuples are: the window side's tuples, or (a
// compacted window) the light tuples the counting pass packed as 8-byte words.
struct TileIn {
    const void *p;
    uint32_t n;        // tuples in the tile
    uint32_t packed;   // 8-byte (key, val) words rather than 16-byte tuples
};

__device__ __forceinline__ TileIn tile_input(const WorkItem it, const sjbg_tuple *__restrict__ L,
                                             const sjbg_tuple *__restrict__ R, const WinPlan *__restrict__ wins,
                                             const uint32_t *__restrict__ tileL, const uint32_t *__restrict__ tileR,
                                             const LearnedModel *__restrict__ models,
                                             const uint64_t *__restrict__ compL, const uint64_t *__restrict__ compR,
                                             const uint32_t *__restrict__ ccnt) {
    const bool right = it.right;
    const uint32_t w = it.w;
    const WinPlan &wp = wins[w];
    const LearnedModel *gm = model_of(wp, models);
    const bool compact = gm && gm->n_heavy && gm->compact;
    const uint64_t nside = compact ? ccnt[2 * w + (right ? 1 : 0)] : (right ? wp.n_right : wp.n_left);
    const uint64_t start = (uint64_t)it.local * kTile;
    TileIn t;
    t.n = (uint32_t)(nside - start < (uint64_t)kTile ? nside - start : (uint64_t)kTile);
    t.packed = compact ? 1u : 0u;
    if (compact)
        t.p = (right ? compR : compL) + (uint64_t)(right ? tileR : tileL)[w] * kTile + start;
    else
        t.p = (right ? R + wp.right_off : L + wp.left_off) + start;
    return t;
}

// The thread's tuples of a tile as (val << 32 | key) words, every load in flight before any use.
__device__ __forceinline__ void tile_load(const TileIn &t, uint64_t (&e)[kScatterPer]) {
#pragma unroll
    for (int k = 0; k < kScatterPer; k++) {
        const uint32_t i = threadIdx.x + k * kPartThreads;
        if (i < t.n) {
            if (t.packed) {
                e[k] = __ldg(static_cast<const uint64_t *>(t.p) + i);
            } else {
                const uint2 v = __ldg(reinterpret_cast<const uint2 *>(static_cast<const sjbg_tuple *>(t.p) + i));
                e[k] = ((uint64_t)v.y << 32) | v.x;   // key and val only
            }
        }
    }
}

// One tile whose tuples are already in e[]: local counting sort by bucket in
// shared memory, one global reservation per non-empty bucket, contiguous
// per-bucket runs written out.  As soon as the tile is staged in shared memory
// e[] is free, so the next tile's loads (next, when given) are issued into it
// before this tile's write-out: they are in flight while it runs.
__device__ __forceinline__ void scatter_tile(const WorkItem it, const TileIn in, uint64_t (&e)[kScatterPer],
                                             const TileIn *next, const WinPlan *__restrict__ wins,
                                             uint32_t *__restrict__ cursor, uint32_t B, uint64_t *__restrict__ outL,
                                             uint64_t *__restrict__ outR, const LearnedModel *__restrict__ models) {
    extern __shared__ __align__(16) uint8_t smem_raw[];
    __shared__ uint32_t warp_tot[32];
    const bool right = it.right;
    const WinPlan wp = wins[it.w];
    const LearnedModel *gm = model_of(wp, models);
    const bool compact = in.packed != 0;
    const uint32_t n = in.n;
    // a model buckets into its own (often smaller) fan-out: only those counters are touched
    const uint32_t P = 1u << (gm ? gm->log2_buckets : wp.log2_buckets);

    uint64_t *stage = reinterpret_cast<uint64_t *>(smem_raw);                  // kTile
    uint16_t *sb = reinterpret_cast<uint16_t *>(stage + kTile);                // kTile bucket ids
    uint32_t *lcnt = reinterpret_cast<uint32_t *>(sb + kTile);                 // P
    uint32_t *gbase = lcnt + P;                                                // P
    __shared__ LearnedCore core;
    const Classifier cls = make_classifier(wp, gm, core);
    const bool heavy = cls.m && cls.m->n_heavy && !compact;
    __shared__ HeavySet hs;
    __shared__ uint32_t kept_s;

    for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) lcnt[i] = 0;
    if (threadIdx.x == 0) kept_s = 0;
    if (heavy) heavy_set_load(hs, gm);
    SJBG_BARRIER();
    uint32_t bk[kScatterPer], rk[kScatterPer];
#pragma unroll
    for (int k = 0; k < kScatterPer; k++) {
        const uint32_t i = threadIdx.x + k * kPartThreads;
        bk[k] = kHeavyBucket;
        if (i < n) {
            const uint32_t key = (uint32_t)e[k];
            if (!heavy || heavy_find(hs, key) == kHeavyBucket) {
                bk[k] = cls.bucket(key);
                rk[k] = atomicAdd(&lcnt[bk[k]], 1u);
            }
        }
    }
    SJBG_BARRIER();
    // the next tile into L2 (its address is known by now), so that the register
    // loads issued once this tile is staged find it there
    if (next && threadIdx.x == 0) l2_prefetch_bulk(next->p, (size_t)next->n * (next->packed ? 8u : 16u));
    // reserve one global range per non-empty bucket
    uint32_t *gcur = cursor + (right ? B : 0) + wp.bucket_base;
    uint32_t kept = 0;
    for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
        const uint32_t c = lcnt[i];
        gbase[i] = c ? atomicAdd(&gcur[i], c) : 0;
        kept += c;
    }
    if (heavy) atomicAdd(&kept_s, kept);
    block_scan_smem(lcnt, P, warp_tot);   // lcnt -> local offsets (ends with a barrier)
    const uint32_t nk = heavy ? kept_s : n;
#pragma unroll
    for (int k = 0; k < kScatterPer; k++) {
        if (bk[k] != kHeavyBucket) {
            const uint32_t pos = lcnt[bk[k]] + rk[k];
            stage[pos] = e[k];
            sb[pos] = (uint16_t)bk[k];
        }
    }
    if (next) tile_load(*next, e);
    SJBG_BARRIER();
    uint64_t *out = right ? outR : outL;
    for (uint32_t j = threadIdx.x; j < nk; j += blockDim.x) {
        const uint32_t b = sb[j];
        out[gbase[b] + (j - lcnt[b])] = stage[j];
    }
}

// scatter_tile for a radix window (no model, no heavy keys, not compacted):
// a tuple's bucket is key & mask, so the staged word carries it and no bucket
// array is kept; the write-out reads one per-bucket delta (global base minus
// local offset) per tuple.
__device__ __forceinline__ void scatter_tile_radix(const WorkItem it, const TileIn in, uint64_t (&e)[kScatterPer],
                                                   const TileIn *next, const WinPlan *__restrict__ wins,
                                                   uint32_t *__restrict__ cursor, uint32_t B,
                                                   uint64_t *__restrict__ outL, uint64_t *__restrict__ outR) {
    extern __shared__ __align__(16) uint8_t smem_raw[];
    __shared__ uint32_t warp_tot[32];
    const WinPlan wp = wins[it.w];
    const uint32_t mask = (1u << wp.log2_buckets) - 1u, P = mask + 1u;
    const uint32_t n = in.n;
    uint64_t *stage = reinterpret_cast<uint64_t *>(smem_raw);   // kTile
    uint32_t *lcnt = reinterpret_cast<uint32_t *>(stage + kTile);  // P
    uint32_t *delta = lcnt + P;                                  // P
    for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) lcnt[i] = 0;
    SJBG_BARRIER();
    uint32_t rk[kScatterPer];
#pragma unroll
    for (int k = 0; k < kScatterPer; k++)
        if (threadIdx.x + k * kPartThreads < n) rk[k] = atomicAdd(&lcnt[(uint32_t)e[k] & mask], 1u);
    SJBG_BARRIER();
    if (next && threadIdx.x == 0) l2_prefetch_bulk(next->p, (size_t)next->n * (next->packed ? 8u : 16u));
    // reserve one global range per non-empty bucket
    uint32_t *gcur = cursor + (it.right ? B : 0) + wp.bucket_base;
    for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
        const uint32_t c = lcnt[i];
        delta[i] = c ? atomicAdd(&gcur[i], c) : 0;
    }
    block_scan_smem(lcnt, P, warp_tot);   // lcnt -> local offsets (ends with a barrier)
#pragma unroll
    for (int k = 0; k < kScatterPer; k++)
        if (threadIdx.x + k * kPartThreads < n) stage[lcnt[(uint32_t)e[k] & mask] + rk[k]] = e[k];
    for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) delta[i] -= lcnt[i];   // (mod 2^32)
    if (next) tile_load(*next, e);
    SJBG_BARRIER();
    uint64_t *out = it.right ? outR : outL;
    for (uint32_t j = threadIdx.x; j < n; j += blockDim.x) {
        const uint64_t x = stage[j];
        out[delta[(uint32_t)x & mask] + j] = x;
    }
}

// kRadixOnly: no window of the call has a model (compiled without the general path).
template <bool kRadixOnly>
__global__ void __launch_bounds__(kPartThreads, kRadixOnly ? 3 : 2)
part_scatter_kernel(const sjbg_tuple *__restrict__ L, const sjbg_tuple *__restrict__ R, const WinPlan *__restrict__ wins,
                    uint32_t nwin, const uint32_t *__restrict__ tileL, const uint32_t *__restrict__ tileR,
                    const uint32_t *__restrict__ workL, const uint32_t *__restrict__ workR,
                    uint32_t *__restrict__ cursor, uint32_t B, uint64_t *__restrict__ outL, uint64_t *__restrict__ outR,
                    const LearnedModel *__restrict__ models, const uint64_t *__restrict__ compL,
                    const uint64_t *__restrict__ compR, const uint32_t *__restrict__ ccnt) {
    // persistent CTAs over the tiles listed by the work prefixes workL / workR
    // (a compacted window's light tiles; a single-level window's tiles), each
    // tile's loads issued while the previous tile is written out
    const uint32_t items = workL[nwin] + workR[nwin];
    uint32_t bt = blockIdx.x;
    if (bt >= items) return;
    WorkItem it = work_item(workL, workR, nwin, bt);
    TileIn in = tile_input(it, L, R, wins, tileL, tileR, models, compL, compR, ccnt);
    uint64_t e[kScatterPer];
    tile_load(in, e);
    for (; bt < items; bt += gridDim.x) {
        SJBG_BARRIER();   // the previous tile's shared-memory readers are done
        const uint32_t nb = bt + gridDim.x;
        WorkItem nit = it;
        TileIn nin = in;
        if (nb < items) {
            nit = work_item(workL, workR, nwin, nb);
            nin = tile_input(nit, L, R, wins, tileL, tileR, models, compL, compR, ccnt);
        }
        if (kRadixOnly || (!in.packed && !model_of(wins[it.w], models)))
            scatter_tile_radix(it, in, e, nb < items ? &nin : nullptr, wins, cursor, B, outL, outR);
        else
            scatter_tile(it, in, e, nb < items ? &nin : nullptr, wins, cursor, B, outL, outR, models);
        it = nit;
        in = nin;
    }
}


// ------------------------------------------------------------------ 3'. fine pass
// Two-level windows: one work item per (window side, coarse partition c,
// group of kGroupTiles tiles) gathers the tiles' runs of partition c (about
// kTile / 2^lgC tuples each, contiguous) with asynchronous 8-byte copies into
// shared memory, and scatters them into the partition's 2^(lg - lgC) fine
// buckets: a local counting sort of up to kFineChunk tuples, one global
// reservation per fine bucket, then contiguous per-bucket runs - coalesced
// writes however many buckets the window has.  Persistent CTAs take the items
// of the windows that need the pass (part_work's prefixes) in turn.
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)),
                 "l"(gmem)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Up to kFineGather tuples of an item are gathered at once (all of a typical
// item's runs, one memory latency), then sorted in chunks of kFineChunk.
// (Measured: prefetching the next item's runs into L2 from here made the pass
// slower - reading that item's rows held a warp past the gather.)
constexpr uint32_t kFineGather = 2 * kFineChunk;
constexpr size_t kFineSmem = kFineGather * sizeof(uint64_t) + kFineChunk * sizeof(uint8_t);

// An item's coarse partition c and its group of tiles [t0, t0 + G).
struct FineRuns {
    uint32_t c, t0, G;
};
__device__ __forceinline__ FineRuns fine_runs(const WorkItem it, const WinPlan *__restrict__ wins,
                                              const uint32_t *__restrict__ tileL, const uint32_t *__restrict__ tileR) {
    const uint32_t *tp = it.right ? tileR : tileL;
    const uint32_t w = it.w;
    const uint32_t ntw = tp[w + 1] - tp[w];
    const uint32_t ngroups = (ntw + kGroupTiles - 1) / kGroupTiles;
    FineRuns f;
    f.c = it.local / ngroups;
    const uint32_t g = it.local % ngroups;
    f.t0 = g * kGroupTiles;
    f.G = min(kGroupTiles, ntw - f.t0);
    return f;
}

__device__ __forceinline__ void fine_item(const WorkItem it, const WinPlan *__restrict__ wins,
                                          uint32_t nwin, const uint32_t *__restrict__ tileL,
                                          const uint32_t *__restrict__ tileR, uint32_t *__restrict__ cursor, uint32_t B,
                                          uint64_t *__restrict__ outL, uint64_t *__restrict__ outR,
                                          const LearnedModel *__restrict__ models, const uint64_t *__restrict__ srcL,
                                          const uint64_t *__restrict__ srcR, const uint32_t *__restrict__ rows) {
    extern __shared__ __align__(16) uint8_t smem_raw[];
    // kFineGather gathered tuples; a chunk is staged, sorted by fine bucket, in
    // its own part of it (its tuples are in registers by then)
    uint64_t *tmp = reinterpret_cast<uint64_t *>(smem_raw);
    uint8_t *sf = reinterpret_cast<uint8_t *>(tmp + kFineGather);   // kFineChunk fine ids
    __shared__ uint32_t runoff[kGroupTiles], runpre[kGroupTiles + 1];
    __shared__ uint32_t fcnt[kCoarseMax], floc[kCoarseMax], fbase[kCoarseMax];
    __shared__ LearnedCore core;
    const bool right = it.right;
    const uint32_t *tp = right ? tileR : tileL;
    const uint32_t w = it.w;
    const WinPlan wp = wins[w];
    const LearnedModel *gm = model_of(wp, models);   // a two-level window that was not compacted
    const uint32_t lg = wp.log2_buckets, lgC = coarse_bits(lg), cshift = lg - lgC, nfine = 1u << cshift;
    const FineRuns fr_it = fine_runs(it, wins, tileL, tileR);
    const uint32_t c = fr_it.c, t0 = fr_it.t0, G = fr_it.G;
    const Classifier cls = make_classifier(wp, gm, core);   // ends with a barrier when there is a model
    const uint32_t *rows_side = rows + (right ? tileL[nwin] : 0) * kRow;
    if (warp_id() == 0) {
        // the runs of partition c in tiles t0 .. t0 + G, and their prefix
        uint32_t len[2], sum = 0;
#pragma unroll
        for (int q = 0; q < 2; q++) {
            const uint32_t i = lane_id() * 2 + q;
            len[q] = 0;
            if (i < G) {
                const uint32_t *row = rows_side + (uint64_t)(tp[w] + t0 + i) * kRow;
                const uint32_t off = row[c];
                len[q] = row[c + 1] - off;
                runoff[i] = (t0 + i) * kTile + off;
            }
            sum += len[q];
        }
        uint32_t tot;
        uint32_t run = warp_excl_scan(sum, &tot);
#pragma unroll
        for (int q = 0; q < 2; q++) {
            const uint32_t i = lane_id() * 2 + q;
            if (i < G) runpre[i] = run;
            run += len[q];
        }
        if (lane_id() == 0) runpre[G] = tot;
    }
    SJBG_BARRIER();
    const uint32_t T = runpre[G];
    const uint64_t *src = (right ? srcR : srcL) + (uint64_t)tp[w] * kTile;
    uint64_t *out = right ? outR : outL;
    uint32_t *gcur = cursor + (right ? B : 0) + wp.bucket_base + (c << cshift);
    constexpr int kPer = kFineChunk / kFineThreads;
    const uint32_t nwarps = blockDim.x >> 5;
    for (uint32_t gw = 0; gw < T; gw += kFineGather) {
        const uint32_t mg = min(kFineGather, T - gw);
        // gather: warp r % nwarps copies the part of run r inside [gw, gw + mg)
        for (uint32_t r = warp_id(); r < G; r += nwarps) {
            const uint32_t a = max(runpre[r], gw), b = min(runpre[r + 1], gw + mg);
            for (uint32_t x = a + lane_id(); x < b; x += 32)
                cp_async8(tmp + (x - gw), src + runoff[r] + (x - runpre[r]));
        }
        cp_async_wait_all();
        SJBG_BARRIER();
        for (uint32_t ch = 0; ch < mg; ch += kFineChunk) {
            const uint32_t m = min(kFineChunk, mg - ch);
            uint64_t *stage = tmp + ch;
            for (uint32_t f = threadIdx.x; f < nfine; f += blockDim.x) fcnt[f] = 0;
            SJBG_BARRIER();
            uint64_t e[kPer];
            uint32_t fr[kPer];
#pragma unroll
            for (int k = 0; k < kPer; k++) {
                const uint32_t j = threadIdx.x + k * kFineThreads;
                fr[k] = 0xFFFFFFFFu;
                if (j < m) {
                    e[k] = tmp[ch + j];
                    const uint32_t f = cls.bucket((uint32_t)e[k]) & (nfine - 1);
                    fr[k] = (f << 16) | atomicAdd(&fcnt[f], 1u);
                }
            }
            SJBG_BARRIER();
            if (warp_id() == 0) {
                uint32_t a[kCoarseMax / 32], sum = 0;
#pragma unroll
                for (int q = 0; q < (int)(kCoarseMax / 32); q++) {
                    const uint32_t f = lane_id() * (kCoarseMax / 32) + q;
                    a[q] = f < nfine ? fcnt[f] : 0u;
                    sum += a[q];
                }
                uint32_t tot;
                uint32_t run = warp_excl_scan(sum, &tot);
#pragma unroll
                for (int q = 0; q < (int)(kCoarseMax / 32); q++) {
                    const uint32_t f = lane_id() * (kCoarseMax / 32) + q;
                    if (f < nfine) {
                        floc[f] = run;
                        fbase[f] = a[q] ? atomicAdd(&gcur[f], a[q]) : 0u;
                    }
                    run += a[q];
                }
            }
            SJBG_BARRIER();
#pragma unroll
            for (int k = 0; k < kPer; k++) {
                if (fr[k] != 0xFFFFFFFFu) {
                    const uint32_t pos = floc[fr[k] >> 16] + (fr[k] & 0xFFFFu);
                    stage[pos] = e[k];
                    sf[pos] = (uint8_t)(fr[k] >> 16);
                }
            }
            SJBG_BARRIER();
            for (uint32_t pos = threadIdx.x; pos < m; pos += blockDim.x) {
                const uint32_t f = sf[pos];
                out[fbase[f] + (pos - floc[f])] = stage[pos];
            }
            SJBG_BARRIER();
        }
    }
}

__global__ void __launch_bounds__(kFineThreads, 4)
part_fine_kernel(const WinPlan *__restrict__ wins, uint32_t nwin, const uint32_t *__restrict__ tileL,
                 const uint32_t *__restrict__ tileR, const uint32_t *__restrict__ work, uint32_t *__restrict__ cursor,
                 uint32_t B, uint64_t *__restrict__ outL, uint64_t *__restrict__ outR,
                 const LearnedModel *__restrict__ models, const uint64_t *__restrict__ srcL,
                 const uint64_t *__restrict__ srcR, const uint32_t *__restrict__ rows) {
    const uint32_t *pl = work + 2 * kWorkFine * (nwin + 1), *pr = pl + (nwin + 1);
    const uint32_t items = pl[nwin] + pr[nwin];
    for (uint32_t bi = blockIdx.x; bi < items; bi += gridDim.x) {
        SJBG_BARRIER();   // the previous item's shared-memory readers are done
        fine_item(work_item(pl, pr, nwin, bi), wins, nwin, tileL, tileR, cursor, B, outL, outR, models, srcL, srcR,
                  rows);
    }
}

// ------------------------------------------------------------------ 4. bucket join
constexpr uint32_t kMaxProbe = 64;   // linear-probe bound of the count tables

// Count-table slots for buckets of about `target` left tuples (load <= 0.77).
static inline uint32_t count_table_cap(uint32_t target) { return (target * 13u / 10u + 31u) & ~31u; }

struct CountTable {
    uint32_t *keys;              // C + 1 (slot C reserved for key 0xFFFFFFFF)
    uint32_t *cnt;               // C + 1
    unsigned long long *sumf;    // C + 1
    uint32_t C;                  // slots (any size: the hash is scaled, not masked)
};

// Home slot of a key in a table of C slots: a 32-bit multiplicative hash scaled to [0, C).
__device__ __forceinline__ uint32_t ct_home(uint32_t key, uint32_t C) {
    return (uint32_t)(((uint64_t)slot_hash(key, 32) * C) >> 32);
}

// Adds f to a table slot's fr-sum as two 32-bit words (native shared atomics;
// the low word's carry, seen in its returned old value, goes to the high word).
// A 64-bit shared atomicAdd is a compare-and-swap loop, which hot keys turn
// into a long serial chain.
__device__ __forceinline__ void ct_add_sum(unsigned long long *slot, unsigned long long f) {
    uint32_t *w2 = reinterpret_cast<uint32_t *>(slot);   // little-endian: low word first
    const uint32_t flo = (uint32_t)f;
    const uint32_t old = atomicAdd(&w2[0], flo);
    atomicAdd(&w2[1], add_carry((uint32_t)(f >> 32), old, flo));
}

// Insert `c` tuples of `key` with fr-sum `f`.  A key that finds neither itself
// nor a free slot within kMaxProbe slots is refused (false) and joined in a
// later pass; lookups use the same bound, so a refused key is never half-found.
// Every lane inserts its own tuple: with the sums' native 32-bit atomics this
// beats combining a warp's equal keys first, at every skew measured.
__device__ __forceinline__ bool ct_insert(const CountTable &t, uint32_t key, uint32_t c, unsigned long long f) {
    const uint32_t C = t.C;
    if (key == kEmptyKey) {
        atomicAdd(&t.cnt[C], c);
        ct_add_sum(&t.sumf[C], f);
        return true;
    }
    uint32_t s = ct_home(key, C);
    for (uint32_t probe = 0; probe < kMaxProbe; probe++) {
        uint32_t k = *(volatile uint32_t *)&t.keys[s];
        if (k == kEmptyKey) {
            const uint32_t prev = atomicCAS(&t.keys[s], kEmptyKey, key);
            k = prev == kEmptyKey ? key : prev;
        }
        if (k == key) {
            atomicAdd(&t.cnt[s], c);
            ct_add_sum(&t.sumf[s], f);
            return true;
        }
        s = s + 1 == C ? 0 : s + 1;
    }
    return false;
}

__device__ __forceinline__ int ct_lookup(const CountTable &t, uint32_t key) {
    const uint32_t C = t.C;
    if (key == kEmptyKey) return t.cnt[C] ? (int)C : -1;
    uint32_t s = ct_home(key, C);
    for (uint32_t probe = 0; probe < kMaxProbe; probe++) {
        const uint32_t k = t.keys[s];
        if (k == key) return (int)s;
        if (k == kEmptyKey) return -1;
        s = s + 1 == C ? 0 : s + 1;
    }
    return -1;
}

constexpr int kJoinPer = 8;   // elements per thread per tile (independent loads in flight)

__device__ __forceinline__ void join_count_bucket(const JoinItem &ji, uint64_t *__restrict__ partL,
                                                  const uint64_t *__restrict__ partR, WinAcc *__restrict__ acc,
                                                  uint32_t cap) {
    extern __shared__ __align__(16) uint8_t smem_raw[];
    __shared__ uint32_t novf;
    const uint32_t nR = ji.nR, nS = ji.nS;
    if (nR == 0 || nS == 0) return;
    uint64_t *Rb = partL + ji.sR;
    const uint64_t *Sb = partR + ji.sS;
    // the table holds at most nR distinct keys: 2 slots per left tuple (at
    // least 64, at most the launch's capacity of 1.3 per target tuple, which
    // lets two CTAs share an SM), so buckets under the target probe at load
    // <= 1/2: with mostly distinct keys a miss then walks ~3 slots, not ~10
    const uint32_t C = min(cap, max(64u, (nR * 2u + 31u) & ~31u));
    CountTable t;
    t.sumf = reinterpret_cast<unsigned long long *>(smem_raw);
    t.keys = reinterpret_cast<uint32_t *>(t.sumf + C + 1);
    t.cnt = t.keys + C + 1;
    t.C = C;
    const uint32_t tile = kJoinPer * blockDim.x;

    unsigned long long count = 0, prod = 0;
    uint32_t n = nR;
    for (;;) {
        for (uint32_t i = threadIdx.x; i <= C; i += blockDim.x) {
            t.keys[i] = kEmptyKey;
            t.cnt[i] = 0;
            t.sumf[i] = 0;
        }
        if (threadIdx.x == 0) novf = 0;
        SJBG_BARRIER();
        // build: kJoinPer independent loads per thread, then insert them
        for (uint32_t base = 0; base < n; base += tile) {
            uint64_t e[kJoinPer];
#pragma unroll
            for (int k = 0; k < kJoinPer; k++) {
                const uint32_t i = base + k * blockDim.x + threadIdx.x;
                e[k] = i < n ? Rb[i] : 0ull;
            }
            SJBG_BARRIER();   // every read of this tile precedes any overflow write
#pragma unroll
            for (int k = 0; k < kJoinPer; k++) {
                const uint32_t i = base + k * blockDim.x + threadIdx.x;
                const bool valid = i < n;
                const bool ok = !valid || ct_insert(t, (uint32_t)e[k], 1u, sjbg_fr((uint32_t)(e[k] >> 32)));
                if (valid && !ok) Rb[atomicAdd(&novf, 1u)] = e[k];
            }
        }
        SJBG_BARRIER();
        // probe: the same independent-load tiling, no barriers needed
        for (uint32_t base = 0; base < nS; base += tile) {
            uint64_t e[kJoinPer];
#pragma unroll
            for (int k = 0; k < kJoinPer; k++) {
                const uint32_t j = base + k * blockDim.x + threadIdx.x;
                e[k] = j < nS ? Sb[j] : ~0ull;
            }
#pragma unroll
            for (int k = 0; k < kJoinPer; k++) {
                const uint32_t j = base + k * blockDim.x + threadIdx.x;
                if (j < nS) {
                    const int s = ct_lookup(t, (uint32_t)e[k]);
                    if (s >= 0) {
                        count += t.cnt[s];
                        prod += t.sumf[s] * sjbg_gs((uint32_t)(e[k] >> 32));
                    }
                }
            }
        }
        SJBG_BARRIER();
        n = novf;
        SJBG_BARRIER();
        if (n == 0) break;
    }
    flush_acc(&acc[ji.w], count, 0, prod);
}

// ---- direct-addressed bucket join (radix windows)
// In a radix window every key of bucket b has key & (2^lg - 1) == b, so key >> lg
// tells the bucket's keys apart.  When those indices span few values the
// build side is a direct table {count, sum of fr} indexed by key >> lg: an
// insert is three shared atomics and a probe two loads, with no key compares
// or probe loop (the hash table spends about 120 thread instructions per tuple
// there, and is issue- and shared-memory-bound).  A pass covers kDirectMax
// indices; a bucket whose indices need more than kDirectPasses passes is left
// to the hash table, decided after the first build pass and before anything is
// counted.  Measured on 1,024 uneven windows (keys in [0, 4W), about 4,096
// left tuples per bucket, two passes): the bucket joins take 2.02 ms, against
// 2.91 ms with hash tables.
constexpr uint32_t kDirectMax = 8192;
constexpr uint32_t kDirectPasses = 2;
// Larger buckets (a radix window's hot keys) keep the hash table: every extra
// pass and the table reset re-read the bucket, which one CTA would do serially.
constexpr uint32_t kDirectMaxRun = 16384;
// A left run of at most kDirectSave tuples keeps each tuple's table index (16
// bits, 0xFFFF outside the pass's range) in shared memory during the build, so
// the table is reset from there instead of from a second read of the run.
constexpr uint32_t kDirectSave = 4096;
constexpr size_t kDirectBytes =
    (sizeof(unsigned long long) + sizeof(uint32_t)) * kDirectMax + sizeof(uint16_t) * kDirectSave;

// `clean`: the leading table entries known to be zero (CTA-uniform); a direct
// bucket leaves the table zero again, a hash-table bucket does not.  Returns
// false when the bucket's key range is too wide (the table is left zero).
__device__ __forceinline__ bool join_count_direct(const JoinItem &ji, const uint64_t *__restrict__ partL,
                                                  const uint64_t *__restrict__ partR, WinAcc *__restrict__ acc,
                                                  uint32_t &clean) {
    extern __shared__ __align__(16) uint8_t smem_raw[];
    __shared__ uint32_t maxidx_s;
    const uint32_t nR = ji.nR, nS = ji.nS, lg = ji.lg;
    if (nR == 0 || nS == 0) return true;
    unsigned long long *dsum = reinterpret_cast<unsigned long long *>(smem_raw);
    uint32_t *dcnt = reinterpret_cast<uint32_t *>(dsum + kDirectMax);
    uint16_t *dsave = reinterpret_cast<uint16_t *>(dcnt + kDirectMax);   // kDirectSave indices
    const bool save = nR <= kDirectSave;
    const uint64_t *Rb = partL + ji.sR;
    const uint64_t *Sb = partR + ji.sS;
    for (uint32_t i = clean + threadIdx.x; i < kDirectMax; i += blockDim.x) {
        dsum[i] = 0;
        dcnt[i] = 0;
    }
    clean = kDirectMax;
    if (threadIdx.x == 0) maxidx_s = 0;
    SJBG_BARRIER();
    const uint32_t tile = kJoinPer * blockDim.x;
    unsigned long long count = 0, prod = 0;
    uint32_t passes = 1;
    for (uint32_t p = 0; p < passes; p++) {
        const uint32_t lo = p * kDirectMax;
        uint32_t tmax = 0;
        // build: the left keys whose index falls in [lo, lo + kDirectMax)
        for (uint32_t base = 0; base < nR; base += tile) {
            uint64_t e[kJoinPer];
#pragma unroll
            for (int k = 0; k < kJoinPer; k++) {
                const uint32_t i = base + k * blockDim.x + threadIdx.x;
                e[k] = i < nR ? Rb[i] : 0ull;
            }
#pragma unroll
            for (int k = 0; k < kJoinPer; k++) {
                const uint32_t i = base + k * blockDim.x + threadIdx.x;
                if (i < nR) {
                    const uint32_t idx = (uint32_t)e[k] >> lg;
                    tmax = max(tmax, idx);
                    const uint32_t d = idx - lo;   // wraps for indices below the range
                    if (save) dsave[i] = d < kDirectMax ? (uint16_t)d : (uint16_t)0xFFFFu;
                    if (d < kDirectMax) {
                        atomicAdd(&dcnt[d], 1u);
                        ct_add_sum(&dsum[d], sjbg_fr((uint32_t)(e[k] >> 32)));
                    }
                }
            }
        }
        if (p == 0) {
            const uint32_t m = __reduce_max_sync(0xFFFFFFFFu, tmax);
            if (lane_id() == 0) atomicMax(&maxidx_s, m);
        }
        SJBG_BARRIER();
        if (p == 0) {
            passes = maxidx_s / kDirectMax + 1;
            if (passes > kDirectPasses) {   // too wide: undo the first pass, the hash table takes the bucket
                for (uint32_t i = threadIdx.x; i < nR; i += blockDim.x) {
                    const uint32_t d = (uint32_t)Rb[i] >> lg;
                    if (d < kDirectMax) {
                        dcnt[d] = 0;
                        dsum[d] = 0;
                    }
                }
                SJBG_BARRIER();
                return false;
            }
        }
        // probe: the right keys in the range
        for (uint32_t base = 0; base < nS; base += tile) {
            uint64_t e[kJoinPer];
#pragma unroll
            for (int k = 0; k < kJoinPer; k++) {
                const uint32_t j = base + k * blockDim.x + threadIdx.x;
                e[k] = j < nS ? Sb[j] : 0ull;
            }
#pragma unroll
            for (int k = 0; k < kJoinPer; k++) {
                const uint32_t d = ((uint32_t)e[k] >> lg) - lo;
                if (base + k * blockDim.x + threadIdx.x < nS && d < kDirectMax) {
                    const uint32_t c = dcnt[d];
                    if (c) {
                        count += c;
                        prod += dsum[d] * sjbg_gs((uint32_t)(e[k] >> 32));
                    }
                }
            }
        }
        SJBG_BARRIER();
        // leave the table zero: the range's build entries (their saved indices,
        // or for a longer run the run again, from L2)
        for (uint32_t i = threadIdx.x; i < nR; i += blockDim.x) {
            const uint32_t d = save ? (uint32_t)dsave[i] : ((uint32_t)Rb[i] >> lg) - lo;
            if (d < kDirectMax) {
                dcnt[d] = 0;
                dsum[d] = 0;
            }
        }
        SJBG_BARRIER();
    }
    flush_acc(&acc[ji.w], count, 0, prod);
    return true;
}

constexpr uint32_t kEnumChunk = 4096;  // left tuples per chained chunk
constexpr uint32_t kNil = 0xFFFFFFFFu;

__device__ __forceinline__ void join_enum_bucket(uint32_t b, const uint64_t *__restrict__ partL,
                                                 const uint64_t *__restrict__ partR,
                                                 const uint32_t *__restrict__ start, const uint32_t *__restrict__ cnt,
                                                 uint32_t B, const uint32_t *__restrict__ bucket_win,
                                                 WinAcc *__restrict__ acc, const WinPlan *__restrict__ wins,
                                                 sjbg_pair *__restrict__ pairs, uint32_t table_bits) {
    extern __shared__ __align__(16) uint8_t smem_raw[];
    const uint32_t nR = cnt[b], nS = cnt[B + b];
    if (nR == 0 || nS == 0) return;
    const uint64_t *Rb = partL + start[b];
    const uint64_t *Sb = partR + start[B + b];
    const uint32_t w = bucket_win[b];
    const uint32_t Cmax = 1u << table_bits;
    uint32_t *keys = reinterpret_cast<uint32_t *>(smem_raw);   // Cmax + 1
    uint32_t *head = keys + Cmax + 1;                          // Cmax + 1
    uint32_t *next = head + Cmax + 1;                          // kEnumChunk
    uint32_t *vals = next + kEnumChunk;                        // kEnumChunk
    const uint64_t pcap = pairs ? wins[w].pairs_cap : 0;
    sjbg_pair *pout = pairs ? pairs + wins[w].pairs_off : nullptr;

    unsigned long long count = 0, prod = 0, xr = 0;
    for (uint32_t c0 = 0; c0 < nR; c0 += kEnumChunk) {
        const uint32_t m = min(kEnumChunk, nR - c0);
        // at least twice as many slots as the chunk has tuples (slot C holds key 0xFFFFFFFF)
        uint32_t bits = 6;
        while (bits < table_bits && (1u << bits) < 2 * m) bits++;
        const uint32_t C = 1u << bits;
        for (uint32_t i = threadIdx.x; i <= C; i += blockDim.x) {
            keys[i] = kEmptyKey;
            head[i] = kNil;
        }
        SJBG_BARRIER();
        // insert: the trip count is uniform per block (bounds checked inside), and
        // every warp reconverges before the barrier
        for (uint32_t i0 = 0; i0 < m; i0 += blockDim.x) {
            const uint32_t i = i0 + threadIdx.x;
            if (i < m) {
                const uint64_t e = Rb[c0 + i];
                const uint32_t key = (uint32_t)e;
                vals[i] = (uint32_t)(e >> 32);
                uint32_t s;
                if (key == kEmptyKey) {
                    s = C;
                } else {
                    s = slot_hash(key, bits);
                    // at most m <= C/2 keys: a free or matching slot exists within C probes
                    for (uint32_t p = 0; p < C; p++) {
                        const uint32_t prev = atomicCAS(&keys[s], kEmptyKey, key);
                        if (prev == kEmptyKey || prev == key) break;
                        s = (s + 1) & (C - 1);
                    }
                }
                next[i] = atomicExch(&head[s], i);
            }
            __syncwarp();
        }
        SJBG_BARRIER();
        // probe: loop bound is uniform per warp so the pair reservation can use shuffles
        for (uint32_t j0 = 0; j0 < nS; j0 += blockDim.x) {
            const uint32_t j = j0 + threadIdx.x;
            uint32_t h = kNil, sv = 0;
            if (j < nS) {
                const uint64_t e = Sb[j];
                const uint32_t key = (uint32_t)e;
                sv = (uint32_t)(e >> 32);
                uint32_t s = kNil;
                if (key == kEmptyKey) {
                    s = C;
                } else {
                    uint32_t q = slot_hash(key, bits);
                    for (uint32_t p = 0; p <= C; p++) {
                        const uint32_t k = keys[q];
                        if (k == key) { s = q; break; }
                        if (k == kEmptyKey) break;
                        q = (q + 1) & (C - 1);
                    }
                }
                if (s != kNil) h = head[s];
            }
            uint32_t mine = 0;
            const unsigned long long gs = sjbg_gs(sv);
            // chains link indices of this chunk: a walk never takes more than m steps
            for (uint32_t i = h, steps = 0; i < m && steps < m; i = next[i], steps++) {
                const uint32_t rv = vals[i];
                xr ^= sjbg_pair_hash(rv, sv);
                prod += sjbg_fr(rv) * gs;
                mine++;
            }
            count += mine;
            if (pout) {
                uint32_t tot;
                const uint32_t ex = warp_excl_scan(mine, &tot);
                unsigned long long base = 0;
                if (lane_id() == 0 && tot) base = atomicAdd(&acc[w].npairs, (unsigned long long)tot);
                base = __shfl_sync(0xFFFFFFFFu, base, 0) + ex;
                for (uint32_t i = h, steps = 0; i < m && steps < m; i = next[i], steps++) {
                    if (base < pcap) pout[base] = sjbg_pair{vals[i], sv};
                    base++;
                }
            }
            __syncwarp();
        }
        SJBG_BARRIER();
    }
    flush_acc(&acc[w], count, xr, prod);
}

// Bucket joins over the join list (items, length *jn; or, without a list,
// buckets 0 .. B-1, hash tables only): one CTA per item (queue == nullptr) or
// persistent CTAs that take items from a device work queue (an atomic counter)
// until it runs dry.  Buckets of radix windows are joined through direct
// tables when their key indices allow it.
//
// A persistent CTA works one item ahead: while it joins item k, item k+1's
// record is already in shared memory and its two runs are being prefetched
// into L2, and item k+2's record is on its way (an asynchronous copy into
// shared memory, from the index claimed during item k-1).  So no step of a
// bucket waits on the queue, the list or the first loads of its runs.
__global__ void __launch_bounds__(kJoinThreads)
bucket_join_count_kernel(uint64_t *__restrict__ partL, const uint64_t *__restrict__ partR,
                         const uint32_t *__restrict__ start, const uint32_t *__restrict__ cnt, uint32_t B,
                         const uint32_t *__restrict__ bucket_win, WinAcc *__restrict__ acc, uint32_t cap,
                         uint32_t *queue, const JoinItem *__restrict__ items, const uint32_t *__restrict__ jn) {
    const uint32_t nitems = items ? *jn : B;
    uint32_t clean = 0;
    auto join = [&](const JoinItem &ji) {
        if (ji.direct && ji.nR + ji.nS <= kDirectMaxRun && join_count_direct(ji, partL, partR, acc, clean)) return;
        join_count_bucket(ji, partL, partR, acc, cap);
        clean = 0;
    };
    if (!queue || !items) {
        if (blockIdx.x >= nitems) return;
        JoinItem ji;
        if (items) {
            ji = items[blockIdx.x];
        } else {
            const uint32_t i = blockIdx.x;
            ji.b = i; ji.nR = cnt[i]; ji.nS = cnt[B + i]; ji.sR = start[i]; ji.sS = start[B + i];
            ji.w = bucket_win[i]; ji.lg = 0; ji.direct = 0;
        }
        join(ji);
        return;
    }
    __shared__ JoinItem slot_s[3];   // item k, k+1, k+2 (by position: cur_s, then the two ahead)
    __shared__ uint32_t cur_s, valid_s;   // slot of item k; bit q: slot (cur + q) % 3 holds an item
    uint32_t claim = 0;                   // thread 0: index claimed for item k+2
    if (threadIdx.x == 0) {
        const uint32_t i0 = atomicAdd(queue, 1u), i1 = atomicAdd(queue, 1u);
        if (i0 < nitems) slot_s[0] = items[i0];
        if (i1 < nitems) slot_s[1] = items[i1];
        cur_s = 0;
        valid_s = (i0 < nitems ? 1u : 0u) | (i1 < nitems ? 2u : 0u);
        claim = atomicAdd(queue, 1u);
    }
    SJBG_BARRIER();
    while (valid_s & 1u) {
        const uint32_t c = cur_s, v = valid_s;
        const JoinItem ji = slot_s[c];
        const uint32_t c1 = c == 2 ? 0u : c + 1u, c2 = c1 == 2 ? 0u : c1 + 1u;
        uint32_t claim_next = 0;
        if (threadIdx.x == 0) {
            if (v & 2u) {   // item k+1: its runs into L2 while item k is joined
                const JoinItem &nx = slot_s[c1];
                l2_prefetch_bulk(partL + nx.sR, sizeof(uint64_t) * nx.nR);
                l2_prefetch_bulk(partR + nx.sS, sizeof(uint64_t) * nx.nS);
            }
            if (claim < nitems) {   // item k+2's record: shared memory, without blocking
                const uint32_t dst = (uint32_t)__cvta_generic_to_shared(&slot_s[c2]);
                const JoinItem *src = items + claim;
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n"
                             "cp.async.cg.shared.global [%2], [%3], 16;\n"
                             "cp.async.commit_group;\n" ::"r"(dst), "l"(src), "r"(dst + 16u),
                             "l"(reinterpret_cast<const uint8_t *>(src) + 16)
                             : "memory");
            }
            claim_next = atomicAdd(queue, 1u);   // read after this item's join
        }
        join(ji);
        if (threadIdx.x == 0) {
            asm volatile("cp.async.wait_all;\n" ::: "memory");
            cur_s = c1;
            valid_s = (v >> 1) | (claim < nitems ? 2u : 0u);
            claim = claim_next;
        }
        SJBG_BARRIER();
    }
}

__global__ void __launch_bounds__(kJoinThreads)
bucket_join_enum_kernel(const uint64_t *__restrict__ partL, const uint64_t *__restrict__ partR,
                        const uint32_t *__restrict__ start, const uint32_t *__restrict__ cnt, uint32_t B,
                        const uint32_t *__restrict__ bucket_win, WinAcc *__restrict__ acc,
                        const WinPlan *__restrict__ wins, sjbg_pair *__restrict__ pairs, uint32_t table_bits,
                        uint32_t *queue, const JoinItem *__restrict__ jitems, const uint32_t *__restrict__ jn) {
    const uint32_t items = jitems ? *jn : B;
    if (!queue) {
        if (blockIdx.x < items)
            join_enum_bucket(jitems ? jitems[blockIdx.x].b : blockIdx.x, partL, partR, start, cnt, B, bucket_win,
                             acc, wins, pairs, table_bits);
        return;
    }
    __shared__ uint32_t item_s;
    for (;;) {
        SJBG_BARRIER();
        if (threadIdx.x == 0) item_s = atomicAdd(queue, 1u);
        SJBG_BARRIER();
        const uint32_t it = item_s;
        if (it >= items) break;
        join_enum_bucket(jitems ? jitems[it].b : it, partL, partR, start, cnt, B, bucket_win, acc, wins, pairs,
                         table_bits);
    }
}

// ------------------------------------------------------------------ host driver
static uint32_t ceil_log2(uint64_t x) {
    uint32_t b = 0;
    while (((uint64_t)1 << b) < x) b++;
    return b;
}

// The partitioner of a call: the configured one, or for SJBG_PART_AUTO the
// autotuner's choice, else one HBM table per window when every window's table
// stays well inside L2 (at most 2^18 left tuples, 2^21 over the call), else
// radix partitioning.
uint32_t choose_partitioner(const sjbg_handle *h, const WinHost *wins, uint32_t n) {
    if (h->cfg.partitioner != SJBG_PART_AUTO) return h->cfg.partitioner;
    if (h->tune.partitioner) return h->tune.partitioner;
    uint64_t tot = 0, mx = 0;
    for (uint32_t w = 0; w < n; w++) {
        tot += wins[w].n_left;
        mx = std::max(mx, wins[w].n_left);
    }
    return (mx <= (1u << 18) && tot <= (1u << 21)) ? SJBG_PART_NONE : SJBG_PART_RADIX;
}

int hj_lazy_batch(sjbg_handle *h, const sjbg_tuple *dL, const sjbg_tuple *dR, const WinHost *wins, uint32_t n,
                  sjbg_pair *dPairs, WinAcc *acc, bool enumerate, uint32_t *part_used) {
    if (n == 0) return SJBG_OK;
    const uint32_t part = choose_partitioner(h, wins, n);
    if (part == SJBG_PART_NONE) {   // one HBM table per window (hj_global.cu)
        if (part_used) *part_used = SJBG_PART_NONE;
        return hj_global_batch(h, dL, dR, wins, n, dPairs, acc, enumerate);
    }
    const bool learned = part == SJBG_PART_LEARNED;
    if (part_used) *part_used = learned ? SJBG_PART_LEARNED : SJBG_PART_RADIX;
    // left tuples per bucket: 2048 when chains are built, else the tuned target
    const uint64_t target = enumerate ? 2048 : h->tune.bucket_target;

    // ---- plan
    std::vector<WinPlan> plan(n);
    std::vector<uint32_t> tileL(n + 1), tileR(n + 1), hgL(n + 1), hgR(n + 1), itL(n + 1), itR(n + 1);
    std::vector<uint32_t> pbL(n + 1), pbR(n + 1);   // window bases in the partitioned arrays
    uint64_t B = 0, totL = 0, totR = 0;
    uint32_t maxP = 1;
    bool any_two = false, any_one = false;
    for (uint32_t w = 0; w < n; w++) {
        const WinHost &wh = wins[w];
        WinPlan &p = plan[w];
        p.left_off = wh.left_off; p.n_left = wh.n_left; p.right_off = wh.right_off; p.n_right = wh.n_right;
        p.pairs_off = wh.pairs_off; p.pairs_cap = dPairs ? wh.pairs_cap : 0;
        uint32_t lg;
        if (learned) lg = learned_log2_buckets(h, wh.n_left);
        else if (h->cfg.radix_bits) lg = h->cfg.radix_bits;
        else lg = ceil_log2((wh.n_left + target - 1) / target);
        lg = std::min(lg, kMaxBucketsLog2);
        if (wh.n_left == 0 || wh.n_right == 0) lg = 0;
        p.log2_buckets = lg;
        p.bucket_base = (uint32_t)B;
        p.model = 0xFFFFFFFFu;
        p.two_level = lg >= kTwoLevelMinLog2 ? 1u : 0u;
        any_two |= p.two_level != 0;
        any_one |= p.two_level == 0;
        B += 1ull << lg;
        maxP = std::max(maxP, 1u << lg);
        tileL[w + 1] = tileL[w] + (uint32_t)((wh.n_left + kTile - 1) / kTile);
        tileR[w + 1] = tileR[w] + (uint32_t)((wh.n_right + kTile - 1) / kTile);
        // fine-pass CTAs: coarse partitions x groups of kGroupTiles tiles
        const uint32_t nc = 1u << coarse_bits(lg);
        itL[w + 1] = itL[w] + nc * ((tileL[w + 1] - tileL[w] + kGroupTiles - 1) / kGroupTiles);
        itR[w + 1] = itR[w] + nc * ((tileR[w + 1] - tileR[w] + kGroupTiles - 1) / kGroupTiles);
        totL += wh.n_left;
        totR += wh.n_right;
        pbL[w + 1] = (uint32_t)std::min<uint64_t>(totL, 0xFFFFFFFFull);
        pbR[w + 1] = (uint32_t)std::min<uint64_t>(totR, 0xFFFFFFFFull);
    }
    if (B > 0xFFFFFFFFull / 4 || totL >= 0xFFFFFFFFull || totR >= 0xFFFFFFFFull)
        return fail(h, SJBG_E_CAPACITY, "hash join batch exceeds 2^32 tuples per side");
    // counting CTAs per window side: shares of about T / (resident CTAs) tiles
    // (at least kHistTiles), so that one wave holds the call when its window
    // sides are large and the set-up of each CTA is paid over many tiles.
    // When many sides are smaller than a share (uneven batches), shares of an
    // eighth of that keep the CTAs small enough to balance the SMs.
    {
        const size_t histSmem = sizeof(uint32_t) * ((maxP + 1) / 2 * 2) + sizeof(uint64_t) * kTile;
        allow_big_smem(part_hist_kernel, histSmem);
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, part_hist_kernel, kPartThreads, histSmem) !=
            cudaSuccess)
            return fail(h, SJBG_E_CUDA, "counting pass occupancy");
        const uint64_t slots = (uint64_t)std::max(per_sm, 1) * (uint64_t)std::max(h->num_sms, 1);
        const uint64_t T = (uint64_t)tileL[n] + tileR[n];
        uint64_t share = std::max<uint64_t>(kHistTiles, (T + slots - 1) / slots);
        uint64_t ctas = 0;
        for (uint32_t w = 0; w < n; w++)
            ctas += (tileL[w + 1] - tileL[w] + share - 1) / share + (tileR[w + 1] - tileR[w] + share - 1) / share;
        if (ctas > slots + slots / 8) share = std::max<uint64_t>(kHistTiles, T / (8 * slots));
        for (uint32_t w = 0; w < n; w++) {
            hgL[w + 1] = hgL[w] + (uint32_t)((tileL[w + 1] - tileL[w] + share - 1) / share);
            hgR[w + 1] = hgR[w] + (uint32_t)((tileR[w + 1] - tileR[w] + share - 1) / share);
        }
    }
    std::vector<uint32_t> bwin(B);
    for (uint32_t w = 0; w < n; w++)
        for (uint32_t k = 0; k < (1u << plan[w].log2_buckets); k++) bwin[plan[w].bucket_base + k] = w;

    // ---- upload plan, tile prefixes, bucket->window map and (learned) the
    // sampling plan in one copy
    const size_t planB = sizeof(WinPlan) * n, tileB = sizeof(uint32_t) * (n + 1), bwB = sizeof(uint32_t) * B;
    const size_t lsOff = (planB + 8 * tileB + bwB + 15) & ~(size_t)15;
    const size_t upB = lsOff + (learned ? learned_stage_bytes(n) : 0);
    uint8_t *hst = static_cast<uint8_t *>(pinned_get(h, 0, upB));
    uint8_t *dev = static_cast<uint8_t *>(ws_get(h, WS_WIN_PLAN, upB));
    if (!hst || !dev) return fail(h, SJBG_E_NOMEM, "plan buffers");
    std::memcpy(hst, plan.data(), planB);
    std::memcpy(hst + planB, tileL.data(), tileB);
    std::memcpy(hst + planB + tileB, tileR.data(), tileB);
    std::memcpy(hst + planB + 2 * tileB, hgL.data(), tileB);
    std::memcpy(hst + planB + 3 * tileB, hgR.data(), tileB);
    std::memcpy(hst + planB + 4 * tileB, itL.data(), tileB);
    std::memcpy(hst + planB + 5 * tileB, itR.data(), tileB);
    std::memcpy(hst + planB + 6 * tileB, pbL.data(), tileB);
    std::memcpy(hst + planB + 7 * tileB, pbR.data(), tileB);
    std::memcpy(hst + planB + 8 * tileB, bwin.data(), bwB);
    LearnedStage lst{};
    if (learned) lst = learned_stage(h, plan.data(), n, hst + lsOff);
    // the bucket counters are zeroed by the same launch as the upload
    uint32_t *dCnt = static_cast<uint32_t *>(ws_get(h, WS_BUCKET_CNT, sizeof(uint32_t) * 2 * B));
    if (!dCnt) return fail(h, SJBG_E_NOMEM, "partition buffers");
    if (int rc_up = stage_copy_zero(h, dev, hst, upB, dCnt, sizeof(uint32_t) * 2 * B)) return rc_up;
    WinPlan *dPlan = reinterpret_cast<WinPlan *>(dev);
    const uint32_t *dTileL = reinterpret_cast<const uint32_t *>(dev + planB);
    const uint32_t *dTileR = reinterpret_cast<const uint32_t *>(dev + planB + tileB);
    const uint32_t *dHgL = reinterpret_cast<const uint32_t *>(dev + planB + 2 * tileB);
    const uint32_t *dHgR = reinterpret_cast<const uint32_t *>(dev + planB + 3 * tileB);
    const uint32_t *dItL = reinterpret_cast<const uint32_t *>(dev + planB + 4 * tileB);
    const uint32_t *dItR = reinterpret_cast<const uint32_t *>(dev + planB + 5 * tileB);
    const uint32_t *dPbL = reinterpret_cast<const uint32_t *>(dev + planB + 6 * tileB);
    const uint32_t *dPbR = reinterpret_cast<const uint32_t *>(dev + planB + 7 * tileB);
    const uint32_t *dBwin = reinterpret_cast<const uint32_t *>(dev + planB + 8 * tileB);

    uint32_t *dStart = static_cast<uint32_t *>(ws_get(h, WS_BUCKET_START, sizeof(uint32_t) * 2 * B));
    uint32_t *dCur = static_cast<uint32_t *>(ws_get(h, WS_BUCKET_CURSOR, sizeof(uint32_t) * 2 * B));
    uint64_t *dPL = static_cast<uint64_t *>(ws_get(h, WS_PART_LEFT, sizeof(uint64_t) * std::max<uint64_t>(totL, 1)));
    uint64_t *dPR = static_cast<uint64_t *>(ws_get(h, WS_PART_RIGHT, sizeof(uint64_t) * std::max<uint64_t>(totR, 1)));
    if (!dCnt || !dStart || !dCur || !dPL || !dPR) return fail(h, SJBG_E_NOMEM, "partition buffers");

    const LearnedModel *dModels = nullptr;
    HeavyAcc *dHeavy = nullptr;
    if (learned) {
        int rc = learned_prepare(h, dL, dR, lst, dev + lsOff, n, dPlan, &dModels, !enumerate);
        if (rc) return rc;
        dHeavy = static_cast<HeavyAcc *>(ws_get(h, WS_HEAVY, sizeof(HeavyAcc) * kMaxHeavy * n));
        if (!dHeavy) return fail(h, SJBG_E_NOMEM, "heavy-key accumulators");
        SJBG_CK(h, cudaMemsetAsync(dHeavy, 0, sizeof(HeavyAcc) * kMaxHeavy * n, h->stream));
    }
    // the counting pass's output: per window side and tile, its light tuples
    // (compacted windows: packed at the side's start; others: sorted by coarse
    // partition inside the tile's own region), plus the tiles' coarse rows
    const uint64_t tiles64 = (uint64_t)tileL[n] + tileR[n];
    uint64_t *dComp = static_cast<uint64_t *>(ws_get(h, WS_COMPACT, sizeof(uint64_t) * kTile * std::max<uint64_t>(tiles64, 1)));
    uint32_t *dRows = static_cast<uint32_t *>(ws_get(h, WS_COARSE_ROWS, sizeof(uint32_t) * kRow * std::max<uint64_t>(tiles64, 1)));
    // per window side its compacted light tuples, then the join list's length
    uint32_t *dCcnt = static_cast<uint32_t *>(ws_get(h, WS_COMPACT_CNT, sizeof(uint32_t) * (2 * n + 1)));
    uint32_t *dJn = dCcnt + 2 * n;
    // the passes' work prefixes (6 arrays of n + 1), then (16-byte aligned) the join list (B items)
    const size_t workWords = (6 * (size_t)(n + 1) + 3) & ~(size_t)3;
    uint32_t *dWork = static_cast<uint32_t *>(
        ws_get(h, WS_TILE_PREFIX, sizeof(uint32_t) * workWords + sizeof(JoinItem) * (size_t)std::max<uint64_t>(B, 1)));
    JoinItem *dJlist = dWork ? reinterpret_cast<JoinItem *>(dWork + workWords) : nullptr;
    if (!dComp || !dRows || !dCcnt || !dWork) return fail(h, SJBG_E_NOMEM, "partition staging buffers");
    SJBG_CK(h, cudaMemsetAsync(dCcnt, 0, sizeof(uint32_t) * (2 * n + 1), h->stream));
    uint64_t *dCompR = dComp + (uint64_t)kTile * tileL[n];

    const uint32_t tiles = tileL[n] + tileR[n];
    if (tiles) {
        const size_t histSmem = sizeof(uint32_t) * ((maxP + 1) / 2 * 2) + sizeof(uint64_t) * kTile;
        SJBG_CK(h, launch(h, "part_hist", part_hist_kernel, dim3(hgL[n] + hgR[n]), dim3(kPartThreads), histSmem, dL,
                          dR, dPlan, n, dTileL, dTileR, dHgL, dHgR, dCnt, (uint32_t)B, dModels, dHeavy, dComp, dCompR,
                          dCcnt, dRows));
        if (learned)
            SJBG_CK(h, launch(h, "heavy_finish", heavy_finish_kernel, dim3(n), dim3(256), 0, (const WinPlan *)dPlan, n,
                              dModels, (const HeavyAcc *)dHeavy, acc));
        // the tiles each later pass has work for (compacted windows: their light tiles only)
        SJBG_CK(h, launch(h, "part_work", part_work_kernel, dim3(1), dim3(192), 0, (const WinPlan *)dPlan, n, dTileL,
                          dTileR, dItL, dItR, dModels, (const uint32_t *)dCcnt, dWork));
        if (learned && !enumerate) {   // compacted windows exist only with heavy keys
            allow_big_smem(part_hist_light_kernel, sizeof(uint32_t) * maxP);
            const uint32_t lgrid = std::min<uint32_t>(tiles, 4u * (uint32_t)h->num_sms);
            SJBG_CK(h, launch(h, "part_hist_light", part_hist_light_kernel, dim3(lgrid), dim3(kPartThreads),
                              sizeof(uint32_t) * maxP, (const WinPlan *)dPlan, n, dTileL, dTileR,
                              (const uint32_t *)dWork, dCnt, (uint32_t)B, dModels, (const uint64_t *)dComp,
                              (const uint64_t *)dCompR, (const uint32_t *)dCcnt));
        }
        SJBG_CK(h, launch(h, "part_scan", part_scan_win_kernel, dim3(n), dim3(1024), 0, (const WinPlan *)dPlan, dPbL,
                          dPbR, (const uint32_t *)dCnt, dStart, dCur, (uint32_t)B, dModels, dJlist, dJn));
        // single-level windows, and compacted windows (their packed light tuples):
        // a local counting sort per tile
        if (any_one || (learned && !enumerate)) {
            const size_t scatterSmem = kTile * (sizeof(uint64_t) + sizeof(uint16_t)) + 2 * sizeof(uint32_t) * maxP;
            // without a learned partitioner every window is radix-partitioned
            auto scatter = learned ? part_scatter_kernel<false> : part_scatter_kernel<true>;
            allow_big_smem(scatter, scatterSmem);
            const uint32_t sgrid = std::min<uint32_t>(tiles, 3u * 4u * (uint32_t)h->num_sms);
            const uint32_t *wS = dWork + 2 * kWorkScatter * (n + 1);
            SJBG_CK(h, launch(h, "part_scatter", scatter, dim3(sgrid), dim3(kPartThreads), scatterSmem,
                              dL, dR, dPlan, n, dTileL, dTileR, wS, wS + (n + 1), dCur, (uint32_t)B, dPL, dPR,
                              dModels, (const uint64_t *)dComp, (const uint64_t *)dCompR, (const uint32_t *)dCcnt));
        }
        // two-level windows: the fine pass over the tiles' coarse runs
        if (any_two && itL[n] + itR[n]) {
            allow_big_smem(part_fine_kernel, kFineSmem);
            const uint32_t fgrid = std::min<uint32_t>(itL[n] + itR[n], 4u * 4u * (uint32_t)h->num_sms);
            SJBG_CK(h, launch(h, "part_fine", part_fine_kernel, dim3(fgrid), dim3(kFineThreads), kFineSmem,
                              (const WinPlan *)dPlan, n, dTileL, dTileR, (const uint32_t *)dWork, dCur, (uint32_t)B,
                              dPL, dPR, dModels, (const uint64_t *)dComp, (const uint64_t *)dCompR,
                              (const uint32_t *)dRows));
        }
    }
    // persistent CTAs draining a work queue of buckets, or one CTA per bucket
    uint32_t *queue = nullptr;
    dim3 jgrid((uint32_t)B);
    // (chain-building joins keep one CTA per bucket)
    if (!enumerate && h->tune.persistent_join && B > (uint64_t)h->num_sms) {
        queue = static_cast<uint32_t *>(ws_get(h, WS_BUCKET_WIN, 64));
        if (!queue) return fail(h, SJBG_E_NOMEM, "work queue");
        SJBG_CK(h, cudaMemsetAsync(queue, 0, 4, h->stream));
        jgrid = dim3((uint32_t)std::min<uint64_t>(B, (uint64_t)h->num_sms));
    }
    if (enumerate) {
        const uint32_t bits = 13;   // 8192 slots for chunks of 4096
        const size_t smem = sizeof(uint32_t) * (2 * ((1u << bits) + 1) + 2 * kEnumChunk);
        allow_big_smem(bucket_join_enum_kernel, smem);
        SJBG_CK(h, launch(h, "bucket_join_enum", bucket_join_enum_kernel, jgrid, dim3(kJoinThreads), smem,
                          dPL, dPR, dStart, dCnt, (uint32_t)B, dBwin, acc, dPlan, dPairs, bits, queue,
                          (const JoinItem *)dJlist, (const uint32_t *)dJn));
    } else {
        const uint32_t cap = count_table_cap((uint32_t)target);
        const size_t smem =
            std::max((sizeof(unsigned long long) + 2 * sizeof(uint32_t)) * (cap + 1) + 16, kDirectBytes);
        allow_big_smem(bucket_join_count_kernel, smem);
        if (queue) {   // as many persistent CTAs as fit on an SM at this table size (at most 2 by registers)
            const uint32_t per_sm = std::max<uint32_t>(1, (uint32_t)((228u << 10) / (smem + 1024)));
            jgrid = dim3((uint32_t)std::min<uint64_t>(B, (uint64_t)h->num_sms * std::min<uint32_t>(per_sm, 2u)));
        }
        SJBG_CK(h, launch(h, "bucket_join_count", bucket_join_count_kernel, jgrid, dim3(kJoinThreads), smem,
                          dPL, dPR, dStart, dCnt, (uint32_t)B, dBwin, acc, cap, queue, (const JoinItem *)dJlist,
                          (const uint32_t *)dJn));
    }
    return SJBG_OK;
}


// ------------------------------------------------------------------ caller-provided scratch
// One window, count mode, radix partitioning, every buffer carved out of the
// caller-provided device scratch `sc` (no allocation, no host-to-device copy:
// the plan is written by a set-up kernel).  Used by the allocation-free entry
// point in noalloc.cu.
struct RawScratch {
    WinPlan plan;
    uint32_t tile[8];   // tileL {0, tL}, tileR {0, tR}, hgL {0, gL}, hgR {0, gR}
    WinAcc acc[2];      // the window's accumulator, then the call's device status word (acc[1].info, kErr* bits)
};

// Byte offsets of the scratch buffers from a 256-byte aligned base: the
// RawScratch record, the bucket arrays (bucket_win P words, counts, starts and
// cursors 2P words each) and the partitioned sides (8 bytes per tuple).  The
// size check of the entry point and the carving below both use it.
struct RawLayout {
    size_t rs, bwin, part_left, part_right, end;
};

static size_t round256(size_t b) { return (b + 255) & ~size_t(255); }

static RawLayout raw_layout(uint64_t nL, uint64_t nR, uint32_t P) {
    RawLayout l;
    l.rs = 0;
    l.bwin = round256(sizeof(RawScratch));
    l.part_left = l.bwin + round256(sizeof(uint32_t) * 7 * (size_t)P);
    l.part_right = l.part_left + sizeof(uint64_t) * std::max<uint64_t>(nL, 1);
    l.end = l.part_right + sizeof(uint64_t) * std::max<uint64_t>(nR, 1);
    return l;
}

// Radix fan-out of a window: about 4,096 left tuples per bucket; one bucket when a side is empty.
static uint32_t raw_log2_buckets(uint64_t nL, uint64_t nR) {
    uint32_t lg = 0;
    while (((uint64_t)4096 << lg) < nL) lg++;
    return (nL == 0 || nR == 0) ? 0 : lg;
}

__global__ void raw_setup_kernel(RawScratch *rs, uint32_t *bucket_win, uint32_t *cnt, uint32_t P, uint64_t nL,
                                 uint64_t nR, uint32_t lg, uint32_t tL, uint32_t tR) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        WinPlan &p = rs->plan;
        p.left_off = 0; p.n_left = nL; p.right_off = 0; p.n_right = nR;
        p.pairs_off = 0; p.pairs_cap = 0;
        p.bucket_base = 0; p.log2_buckets = lg; p.model = 0xFFFFFFFFu; p.two_level = 0;
        rs->tile[0] = 0; rs->tile[1] = tL;
        rs->tile[2] = 0; rs->tile[3] = tR;
        rs->tile[4] = 0; rs->tile[5] = (tL + kHistTiles - 1) / kHistTiles;
        rs->tile[6] = 0; rs->tile[7] = (tR + kHistTiles - 1) / kHistTiles;
        rs->acc[0] = WinAcc{0, 0, 0, 0, 0};
        rs->acc[1] = WinAcc{0, 0, 0, 0, 0};
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < 2 * P; i += gridDim.x * blockDim.x) {
        cnt[i] = 0;
        if (i < P) bucket_win[i] = 0;
    }
}

// The window's result, with the device status word turned into a status code
// (the bits the batched path maps in device_status_error).
__global__ void raw_finish_kernel(const RawScratch *rs, sjbg_window_result *out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const unsigned long long bits = rs->acc[1].info;
        sjbg_window_result r;
        r.count = rs->acc[0].count;
        r.xor_checksum = 0;
        r.prod_checksum = rs->acc[0].prod;
        r.n_pairs = 0;
        r.status = !bits ? SJBG_OK
                         : (bits & kErrTimeout) ? SJBG_E_TIMEOUT
                                                : SJBG_E_CAPACITY;   // a table or queue could not take its input
        r.flags = 0;
        r.partitioner_used = SJBG_PART_RADIX;
        r.ms = 0.0f;
        *out = r;
    }
}

size_t hj_raw_scratch_bytes(uint64_t max_tuples) {
    const uint32_t P = 1u << raw_log2_buckets(max_tuples, max_tuples);
    return 255 + raw_layout(max_tuples, max_tuples, P).end;   // 255: aligning the caller's base
}

static uint8_t *align256(uint8_t *p) { return reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(p) + 255) & ~uintptr_t(255)); }

int hj_count_window_raw(const sjbg_tuple *dL, uint64_t nL, const sjbg_tuple *dR, uint64_t nR, uint8_t *sc,
                        size_t sc_bytes, sjbg_window_result *dOut, cudaStream_t st) {
    const uint32_t lg = raw_log2_buckets(nL, nR);
    const uint32_t P = 1u << lg;
    const uint32_t tL = (uint32_t)((nL + kTile - 1) / kTile), tR = (uint32_t)((nR + kTile - 1) / kTile);
    uint8_t *base = align256(sc);
    const RawLayout lay = raw_layout(nL, nR, P);
    if (base + lay.end > sc + sc_bytes)
        return fail(nullptr, SJBG_E_CAPACITY, "sjbg_lazy_hj_noalloc: the window does not fit the fixed scratch");
    RawScratch *rs = reinterpret_cast<RawScratch *>(base + lay.rs);
    uint32_t *bwin = reinterpret_cast<uint32_t *>(base + lay.bwin);
    uint32_t *cnt = bwin + P;
    uint32_t *start = cnt + 2 * P;
    uint32_t *cur = start + 2 * P;
    uint64_t *pL = reinterpret_cast<uint64_t *>(base + lay.part_left);
    uint64_t *pR = reinterpret_cast<uint64_t *>(base + lay.part_right);
    // an error left pending by the caller's own earlier work is not this call's
    cudaGetLastError();
    auto launched = [](const char *what) -> int {
        const cudaError_t e = cudaGetLastError();
        return e == cudaSuccess ? SJBG_OK : cuda_fail(nullptr, e, what);
    };
    raw_setup_kernel<<<4, 256, 0, st>>>(rs, bwin, cnt, P, nL, nR, lg, tL, tR);
    if (int rc = launched("sjbg_lazy_hj_noalloc: raw_setup_kernel")) return rc;
    const uint32_t *tl = rs->tile;
    if (tL && tR) {
        const uint32_t groups = (tL + kHistTiles - 1) / kHistTiles + (tR + kHistTiles - 1) / kHistTiles;
        allow_big_smem(part_hist_kernel, sizeof(uint32_t) * P);
        part_hist_kernel<<<groups, kPartThreads, sizeof(uint32_t) * P, st>>>(
            dL, dR, &rs->plan, 1, tl, tl + 2, tl + 4, tl + 6, cnt, P, nullptr, nullptr, nullptr, nullptr, nullptr,
            nullptr);
        if (int rc = launched("sjbg_lazy_hj_noalloc: part_hist_kernel")) return rc;
        part_scan_kernel<<<1, 1024, 0, st>>>(cnt, start, cur, P);
        if (int rc = launched("sjbg_lazy_hj_noalloc: part_scan_kernel")) return rc;
        const size_t scatterSmem = kTile * (sizeof(uint64_t) + sizeof(uint16_t)) + 2 * sizeof(uint32_t) * P;
        allow_big_smem(part_scatter_kernel<true>, scatterSmem);
        // a single-level radix window: the scatter work is every tile
        part_scatter_kernel<true><<<tL + tR, kPartThreads, scatterSmem, st>>>(dL, dR, &rs->plan, 1, tl, tl + 2, tl, tl + 2,
                                                                          cur, P, pL, pR, nullptr, nullptr, nullptr,
                                                                          nullptr);
        if (int rc = launched("sjbg_lazy_hj_noalloc: part_scatter_kernel")) return rc;
        const uint32_t cap = count_table_cap(4096);
        const size_t smem = (sizeof(unsigned long long) + 2 * sizeof(uint32_t)) * (cap + 1) + 16;
        allow_big_smem(bucket_join_count_kernel, smem);
        bucket_join_count_kernel<<<P, kJoinThreads, smem, st>>>(pL, pR, start, cnt, P, bwin, rs->acc, cap, nullptr,
                                                                nullptr, nullptr);
        if (int rc = launched("sjbg_lazy_hj_noalloc: bucket_join_count_kernel")) return rc;
    }
    raw_finish_kernel<<<1, 32, 0, st>>>(rs, dOut);
    return launched("sjbg_lazy_hj_noalloc: raw_finish_kernel");
}

}  // namespace sjbg
