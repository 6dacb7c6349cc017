// hj_global.cu - lazy hash join without partitioning (SJBG_PART_NONE): one
// open-addressing table per window in HBM, built from the left side and
// probed by the right side.
//
// The reference's lazy GPU hash join builds a bucket-chained table in HBM,
// bucket = key % numDistinctKeys (src/sjb/windowing/lazy/executor/GPU/GPU_HJ.cu:9-60
// build, :62-120 probe).  Here the table is open-addressed with linear
// probing at load <= 1/2, sized per window (no key-domain hint needed):
//   count mode  slot = {~key, count, sum fr(val)} (16 B): a probe reads one
//               sector and adds count and count-weighted checksum sums;
//               equal keys within a warp are combined before the atomics;
//   enum mode   slot = {~key, chain head + 1} (8 B), plus per left tuple its
//               val and the next index of its key's chain; every pair is
//               visited for the xor checksum and optionally written.
// Stored tags are ~key, so an all-zero table is empty (one memset clears
// every window); key 0xFFFFFFFF (tag 0) owns the extra slot C of its table.
// Fits windows whose tables stay in L2; large windows are better served by
// the partitioned join in hj.cu.
#include <algorithm>
#include <cstring>
#include <vector>

#include "runtime.h"

namespace sjbg {

constexpr int kGThreads = 256;
constexpr int kGPer = 8;
constexpr uint32_t kGTile = kGThreads * kGPer;   // tuples per CTA

struct GWin {
    uint64_t left_off, n_left, right_off, n_right, pairs_off, pairs_cap;
    uint64_t table_off;   // first slot of this window's table
    uint64_t lbase;       // first entry of this window's next / vals arrays
    uint32_t bits;        // table of 2^bits slots (+1 for key 0xFFFFFFFF)
    uint32_t pad;
};

struct __align__(16) GSlot {
    uint32_t tag;   // ~key; 0 = empty
    uint32_t cnt;
    unsigned long long sumf;
};

__device__ __forceinline__ uint32_t gfind_window(const uint32_t *prefix, uint32_t n, uint32_t t) {
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (prefix[mid] <= t) lo = mid; else hi = mid;
    }
    return lo;
}

// 128-bit compare-and-swap of a slot held as two 64-bit words (lo = tag |
// count << 32, hi = sum): installs want when the slot equals cmp; returns the
// slot's prior low word (tag and count), which is all the callers test.
__device__ __forceinline__ unsigned long long gslot_cas(GSlot *s, unsigned long long cmp_lo, unsigned long long cmp_hi,
                                                        unsigned long long want_lo, unsigned long long want_hi) {
    unsigned long long lo, hi;
    asm volatile(
        "{\n\t.reg .b128 d, b, c;\n\t"
        "mov.b128 b, {%2, %3};\n\t"
        "mov.b128 c, {%4, %5};\n\t"
        "atom.global.cas.b128 d, [%6], b, c;\n\t"
        "mov.b128 {%0, %1}, d;\n\t}"
        : "=l"(lo), "=l"(hi)
        : "l"(cmp_lo), "l"(cmp_hi), "l"(want_lo), "l"(want_hi), "l"(s)
        : "memory");
    (void)hi;
    return lo;
}

// Slot of `key` in a table of 2^bits slots: claimed when absent (insert) or
// looked up (insert == false, returns 0xFFFFFFFF when absent).  The table is
// at most half full, so a probe ends within 2^bits steps.
template <typename Slot>
__device__ __forceinline__ uint32_t gslot(Slot *t, uint32_t bits, uint32_t key, bool insert, uint32_t *err) {
    const uint32_t C = 1u << bits;
    if (key == 0xFFFFFFFFu) return C;
    const uint32_t tag = ~key;
    uint32_t s = slot_hash(key, bits);
    for (uint32_t p = 0; p < C; p++) {
        uint32_t cur = *(volatile uint32_t *)&t[s].tag;
        if (cur == 0u) {
            if (!insert) return 0xFFFFFFFFu;
            const uint32_t prev = atomicCAS(&t[s].tag, 0u, tag);
            cur = prev == 0u ? tag : prev;
        }
        if (cur == tag) return s;
        s = (s + 1) & (C - 1);
    }
    atomicOr(err, kErrTableFull);
    return 0xFFFFFFFFu;
}

__global__ void __launch_bounds__(kGThreads, 4)
gbuild_count_kernel(const sjbg_tuple *__restrict__ L, const GWin *__restrict__ wins, uint32_t nwin,
                    const uint32_t *__restrict__ tiles, GSlot *__restrict__ table, uint32_t *err) {
    const uint32_t w = gfind_window(tiles, nwin, blockIdx.x);
    const GWin wp = wins[w];
    GSlot *t = table + wp.table_off;
    const uint64_t start = (uint64_t)(blockIdx.x - tiles[w]) * kGTile;
    const uint2 *src = reinterpret_cast<const uint2 *>(L + wp.left_off + start);
    const uint64_t n = wp.n_left - start;
    uint2 v[kGPer];
#pragma unroll
    for (int k = 0; k < kGPer; k++) {
        const uint32_t i = threadIdx.x + k * kGThreads;
        v[k] = i < n ? __ldg(src + 2 * i) : make_uint2(0u, 0u);
    }
    const unsigned full = 0xFFFFFFFFu;
    const uint32_t C = 1u << wp.bits;
    // four tuples at a time: their groups, then their slots claimed or found at
    // once (one round trip for the four, not one per tuple)
    constexpr int kGroup = 4;
    static_assert(kGPer % kGroup == 0, "tuples per thread in groups of four");
#pragma unroll
    for (int g = 0; g < kGPer; g += kGroup) {
        // lanes with equal keys: the leader adds the group's count and fr-sum
        unsigned lead = 0;   // bit q: this lane leads tuple g + q's group
        uint32_t gcnt[kGroup];
        unsigned long long gsum[kGroup];
#pragma unroll
        for (int q = 0; q < kGroup; q++) {
            const int k = g + q;
            const bool valid = threadIdx.x + k * kGThreads < n;
            const uint32_t key = v[k].x;
            const unsigned long long f = valid ? sjbg_fr(v[k].y) : 0ull;
            const unsigned active = __ballot_sync(full, valid);
            unsigned grp = __match_any_sync(full, key) & active;
            if (!valid) grp = 1u << lane_id();
            const int leader = __ffs(grp) - 1;
            gsum[q] = f;
            gcnt[q] = __popc(grp);
            unsigned multi = __ballot_sync(full, valid && __popc(grp) > 1 && (int)lane_id() == leader);
            while (multi) {
                const int ld = __ffs(multi) - 1;
                multi &= multi - 1;
                const unsigned m = __shfl_sync(full, grp, ld);
                const unsigned long long sm = warp_sum_u64(((m >> lane_id()) & 1u) ? f : 0ull);
                if ((int)lane_id() == ld) gsum[q] = sm;
            }
            if (valid && (int)lane_id() == leader) lead |= 1u << q;
        }
        // A 128-bit compare-and-swap of an all-zero slot installs {tag, count,
        // sum} whole, so a key new to the table costs one atomic; otherwise it
        // returns the slot, and a slot holding the key gets the count and sum
        // added (a taken slot's count is never 0)
        uint32_t slot[kGroup], got[kGroup];   // got: the tag found in the slot
#pragma unroll
        for (int q = 0; q < kGroup; q++) {
            const uint32_t key = v[g + q].x;
            slot[q] = C;
            got[q] = 0u;
            if (((lead >> q) & 1u) && key != 0xFFFFFFFFu) {
                slot[q] = slot_hash(key, wp.bits);
                const unsigned long long old = gslot_cas(&t[slot[q]], 0ull, 0ull,
                                                         (unsigned long long)(~key) | ((unsigned long long)gcnt[q] << 32),
                                                         gsum[q]);
                got[q] = (uint32_t)old;
                if ((old >> 32) == 0ull) lead &= ~(1u << q);   // installed: nothing left to add
            }
        }
#pragma unroll
        for (int q = 0; q < kGroup; q++) {
            if (!((lead >> q) & 1u)) continue;
            const uint32_t key = v[g + q].x;
            if (key != 0xFFFFFFFFu) {
                const uint32_t tag = ~key;
                uint32_t p = 1;
                bool installed = false;
                while (got[q] != tag && p < C) {
                    slot[q] = (slot[q] + 1) & (C - 1);
                    const unsigned long long old = gslot_cas(&t[slot[q]], 0ull, 0ull,
                                                             (unsigned long long)tag | ((unsigned long long)gcnt[q] << 32),
                                                             gsum[q]);
                    if ((old >> 32) == 0ull) {
                        installed = true;
                        break;
                    }
                    got[q] = (uint32_t)old;
                    p++;
                }
                if (installed) continue;
                if (got[q] != tag) {   // the whole table is taken: cannot happen at load <= 1/2
                    atomicOr(err, kErrTableFull);
                    continue;
                }
            }
            atomicAdd(&t[slot[q]].cnt, gcnt[q]);
            atomicAdd(&t[slot[q]].sumf, gsum[q]);
        }
    }
}

__global__ void __launch_bounds__(kGThreads, 4)
gprobe_count_kernel(const sjbg_tuple *__restrict__ R, const GWin *__restrict__ wins, uint32_t nwin,
                    const uint32_t *__restrict__ tiles, const GSlot *__restrict__ table, WinAcc *__restrict__ acc) {
    const uint32_t w = gfind_window(tiles, nwin, blockIdx.x);
    const GWin wp = wins[w];
    const GSlot *t = table + wp.table_off;
    const uint64_t start = (uint64_t)(blockIdx.x - tiles[w]) * kGTile;
    const uint2 *src = reinterpret_cast<const uint2 *>(R + wp.right_off + start);
    const uint64_t n = wp.n_right - start;
    const uint32_t C = 1u << wp.bits;
    uint2 v[kGPer];
#pragma unroll
    for (int k = 0; k < kGPer; k++) {
        const uint32_t i = threadIdx.x + k * kGThreads;
        v[k] = i < n ? __ldg(src + 2 * i) : make_uint2(0u, 0u);
    }
    unsigned long long count = 0, prod = 0;
    // every tuple's home slot is read at once (one 16-byte load: tag, count
    // and sum together), then collisions walk on
    GSlot e[kGPer];
    uint32_t slot[kGPer];
#pragma unroll
    for (int k = 0; k < kGPer; k++) {
        const uint32_t key = v[k].x;
        slot[k] = key == 0xFFFFFFFFu ? C : slot_hash(key, wp.bits);
        if (threadIdx.x + k * kGThreads < n) {
            const uint4 q = __ldg(reinterpret_cast<const uint4 *>(&t[slot[k]]));
            e[k].tag = q.x;
            e[k].cnt = q.y;
            e[k].sumf = ((unsigned long long)q.w << 32) | q.z;
        } else {
            e[k].tag = 0u;
            e[k].cnt = 0u;
            e[k].sumf = 0ull;
        }
    }
#pragma unroll
    for (int k = 0; k < kGPer; k++) {
        if (threadIdx.x + k * kGThreads >= n) continue;
        const uint32_t key = v[k].x;
        if (key != 0xFFFFFFFFu) {   // (slot C of key 0xFFFFFFFF needs no tag test)
            const uint32_t tag = ~key;
            for (uint32_t p = 1; e[k].tag != tag && e[k].tag != 0u && p < C; p++) {
                slot[k] = (slot[k] + 1) & (C - 1);
                const uint4 q = __ldg(reinterpret_cast<const uint4 *>(&t[slot[k]]));
                e[k].tag = q.x;
                e[k].cnt = q.y;
                e[k].sumf = ((unsigned long long)q.w << 32) | q.z;
            }
            if (e[k].tag != tag) continue;
        }
        count += e[k].cnt;
        prod += e[k].sumf * sjbg_gs(v[k].y);
    }
    flush_acc(&acc[w], count, 0, prod);
}

struct ESlot {
    uint32_t tag;    // ~key; 0 = empty
    uint32_t head;   // chain head + 1; 0 = none
};

__global__ void __launch_bounds__(kGThreads)
gbuild_enum_kernel(const sjbg_tuple *__restrict__ L, const GWin *__restrict__ wins, uint32_t nwin,
                   const uint32_t *__restrict__ tiles, ESlot *__restrict__ table, uint32_t *__restrict__ next,
                   uint32_t *__restrict__ vals, uint32_t *err) {
    const uint32_t w = gfind_window(tiles, nwin, blockIdx.x);
    const GWin wp = wins[w];
    ESlot *t = table + wp.table_off;
    const uint64_t start = (uint64_t)(blockIdx.x - tiles[w]) * kGTile;
    const uint2 *src = reinterpret_cast<const uint2 *>(L + wp.left_off);
#pragma unroll
    for (int k = 0; k < kGPer; k++) {
        const uint64_t i = start + threadIdx.x + k * kGThreads;
        if (i >= wp.n_left) continue;
        const uint2 e = __ldg(src + 2 * i);
        vals[wp.lbase + i] = e.y;
        const uint32_t s = gslot(t, wp.bits, e.x, true, err);
        if (s != 0xFFFFFFFFu) next[wp.lbase + i] = atomicExch(&t[s].head, (uint32_t)i + 1u);
    }
}

__global__ void __launch_bounds__(kGThreads)
gprobe_enum_kernel(const sjbg_tuple *__restrict__ R, const GWin *__restrict__ wins, uint32_t nwin,
                   const uint32_t *__restrict__ tiles, const ESlot *__restrict__ table,
                   const uint32_t *__restrict__ next, const uint32_t *__restrict__ vals, WinAcc *__restrict__ acc,
                   sjbg_pair *__restrict__ pairs) {
    const uint32_t w = gfind_window(tiles, nwin, blockIdx.x);
    const GWin wp = wins[w];
    const ESlot *t = table + wp.table_off;
    const uint32_t *nx = next + wp.lbase;
    const uint32_t *vl = vals + wp.lbase;
    const uint64_t start = (uint64_t)(blockIdx.x - tiles[w]) * kGTile;
    const uint2 *src = reinterpret_cast<const uint2 *>(R + wp.right_off);
    const uint32_t C = 1u << wp.bits;
    const uint64_t pcap = pairs ? wp.pairs_cap : 0;
    sjbg_pair *pout = pairs ? pairs + wp.pairs_off : nullptr;
    unsigned long long count = 0, prod = 0, xr = 0;
    // the loop bound is uniform per warp, so the pair reservation can use shuffles
    for (int k = 0; k < kGPer; k++) {
        const uint64_t j = start + threadIdx.x + k * kGThreads;
        uint32_t h = 0, sv = 0;
        if (j < wp.n_right) {
            const uint2 e = __ldg(src + 2 * j);
            sv = e.y;
            uint32_t s = 0xFFFFFFFFu;
            if (e.x == 0xFFFFFFFFu) {
                s = C;
            } else {
                const uint32_t tag = ~e.x;
                uint32_t q = slot_hash(e.x, wp.bits);
                for (uint32_t p = 0; p < C; p++) {
                    const uint32_t cur = t[q].tag;
                    if (cur == tag) { s = q; break; }
                    if (cur == 0u) break;
                    q = (q + 1) & (C - 1);
                }
            }
            if (s != 0xFFFFFFFFu) h = t[s].head;
        }
        const unsigned long long gs = sjbg_gs(sv);
        uint32_t mine = 0;
        // a chain links distinct left indices of this window: at most n_left steps
        for (uint32_t i = h, steps = 0; i != 0 && steps < wp.n_left; i = nx[i - 1], steps++) {
            const uint32_t rv = vl[i - 1];
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
            for (uint32_t i = h, steps = 0; i != 0 && steps < wp.n_left; i = nx[i - 1], steps++) {
                if (base < pcap) pout[base] = sjbg_pair{vl[i - 1], sv};
                base++;
            }
        }
        __syncwarp();
    }
    flush_acc(&acc[w], count, xr, prod);
}

int hj_global_batch(sjbg_handle *h, const sjbg_tuple *dL, const sjbg_tuple *dR, const WinHost *wins, uint32_t n,
                    sjbg_pair *dPairs, WinAcc *acc, bool enumerate) {
    if (n == 0) return SJBG_OK;
    std::vector<GWin> gw(n);
    std::vector<uint32_t> tl(n + 1, 0), tr(n + 1, 0);
    uint64_t slots = 0, lefts = 0;
    for (uint32_t w = 0; w < n; w++) {
        const WinHost &x = wins[w];
        GWin &g = gw[w];
        g.left_off = x.left_off; g.n_left = x.n_left; g.right_off = x.right_off; g.n_right = x.n_right;
        g.pairs_off = x.pairs_off; g.pairs_cap = dPairs ? x.pairs_cap : 0;
        uint32_t bits = 6;
        while (bits < 31 && (1ull << bits) < 2 * x.n_left) bits++;
        g.bits = bits;
        g.pad = 0;
        g.table_off = slots;
        g.lbase = lefts;
        slots += (1ull << bits) + 1;
        lefts += x.n_left;
        const uint64_t ltiles = x.n_right ? (x.n_left + kGTile - 1) / kGTile : 0;   // empty right: nothing to build
        const uint64_t rtiles = x.n_left ? (x.n_right + kGTile - 1) / kGTile : 0;
        if (tl[w] + ltiles > 0xFFFFFFFFull || tr[w] + rtiles > 0xFFFFFFFFull)
            return fail(h, SJBG_E_CAPACITY, "hash join batch exceeds 2^32 tiles");
        tl[w + 1] = tl[w] + (uint32_t)ltiles;
        tr[w + 1] = tr[w] + (uint32_t)rtiles;
    }
    const size_t slotB = enumerate ? sizeof(ESlot) : sizeof(GSlot);
    const size_t gwB = sizeof(GWin) * n, tB = sizeof(uint32_t) * (n + 1);
    const size_t upB = gwB + 2 * tB;
    uint8_t *hst = static_cast<uint8_t *>(pinned_get(h, 0, upB));
    uint8_t *dev = static_cast<uint8_t *>(ws_get(h, WS_WIN_PLAN, upB));
    void *dTab = ws_get(h, WS_AUX3, slotB * slots);
    uint32_t *dNext = nullptr, *dVals = nullptr;
    if (enumerate) {
        dNext = static_cast<uint32_t *>(ws_get(h, WS_PART_LEFT, sizeof(uint32_t) * std::max<uint64_t>(lefts, 1)));
        dVals = static_cast<uint32_t *>(ws_get(h, WS_PART_RIGHT, sizeof(uint32_t) * std::max<uint64_t>(lefts, 1)));
    }
    if (!hst || !dev || !dTab || (enumerate && (!dNext || !dVals))) return fail(h, SJBG_E_NOMEM, "hash table buffers");
    std::memcpy(hst, gw.data(), gwB);
    std::memcpy(hst + gwB, tl.data(), tB);
    std::memcpy(hst + gwB + tB, tr.data(), tB);
    if (int rc_up = stage_copy_zero(h, dev, hst, upB, dTab, slotB * slots)) return rc_up;
    const GWin *dW = reinterpret_cast<const GWin *>(dev);
    const uint32_t *dTl = reinterpret_cast<const uint32_t *>(dev + gwB);
    const uint32_t *dTr = reinterpret_cast<const uint32_t *>(dev + gwB + tB);
    uint32_t *dErr = reinterpret_cast<uint32_t *>(&acc[n].info);   // the call's status word (low half)
    if (enumerate) {
        ESlot *t = static_cast<ESlot *>(dTab);
        if (tl[n])
            SJBG_CK(h, launch(h, "ht_build_enum", gbuild_enum_kernel, dim3(tl[n]), dim3(kGThreads), 0, dL, dW, n, dTl,
                              t, dNext, dVals, dErr));
        if (tr[n])
            SJBG_CK(h, launch(h, "ht_probe_enum", gprobe_enum_kernel, dim3(tr[n]), dim3(kGThreads), 0, dR, dW, n, dTr,
                              (const ESlot *)t, (const uint32_t *)dNext, (const uint32_t *)dVals, acc, dPairs));
    } else {
        GSlot *t = static_cast<GSlot *>(dTab);
        if (tl[n])
            SJBG_CK(h, launch(h, "ht_build_count", gbuild_count_kernel, dim3(tl[n]), dim3(kGThreads), 0, dL, dW, n,
                              dTl, t, dErr));
        if (tr[n])
            SJBG_CK(h, launch(h, "ht_probe_count", gprobe_count_kernel, dim3(tr[n]), dim3(kGThreads), 0, dR, dW, n,
                              dTr, (const GSlot *)t, acc));
    }
    return SJBG_OK;
}

}  // namespace sjbg
