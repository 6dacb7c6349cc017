// eager_dev.cuh - device routines of the eager joins shared by the per-batch
// kernels (eager.cu) and the persistent eager kernel (eager_pk.cu): the
// side tables of the hash join and the searches of the sort-merge join.
#pragma once

#include "eager.cuh"

namespace sjbg {

constexpr uint32_t kNilIdx = 0xFFFFFFFFu;

struct ETab {
    uint32_t *keys, *cnt, *head, *next;
    unsigned long long *sum;
    uint32_t bits;
};

__device__ __forceinline__ int etab_lookup(const ETab &t, uint32_t key) {
    const uint32_t C = 1u << t.bits;
    if (key == kEmptyKey) return t.cnt[C] ? (int)C : -1;
    uint32_t s = slot_hash(key, t.bits);
    for (uint32_t p = 0; p < C; p++) {
        const uint32_t k = t.keys[s];
        if (k == key) return (int)s;
        if (k == kEmptyKey) return -1;
        s = (s + 1) & (C - 1);
    }
    return -1;
}

__device__ __forceinline__ uint32_t etab_claim(const ETab &t, uint32_t key) {
    const uint32_t C = 1u << t.bits;
    if (key == kEmptyKey) return C;
    uint32_t s = slot_hash(key, t.bits);
    for (uint32_t p = 0; p < C; p++) {   // the table is at most half full
        const uint32_t prev = atomicCAS(&t.keys[s], kEmptyKey, key);
        if (prev == kEmptyKey || prev == key) return s;
        s = (s + 1) & (C - 1);
    }
    return C;   // unreachable by sizing
}

__device__ __forceinline__ unsigned long long own_hash(int side, uint32_t val) {
    return sjbg_fside(val, side == 0 ? 0u : 1u);
}

__device__ __forceinline__ void flush_batch(WinAcc *acc, unsigned long long *bcount, unsigned long long count,
                                            unsigned long long xr, unsigned long long prod) {
    flush_acc(acc, count, xr, prod);
    const unsigned long long c = warp_sum_u64(count);
    if (lane_id() == 0 && c) atomicAdd(bcount, c);
}

// One incoming tuple of a hash-join batch (called by whole warps; `valid`
// false for the lanes past the batch): probe the other side's table (count
// and prod in O(1); the chain of the other side's tuple indices for the xor
// checksum and the pairs), then add the tuple, which sits at index `idx` of
// its side's tuple store, to its own side's table.  The batch's matches go
// to *bcount and the window totals to *acc.
template <bool kEnum, bool kPairs>
__device__ __forceinline__ void eager_hj_step(bool valid, uint32_t key, uint32_t val, uint32_t idx, int side,
                                              const ETab &own, const ETab &oth, const sjbg_tuple *oth_tuples,
                                              uint32_t oth_n, WinAcc *acc, unsigned long long *bcount,
                                              sjbg_pair *pairs, uint64_t pcap) {
    const unsigned long long oh = own_hash(side, val);
    unsigned long long count = 0, xr = 0, prod = 0;
    uint32_t head = kNilIdx, mine = 0;
    if (valid) {
        const int s = etab_lookup(oth, key);
        if (s >= 0) {
            mine = oth.cnt[s];
            count = mine;
            prod = oh * oth.sum[s];
            head = oth.head[s];
        }
    }
    // chains hold indices of the other side's tuples; walks stop at its size
    if (kEnum) {
        uint32_t steps = 0;
        for (uint32_t j = head; j < oth_n && steps < oth_n; j = oth.next[j], steps++) {
            const uint32_t ov = oth_tuples[j].val;
            xr ^= side == 0 ? sjbg_pair_hash(val, ov) : sjbg_pair_hash(ov, val);
        }
    }
    if (kPairs) {
        uint32_t tot;
        const uint32_t ex = warp_excl_scan(mine, &tot);
        unsigned long long b = 0;
        if (lane_id() == 0 && tot) b = atomicAdd(&acc->npairs, (unsigned long long)tot);
        b = __shfl_sync(0xFFFFFFFFu, b, 0) + ex;
        uint32_t steps = 0;
        for (uint32_t j = head; j < oth_n && steps < oth_n; j = oth.next[j], b++, steps++) {
            const uint32_t ov = oth_tuples[j].val;
            if (b < pcap) pairs[b] = side == 0 ? sjbg_pair{val, ov} : sjbg_pair{ov, val};
        }
    }
    if (valid) {   // add the tuple to its own side's table
        const uint32_t s = etab_claim(own, key);
        atomicAdd(&own.cnt[s], 1u);
        atomicAdd(&own.sum[s], oh);
        own.next[idx] = atomicExch(&own.head[s], idx);
    }
    flush_batch(acc, bcount, count, xr, prod);
}

__device__ __forceinline__ uint32_t lower_bound_u32(const uint32_t *a, uint32_t n, uint32_t key) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}
__device__ __forceinline__ uint32_t upper_bound_u32(const uint32_t *a, uint32_t n, uint32_t key) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (a[mid] <= key) lo = mid + 1; else hi = mid;
    }
    return lo;
}


}  // namespace sjbg
