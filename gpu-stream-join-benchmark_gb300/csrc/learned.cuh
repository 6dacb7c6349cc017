// learned.cuh - learned key-CDF partitioner: model layout and device-side inference.
//
// No reference counterpart.  A window's model is a monotone two-stage
// piecewise-linear approximation of the CDF of its light (non-heavy) keys:
//   x      = clamp((key - kmin) * inv_range, 0, 1)                (FP32)
//   leaf   = clamp(floor((root_a * x + root_b) * leaves), 0, leaves-1)
//   cdf    = clamp(slope[leaf] * x + icpt[leaf], lo[leaf], hi[leaf])
//            (the leaf's least-squares line, fitted around its centroid,
//            stored as slope and intercept: one 128-bit load per lookup)
//   bucket = min(P - 1, floor(cdf * P))
// lo/hi are the smallest/largest sampled CDF values routed to the leaf, made
// non-decreasing across leaves, which keeps the whole map monotone in key.
// Heavy keys (sampled frequency above one bucket's fair share) are not
// partitioned at all: their per-window count and checksum sums are
// aggregated while partitioning and combined as |L_k|*|R_k| at the end.
#pragma once

#include <cstddef>

#include "common.cuh"

namespace sjbg {

constexpr uint32_t kMaxLeaves = 256;
constexpr uint32_t kMaxHeavy = 1024;
constexpr uint32_t kHeavySlotsLog2 = 12;
constexpr uint32_t kHeavySlots = 1u << kHeavySlotsLog2;   // shared-memory heavy-key table
constexpr uint32_t kHeavyBucketsLog2 = kHeavySlotsLog2 - 1;   // buckets of two slots (16 bytes)
constexpr uint32_t kHeavyBucket = 0xFFFFFFFFu;            // classify(): heavy key marker
constexpr unsigned long long kHeavyEmpty = ~0ull;

// Shared-memory heavy-key set: 2,048 buckets of two slots, slot = key << 32 |
// index, all ones when empty (a heavy index is < kMaxHeavy, so no entry is
// all ones).  A key lives in one of the two slots of its bucket or not at all,
// so a lookup is one 128-bit load and two compares, with no loop: the per-tuple
// code stays free of branches.  A key that finds its bucket full (the two
// heavier keys of the bucket keep it; about 1% of 512 keys) is not a heavy key:
// every kernel classifies it as light, so its tuples are joined through the
// buckets like any light key.
struct __align__(16) HeavySet {   // 16-byte aligned: copied with 128-bit loads and stores
    unsigned long long slot[kHeavySlots];
};

// What classification reads: copied into shared memory (128-bit loads and
// stores, hence the alignment) by the CTAs that classify.
struct __align__(16) LearnedCore {
    float kmin, inv_range, root_a, root_b;
    uint32_t leaves, log2_buckets, fallback, n_heavy;
    uint32_t compact;     // light tuples are compacted while counting (most tuples are heavy)
    uint32_t cost_check;  // few heavy keys: the check also buckets the sample by radix (the cost rule)
    uint32_t pad_[2];
    float4 leaf[kMaxLeaves];   // per leaf {slope, intercept, lo, hi}
};

struct LearnedModel : LearnedCore {
    uint32_t heavy_keys[kMaxHeavy];
    HeavySet heavy_set;   // built once by the fit, copied into shared memory by each CTA
};

static_assert(sizeof(LearnedCore) % 16 == 0, "LearnedCore is copied in 16-byte units");
static_assert(sizeof(HeavySet) % 16 == 0, "HeavySet is copied in 16-byte units");
static_assert(sizeof(LearnedModel) % 16 == 0, "models are stored back to back");
static_assert(alignof(HeavySet) == 16, "the heavy set (a member at a 16-byte multiple) is copied in 16-byte units");

// Per-window, per-heavy-key aggregates.
struct HeavyAcc {
    unsigned long long cnt_l, sum_l, cnt_r, sum_r;
};

__device__ __forceinline__ uint32_t learned_bucket(const LearnedCore &m, uint32_t key) {
    const uint32_t P = 1u << m.log2_buckets;
    float x = ((float)key - m.kmin) * m.inv_range;
    x = fminf(fmaxf(x, 0.0f), 1.0f);
    int leaf = (int)floorf((m.root_a * x + m.root_b) * (float)m.leaves);
    leaf = min(max(leaf, 0), (int)m.leaves - 1);
    const float4 lf = m.leaf[leaf];
    float y = fmaf(lf.x, x, lf.y);
    y = fminf(fmaxf(y, lf.z), lf.w);
    uint32_t b = (uint32_t)(y * (float)P);
    return b < P ? b : P - 1;
}

// Bucket of a key in the heavy set: the top bits of key * 0x9E3779B97F4A7C15
// (mod 2^64).  The 32-bit product's top bits were measured worse: on the
// streaming workload's keys (Zipf ranks permuted over 2^26) they left 6 of the
// 512 heaviest keys without a slot against 1, and 19 of 30 windows fell back
// to radix partitioning.
__device__ __forceinline__ uint32_t heavy_bucket_of(uint32_t key) { return slot_hash(key, kHeavyBucketsLog2); }

// Build a heavy-key set from keys[0..n) (sorted heaviest first; one CTA; ends
// with a barrier).  claim: 2 * 2^kHeavyBucketsLog2 words of shared scratch.
// Each bucket's first slot goes to its smallest key index, the second to the
// next smallest: the same set whatever the order the threads run in.
__device__ __forceinline__ void heavy_set_build(HeavySet &hs, const uint32_t *keys, uint32_t n, uint32_t *claim) {
    constexpr uint32_t nb = 1u << kHeavyBucketsLog2;
    uint32_t *first = claim, *second = claim + nb;
    for (uint32_t i = threadIdx.x; i < 2 * nb; i += blockDim.x) claim[i] = 0xFFFFFFFFu;
    SJBG_BARRIER();
    for (uint32_t h = threadIdx.x; h < n; h += blockDim.x) atomicMin(&first[heavy_bucket_of(keys[h])], h);
    SJBG_BARRIER();
    for (uint32_t h = threadIdx.x; h < n; h += blockDim.x) {
        const uint32_t b = heavy_bucket_of(keys[h]);
        if (first[b] != h) atomicMin(&second[b], h);
    }
    SJBG_BARRIER();
    for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x) {
        const uint32_t a = first[b], c = second[b];
        hs.slot[2 * b] = a != 0xFFFFFFFFu ? (((unsigned long long)keys[a] << 32) | a) : kHeavyEmpty;
        hs.slot[2 * b + 1] = c != 0xFFFFFFFFu ? (((unsigned long long)keys[c] << 32) | c) : kHeavyEmpty;
    }
    SJBG_BARRIER();
}

// Whether heavy key index h of keys[] got a slot (after heavy_set_build, with its claim scratch).
__device__ __forceinline__ bool heavy_placed(const uint32_t *keys, uint32_t h, const uint32_t *claim) {
    const uint32_t b = heavy_bucket_of(keys[h]);
    return claim[b] == h || claim[(1u << kHeavyBucketsLog2) + b] == h;
}

// Copy `bytes` (a multiple of 16) from global to shared memory (all threads; ends with a barrier).
__device__ __forceinline__ void copy_to_smem(void *dst, const void *src, uint32_t bytes) {
    const uint4 *s = reinterpret_cast<const uint4 *>(src);
    uint4 *d = reinterpret_cast<uint4 *>(dst);
    for (uint32_t i = threadIdx.x; i < bytes / 16; i += blockDim.x) d[i] = s[i];
    SJBG_BARRIER();
}

// Copy a model's prebuilt heavy-key set into shared memory (all threads; ends with a barrier).
__device__ __forceinline__ void heavy_set_load(HeavySet &hs, const LearnedModel *m) {
    copy_to_smem(&hs, &m->heavy_set, sizeof(HeavySet));
}

// Index of `key` among the heavy keys, or kHeavyBucket when it is light.
// An empty slot reads as key 0xFFFFFFFF with index kHeavyBucket, so it needs
// no test of its own (a bucket fills its first slot first).
__device__ __forceinline__ uint32_t heavy_find(const HeavySet &hs, uint32_t key) {
    const uint4 b = reinterpret_cast<const uint4 *>(hs.slot)[heavy_bucket_of(key)];
    // little-endian slots: .x index and .y key of the first, .z and .w of the second
    return b.y == key ? b.x : (b.w == key ? b.z : kHeavyBucket);
}

}  // namespace sjbg

struct sjbg_handle;
namespace sjbg {
struct WinPlan;
uint32_t learned_log2_buckets(sjbg_handle *h, uint64_t n_left);
// Sizes of the sampling buffers, from the windows' plans.
struct LearnedStage {
    uint64_t table_total, keys_total, list_total;
    uint32_t max_m, max_list;
};
// Host bytes the sampling plan of n windows takes (uploaded with the batch plan).
size_t learned_stage_bytes(uint32_t n);
// Writes the sampling plan of n windows (learned_stage_bytes(n) bytes) to hst.
LearnedStage learned_stage(sjbg_handle *h, const WinPlan *plan, uint32_t n, uint8_t *hst);
// Sample, fit and check every window's model from the uploaded sampling plan
// (dstage, on the device); writes models and sets WinPlan::model on device
// (dPlan) for the windows that keep their model.  allow_heavy = false keeps
// every key in the partitions (needed when pairs are enumerated).
int learned_prepare(sjbg_handle *h, const sjbg_tuple *dL, const sjbg_tuple *dR, const LearnedStage &st,
                    uint8_t *dstage, uint32_t n, WinPlan *dPlan, const LearnedModel **dModels, bool allow_heavy);
}  // namespace sjbg
