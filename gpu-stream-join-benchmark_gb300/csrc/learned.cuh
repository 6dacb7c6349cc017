// learned.cuh - learned key-CDF partitioner: model layout and device-side inference.
//
// No reference counterpart.  A window's model is a monotone two-stage
// piecewise-linear approximation of the CDF of its light (non-heavy) keys:
//   x      = clamp((key - kmin) * inv_range, 0, 1)                (FP32)
//   leaf   = clamp(floor((root_a * x + root_b) * leaves), 0, leaves-1)
//   cdf    = clamp(mean_y[leaf] + slope[leaf] * (x - mean_x[leaf]), lo[leaf], hi[leaf])
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
constexpr uint32_t kMaxHeavy = 512;
constexpr uint32_t kHeavySlotsLog2 = 12;
constexpr uint32_t kHeavySlots = 1u << kHeavySlotsLog2;   // shared-memory heavy-key table (load <= 1/8)
constexpr uint32_t kHeavyBucket = 0xFFFFFFFFu;            // classify(): heavy key marker
constexpr unsigned long long kHeavyEmpty = ~0ull;

// Shared-memory heavy-key set: slot = key << 32 | index, all ones when empty
// (a heavy index is < kMaxHeavy, so no entry is all ones).  One 64-bit load
// per probe.
struct __align__(16) HeavySet {   // 16-byte aligned: copied with 128-bit loads and stores
    unsigned long long slot[kHeavySlots];
};

// What classification reads: copied into shared memory (128-bit loads and
// stores, hence the alignment) by the CTAs that classify.
struct __align__(16) LearnedCore {
    float kmin, inv_range, root_a, root_b;
    uint32_t leaves, log2_buckets, fallback, n_heavy;
    uint32_t compact;     // light tuples are compacted while counting (most tuples are heavy)
    uint32_t pad_[3];
    float slope[kMaxLeaves], mean_x[kMaxLeaves], mean_y[kMaxLeaves], lo[kMaxLeaves], hi[kMaxLeaves];
};

struct LearnedModel : LearnedCore {
    uint32_t heavy_keys[kMaxHeavy];
    HeavySet heavy_set;   // built once by the fit, copied into shared memory by each CTA
};

static_assert(sizeof(LearnedCore) % 16 == 0, "LearnedCore is copied in 16-byte units");
static_assert(sizeof(HeavySet) % 16 == 0, "HeavySet is copied in 16-byte units");
static_assert(sizeof(LearnedModel) % 16 == 0, "models are stored back to back");
static_assert(offsetof(LearnedModel, heavy_set) % 16 == 0, "the heavy set is copied in 16-byte units");

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
    float y = m.mean_y[leaf] + m.slope[leaf] * (x - m.mean_x[leaf]);
    y = fminf(fmaxf(y, m.lo[leaf]), m.hi[leaf]);
    uint32_t b = (uint32_t)(y * (float)P);
    return b < P ? b : P - 1;
}

__device__ __forceinline__ uint32_t heavy_slot(uint32_t key) { return slot_hash(key, kHeavySlotsLog2); }

// Build a heavy-key set from keys[0..n) (one CTA; ends with a barrier).
__device__ __forceinline__ void heavy_set_build(HeavySet &hs, const uint32_t *keys, uint32_t n) {
    for (uint32_t i = threadIdx.x; i < kHeavySlots; i += blockDim.x) hs.slot[i] = kHeavyEmpty;
    SJBG_BARRIER();
    for (uint32_t h = threadIdx.x; h < n; h += blockDim.x) {
        const uint32_t key = keys[h];
        const unsigned long long e = ((unsigned long long)key << 32) | h;
        uint32_t s = heavy_slot(key);
        for (uint32_t p = 0; p < kHeavySlots; p++) {
            if (atomicCAS(&hs.slot[s], kHeavyEmpty, e) == kHeavyEmpty) break;
            s = (s + 1) & (kHeavySlots - 1);
        }
    }
    SJBG_BARRIER();
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
// At load <= 1/8 the first slot decides almost always, so it is read without
// a loop; only a collision walks on.
__device__ __forceinline__ uint32_t heavy_find(const HeavySet &hs, uint32_t key) {
    uint32_t s = heavy_slot(key);
    unsigned long long v = hs.slot[s];
    if (v == kHeavyEmpty) return kHeavyBucket;
    if ((uint32_t)(v >> 32) == key) return (uint32_t)v;
    for (uint32_t p = 1; p < kHeavySlots; p++) {
        s = (s + 1) & (kHeavySlots - 1);
        v = hs.slot[s];
        if (v == kHeavyEmpty) return kHeavyBucket;
        if ((uint32_t)(v >> 32) == key) return (uint32_t)v;
    }
    return kHeavyBucket;
}

}  // namespace sjbg

struct sjbg_handle;
namespace sjbg {
struct WinPlan;
uint32_t learned_log2_buckets(sjbg_handle *h, uint64_t n_left);
// Sample, fit and check every window's model; writes models and sets
// WinPlan::model on device (dPlan) for the windows that keep their model.
// allow_heavy = false keeps every key in the partitions (needed when pairs are enumerated).
int learned_prepare(sjbg_handle *h, const sjbg_tuple *dL, const sjbg_tuple *dR, const WinPlan *plan, uint32_t n,
                    WinPlan *dPlan, const LearnedModel **dModels, bool allow_heavy);
}  // namespace sjbg
