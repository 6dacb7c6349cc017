// sort.cuh - segmented LSD radix sort of (key, val) pairs and segmented scans
// (device building blocks of the sort-merge join).
#pragma once

#include <vector>

#include "runtime.h"

namespace sjbg {

constexpr uint32_t kSortTile = 4096;   // elements per sort tile (16 KB of keys)

// One segment (window side) of the SoA key/val arrays.  A segment occupies
// [off, off + round_up(n + 1, kSortTile)) so every tile is a whole 16 KB block
// and position off + n exists (the end of a prefix-sum array).
struct SortSeg {
    uint64_t off;     // first element (multiple of kSortTile)
    uint64_t src;     // first tuple of the segment in the AoS input
    uint32_t n;       // valid elements
    uint32_t tile0;   // first tile of this segment in the batch
    uint32_t ntiles;  // tiles of this segment
    uint32_t pad;
};

struct SortPlan {
    std::vector<SortSeg> segs;
    uint32_t tiles = 0;
    uint64_t elems = 0;   // padded total
    const uint32_t *tile_seg = nullptr;   // device: segment of every tile (sort_tile_map)
};

// Plan segments of lengths n[0..k) read from AoS offsets src[0..k): padded
// offsets and tile ranges.
SortPlan sort_plan(const uint64_t *n, const uint64_t *src, uint32_t k);

// *kmax = a device word zeroed on the stream, for the largest key of a sort's input.
int sort_key_max(sjbg_handle *h, uint32_t **kmax);

// Raise *out to the largest m of the calling CTA (at most 256 threads, all of
// them calling): one atomic per CTA, and only when it can raise the value seen
// (a stale read only costs an atomic: atomicMax decides).
__device__ __forceinline__ void block_key_max(uint32_t m, uint32_t *out) {
    __shared__ uint32_t wm[8];
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xFFFFFFFFu, m, o));
    if (lane_id() == 0) wm[warp_id()] = m;
    SJBG_BARRIER();
    if (threadIdx.x == 0) {
        for (uint32_t q = 1; q < blockDim.x / 32; q++) m = max(m, wm[q]);
        if (m > *(volatile const uint32_t *)out) atomicMax(out, m);
    }
}

// AoS tuples -> SoA keys/vals for every segment; segments [0, split) read
// srcA, the others srcB.  kmax (from sort_key_max, or null) receives the
// largest key.
int sort_extract(sjbg_handle *h, const sjbg_tuple *srcA, const sjbg_tuple *srcB, uint32_t split, const SortPlan &plan,
                 const SortSeg *dSegs, uint32_t *keys, uint32_t *vals, uint32_t *kmax);

// Writes the segment of every tile of the plan into a workspace array (one
// launch) and points plan.tile_seg at it: the per-tile kernels then find
// their segment with one load instead of a binary search over the segments.
int sort_tile_map(sjbg_handle *h, SortPlan &plan, const SortSeg *dSegs);

__device__ __forceinline__ uint32_t find_seg(const uint32_t *tile_seg, uint32_t tile) { return tile_seg[tile]; }

// Where a sort's result lies (device memory, written by the sort): the
// passes alternate between the two buffer pairs, and under graph capture only
// the device knows how many ran.
struct SortView {
    const uint32_t *keys;
    const uint32_t *vals;
};

// Stable LSD sort of every segment by key; keys/vals hold the input, and the
// result is in keys/vals or keys2/vals2 as *view (a device pointer) says.
// Four 8-bit passes are launched; each skips itself on the device when its
// digit is zero in every key (the largest key is found on the device), so the
// host never waits and the launches are the same under graph capture.
// status: a device word that receives kErrTimeout if a tile's bulk copy never lands.
// kmax: the largest key when the kernel that wrote keys found it (sort_key_max),
// or null, and the sort finds it with a pass of its own.
int radix_sort_segments(sjbg_handle *h, const SortPlan &plan, const SortSeg *dSegs, uint32_t *keys, uint32_t *vals,
                        uint32_t *keys2, uint32_t *vals2, uint32_t *status, const SortView **view,
                        uint32_t *kmax = nullptr);

// Exclusive prefix sums of fr(val) (u64, mod 2^64) of the first nseg
// segments into out (same padded layout; positions 0..n of each segment);
// vals are the sort's (view).
int segmented_fr_prefix(sjbg_handle *h, const SortPlan &plan, uint32_t nseg, const SortSeg *dSegs,
                        const SortView *view, unsigned long long *out);

}  // namespace sjbg
