// smj.cu - lazy sort-merge join (sm_103a).
//
// Replaces the reference's lazy GPU sort-merge family
// (src/sjb/windowing/lazy/executor/GPU/GPU_SMJ.cu:9-243 and its NoOutput /
// CountKernel / EstimatedSelectivity / Atomic variants), whose matching rule
// is the lazy CPU_SMJ's (src/sjb/windowing/lazy/executor/CPU/CPU_SMJ.cpp:23-139):
// both sides sorted by key, then every key group's cartesian product.
//
// Steps for a batch of windows (left sides are segments [0, n), right sides
// [n, 2n) of one segmented sort):
//   1. sort_extract + radix_sort_segments (sort.cu): stable LSD sort of
//      (key, val) for every window side;
//   2. segmented_fr_prefix: F[i] = sum of fr(val) over the first i sorted left
//      tuples, so any left key group's checksum sum is F[hi] - F[lo];
//   3. merge-path co-ranking: the merged order of a window's sorted left (A)
//      and right (B) keys, ties A first, is cut into tiles of kMergeTile
//      elements; one thread per cut binary-searches its co-rank i
//      (A elements before the cut), so tiles are equal work however skewed;
//   4. merge join: per tile the A keys [i0, i1) are staged in shared memory;
//      each B element j of [j0, j1) finds hi = #A <= key inside the tile and
//      lo = #A < key (in the tile, or by a global search when its key group
//      starts before the tile): count += hi - lo, prod += gs * (F[hi] - F[lo]);
//      when enumerating, the pairs (A[lo..hi), j) feed the xor checksum and
//      the pair output (one atomic reservation per warp).
#include <algorithm>
#include <cstring>
#include <vector>

#include "sort.cuh"

namespace sjbg {

constexpr uint32_t kMergeTile = 4096;   // merged elements per tile
constexpr int kMergeThreads = 256;

struct MergeWin {
    uint64_t a_off, b_off;   // sorted segments in the SoA arrays
    uint32_t na, nb;
    uint32_t cut0;           // first co-rank slot of this window
    uint32_t tile0;          // first merge tile of this window
    uint32_t ntiles;
    uint32_t pad;
    uint64_t pairs_off, pairs_cap;
};

__device__ __forceinline__ uint32_t find_merge_win(const MergeWin *w, uint32_t n, uint32_t tile) {
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (w[mid].tile0 <= tile) lo = mid; else hi = mid;
    }
    return lo;
}

// co-rank of diagonal d: number of A elements among the first d merged ones
__device__ __forceinline__ uint32_t corank(const uint32_t *A, uint32_t na, const uint32_t *B, uint32_t nb, uint32_t d) {
    uint32_t lo = d > nb ? d - nb : 0, hi = min(d, na);
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;   // A[mid] goes first iff A[mid] <= B[d - mid - 1]
        if (A[mid] <= B[d - mid - 1]) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// One thread per cut (all windows): cuts[cut0 + t] = co-rank of diagonal t * kMergeTile (clamped).
__global__ void merge_corank_kernel(const SortView *__restrict__ view, const MergeWin *__restrict__ wins, uint32_t nwin,
                                    uint32_t total_cuts, uint32_t *__restrict__ cuts) {
    const uint32_t *__restrict__ keys = view->keys;
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= total_cuts) return;
    uint32_t lo = 0, hi = nwin;   // window owning cut c: largest w with cut0 <= c
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (wins[mid].cut0 <= c) lo = mid; else hi = mid;
    }
    const MergeWin mw = wins[lo];
    const uint32_t t = c - mw.cut0;
    const uint64_t d64 = (uint64_t)t * kMergeTile;
    const uint64_t tot = (uint64_t)mw.na + mw.nb;
    const uint32_t d = (uint32_t)(d64 < tot ? d64 : tot);
    cuts[c] = corank(keys + mw.a_off, mw.na, keys + mw.b_off, mw.nb, d);
}

template <bool kEnum, bool kPairs>
__global__ void __launch_bounds__(kMergeThreads)
merge_join_kernel(const SortView *__restrict__ view, const unsigned long long *__restrict__ F,
                  const MergeWin *__restrict__ wins, uint32_t nwin, const uint32_t *__restrict__ cuts,
                  WinAcc *__restrict__ acc, sjbg_pair *__restrict__ pairs) {
    const uint32_t *__restrict__ keys = view->keys;
    const uint32_t *__restrict__ vals = view->vals;
    __shared__ uint32_t sa[kMergeTile];
    const uint32_t w = find_merge_win(wins, nwin, blockIdx.x);
    const MergeWin mw = wins[w];
    const uint32_t t = blockIdx.x - mw.tile0;
    const uint32_t total = mw.na + mw.nb;
    const uint32_t d0 = t * kMergeTile, d1 = min(total, d0 + kMergeTile);
    const uint32_t i0 = cuts[mw.cut0 + t], i1 = cuts[mw.cut0 + t + 1];
    const uint32_t j0 = d0 - i0, j1 = d1 - i1;
    const uint32_t *A = keys + mw.a_off;
    const uint32_t *Av = vals + mw.a_off;
    const uint32_t *B = keys + mw.b_off;
    const uint32_t *Bv = vals + mw.b_off;
    const unsigned long long *Fa = F + mw.a_off;
    const uint32_t m = i1 - i0;
    for (uint32_t i = threadIdx.x; i < m; i += kMergeThreads) sa[i] = A[i0 + i];
    SJBG_BARRIER();
    const uint64_t pcap = kPairs ? mw.pairs_cap : 0;
    sjbg_pair *pout = kPairs ? pairs + mw.pairs_off : nullptr;

    unsigned long long count = 0, prod = 0, xr = 0;
    // the next B element's key and val are loaded while this one is searched
    uint32_t nkey = 0, nval = 0;
    if (j0 + threadIdx.x < j1) {
        nkey = B[j0 + threadIdx.x];
        nval = Bv[j0 + threadIdx.x];
    }
    for (uint32_t jb = j0; jb < j1; jb += kMergeThreads) {   // uniform trip count (warp collectives below)
        const uint32_t j = jb + threadIdx.x;
        uint32_t lo = 0, hi = 0, bval = 0;
        const uint32_t ckey = nkey, cval = nval;
        if (j + kMergeThreads < j1) {
            nkey = B[j + kMergeThreads];
            nval = Bv[j + kMergeThreads];
        }
        if (j < j1) {
            const uint32_t key = ckey;
            bval = cval;
            // hi: first A position in the tile with A > key
            uint32_t l = 0, r = m;
            while (l < r) {
                const uint32_t mid = (l + r) >> 1;
                if (sa[mid] <= key) l = mid + 1; else r = mid;
            }
            hi = i0 + l;
            // the A element just before hi (in the tile, or the last one before it)
            const bool match = l > 0 ? sa[l - 1] == key : (i0 > 0 && A[i0 - 1] == key);
            if (!match) {
                lo = hi;
            } else if (l > 0 && sa[0] < key) {   // the key group starts inside the tile
                uint32_t l2 = 0, r2 = l;
                while (l2 < r2) {
                    const uint32_t mid = (l2 + r2) >> 1;
                    if (sa[mid] < key) l2 = mid + 1; else r2 = mid;
                }
                lo = i0 + l2;
            } else {   // it starts at or before the tile: first A >= key in A[0, i0]
                uint32_t l3 = 0, r3 = i0;
                while (l3 < r3) {
                    const uint32_t mid = (l3 + r3) >> 1;
                    if (A[mid] < key) l3 = mid + 1; else r3 = mid;
                }
                lo = l3;
            }
            count += hi - lo;
            if (hi > lo) prod += (Fa[hi] - Fa[lo]) * sjbg_gs(bval);   // (no prefix loads without a match)
            if (kEnum)
                for (uint32_t a = lo; a < hi; a++) xr ^= sjbg_pair_hash(Av[a], bval);
        }
        if (kPairs) {
            const uint32_t mine = hi - lo;
            uint32_t tot;
            const uint32_t ex = warp_excl_scan(mine, &tot);
            unsigned long long base = 0;
            if (lane_id() == 0 && tot) base = atomicAdd(&acc[w].npairs, (unsigned long long)tot);
            base = __shfl_sync(0xFFFFFFFFu, base, 0) + ex;
            for (uint32_t a = lo; a < hi; a++, base++)
                if (base < pcap) pout[base] = sjbg_pair{Av[a], bval};
        }
    }
    flush_acc(&acc[w], count, xr, prod);
}

int smj_lazy_batch(sjbg_handle *h, const sjbg_tuple *dL, const sjbg_tuple *dR, const WinHost *wins, uint32_t n,
                   sjbg_pair *dPairs, WinAcc *acc, bool enumerate) {
    if (n == 0) return SJBG_OK;
    std::vector<uint64_t> lens(2 * n), srcs(2 * n);
    for (uint32_t w = 0; w < n; w++) {
        if (wins[w].n_left >= 0x7FFFFFFFull || wins[w].n_right >= 0x7FFFFFFFull ||
            wins[w].n_left + wins[w].n_right >= 0xFFFFFFFFull)
            return fail(h, SJBG_E_CAPACITY, "sort-merge windows are limited to 2^31 tuples per side");
        lens[w] = wins[w].n_left;
        srcs[w] = wins[w].left_off;
        lens[n + w] = wins[w].n_right;
        srcs[n + w] = wins[w].right_off;
    }
    SortPlan plan = sort_plan(lens.data(), srcs.data(), 2 * n);
    std::vector<MergeWin> mw(n);
    uint32_t cuts = 0, tiles = 0;
    for (uint32_t w = 0; w < n; w++) {
        MergeWin &m = mw[w];
        std::memset(&m, 0, sizeof(m));
        m.a_off = plan.segs[w].off;
        m.b_off = plan.segs[n + w].off;
        m.na = (uint32_t)wins[w].n_left;
        m.nb = (uint32_t)wins[w].n_right;
        m.pairs_off = wins[w].pairs_off;
        m.pairs_cap = dPairs ? wins[w].pairs_cap : 0;
        const uint64_t total = (uint64_t)m.na + m.nb;
        m.ntiles = (m.na && m.nb) ? (uint32_t)((total + kMergeTile - 1) / kMergeTile) : 0;
        m.cut0 = cuts;
        m.tile0 = tiles;
        cuts += m.ntiles + 1;
        tiles += m.ntiles;
    }
    const size_t segB = sizeof(SortSeg) * plan.segs.size(), mwB = sizeof(MergeWin) * n;
    uint8_t *hst = static_cast<uint8_t *>(pinned_get(h, 0, segB + mwB));
    uint8_t *dev = static_cast<uint8_t *>(ws_get(h, WS_WIN_PLAN, segB + mwB));
    uint32_t *k0 = static_cast<uint32_t *>(ws_get(h, WS_SORT_K0, sizeof(uint32_t) * plan.elems));
    uint32_t *v0 = static_cast<uint32_t *>(ws_get(h, WS_SORT_V0, sizeof(uint32_t) * plan.elems));
    uint32_t *k1 = static_cast<uint32_t *>(ws_get(h, WS_SORT_K1, sizeof(uint32_t) * plan.elems));
    uint32_t *v1 = static_cast<uint32_t *>(ws_get(h, WS_SORT_V1, sizeof(uint32_t) * plan.elems));
    unsigned long long *F = static_cast<unsigned long long *>(ws_get(h, WS_PART_LEFT, sizeof(unsigned long long) * plan.elems));
    uint32_t *dCuts = static_cast<uint32_t *>(ws_get(h, WS_BUCKET_START, sizeof(uint32_t) * std::max(cuts, 1u)));
    if (!hst || !dev || !k0 || !v0 || !k1 || !v1 || !F || !dCuts) return fail(h, SJBG_E_NOMEM, "sort-merge buffers");
    std::memcpy(hst, plan.segs.data(), segB);
    std::memcpy(hst + segB, mw.data(), mwB);
    if (int rc_up = stage_copy(h, dev, hst, segB + mwB)) return rc_up;
    const SortSeg *dSegs = reinterpret_cast<const SortSeg *>(dev);
    const MergeWin *dMw = reinterpret_cast<const MergeWin *>(dev + segB);
    if (int rc_map = sort_tile_map(h, plan, dSegs)) return rc_map;

    const SortView *view = nullptr;
    uint32_t *kmax = nullptr;
    int rc = sort_key_max(h, &kmax);
    if (!rc) rc = sort_extract(h, dL, dR, n, plan, dSegs, k0, v0, kmax);
    if (!rc)
        rc = radix_sort_segments(h, plan, dSegs, k0, v0, k1, v1, reinterpret_cast<uint32_t *>(&acc[n].info), &view,
                                 kmax);
    if (!rc) rc = segmented_fr_prefix(h, plan, n, dSegs, view, F);
    if (rc) return rc;
    if (tiles == 0) return SJBG_OK;
    SJBG_CK(h, launch(h, "merge_corank", merge_corank_kernel, dim3((cuts + 255) / 256), dim3(256), 0,
                      view, dMw, n, cuts, dCuts));
    if (dPairs)
        SJBG_CK(h, launch(h, "merge_join_pairs", merge_join_kernel<true, true>, dim3(tiles), dim3(kMergeThreads), 0,
                          view, (const unsigned long long *)F, dMw, n,
                          (const uint32_t *)dCuts, acc, dPairs));
    else if (enumerate)
        SJBG_CK(h, launch(h, "merge_join_xor", merge_join_kernel<true, false>, dim3(tiles), dim3(kMergeThreads), 0,
                          view, (const unsigned long long *)F, dMw, n,
                          (const uint32_t *)dCuts, acc, dPairs));
    else
        SJBG_CK(h, launch(h, "merge_join_count", merge_join_kernel<false, false>, dim3(tiles), dim3(kMergeThreads), 0,
                          view, (const unsigned long long *)F, dMw, n,
                          (const uint32_t *)dCuts, acc, dPairs));
    return SJBG_OK;
}

}  // namespace sjbg
