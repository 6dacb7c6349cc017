// eager_run.cu - a whole recorded eager stream in a few launches (sm_103a).
//
// sjbg_eager_run receives every batch of both streams at once, so it does not
// have to replay the stream batch by batch.  Its results are those of the
// per-batch executors (eager.cu) fed as the reference feeds them - L0, R0,
// L1, R1, ... (src/sjb/source/Source.cpp:20-28), a window closed before a
// batch once either side holds window_size tuples
// (include/sjb/windowing/eager/CountBased.cuh:38-46) - because those are
// fixed by the data alone:
//   * a window's totals (count, xor, prod) are the join of all its tuples;
//   * a batch's count is the number of pairs it forms with the other side's
//     tuples that arrived earlier in the same window.  Batch i of the left
//     stream arrives at position 2i, batch j of the right at 2j + 1, so the
//     pair of left batch i and right batch j is counted by left batch i when
//     i > j and by right batch j otherwise.
// Nested-loop join: every (left batch, right batch) block pair of a window is
// compared by one grid of register-blocked CTAs (nlj.cu's block routine); a
// block pair adds its matches to the later batch's count and its checksums to
// the window.
// Hash and sort-merge joins: the window totals come from the lazy join of the
// windows (hj.cu / smj.cu), and the batch counts from one stable sort per
// window: the window's (key, batch tag) pairs in arrival order are sorted by
// key (sort.cu), so each key group lists its tuples in arrival order and a
// tuple's count is the number of other-side tuples before it in its group,
// which prefix counts over the sorted window give directly.
#include <algorithm>
#include <cstring>
#include <vector>

#include "eager.cuh"
#include "sort.cuh"

namespace sjbg {

// ---------------------------------------------------------------- sort-based batch counts
constexpr uint32_t kAttrThreads = 256;
constexpr uint32_t kAttrPer = kSortTile / kAttrThreads;   // 16
constexpr uint32_t kTagSmem = 4096;                       // batch counters kept in shared memory
// dynamic shared memory of eattr_kernel: keys, right prefix, group starts, batch counters
constexpr size_t kAttrSmem = 3 * sizeof(uint32_t) * kSortTile + sizeof(unsigned long long) * kTagSmem;

// Per window: the batch-counter range its tags fall in.
struct ESegMeta {
    uint32_t tag_lo, tag_n;
};

// One copy item: batch `batch` of side `side` -> positions [dst, dst + B) of the window's segment.
struct EGather {
    uint64_t dst;
    uint32_t batch, side;
};

__global__ void __launch_bounds__(256)
egather_kernel(const sjbg_tuple *__restrict__ L, const sjbg_tuple *__restrict__ R, const EGather *__restrict__ items,
               uint32_t B, uint32_t *__restrict__ keys, uint32_t *__restrict__ tags) {
    const EGather it = items[blockIdx.x];
    const sjbg_tuple *src = (it.side ? R : L) + (uint64_t)it.batch * B;
    const uint32_t tag = 2u * it.batch + it.side;
    for (uint32_t i = threadIdx.x; i < B; i += blockDim.x) {
        keys[it.dst + i] = __ldg(reinterpret_cast<const uint32_t *>(src + i));
        tags[it.dst + i] = tag;
    }
}

// Right-side tuples per sort tile.
__global__ void __launch_bounds__(256)
etile_count_kernel(const SortView *__restrict__ view, const SortSeg *__restrict__ segs,
                   const uint32_t *__restrict__ tile_seg, uint32_t *__restrict__ tcount) {
    const uint32_t *__restrict__ tags = view->vals;
    const uint32_t s = find_seg(tile_seg, blockIdx.x);
    const SortSeg sg = segs[s];
    const uint32_t base = (blockIdx.x - sg.tile0) * kSortTile;
    uint32_t c = 0;
    for (uint32_t i = threadIdx.x; i < kSortTile; i += blockDim.x)
        if (base + i < sg.n) c += tags[sg.off + base + i] & 1u;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xFFFFFFFFu, c, o);
    __shared__ uint32_t part[8];
    if (lane_id() == 0) part[warp_id()] = c;
    SJBG_BARRIER();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (uint32_t q = 0; q < blockDim.x / 32; q++) t += part[q];
        tcount[blockIdx.x] = t;
    }
}

// One warp per segment: exclusive scan of its tiles' right counts.
__global__ void etile_scan_kernel(const SortSeg *__restrict__ segs, uint32_t nseg, const uint32_t *__restrict__ tcount,
                                  uint32_t *__restrict__ tpre) {
    const uint32_t s = blockIdx.x;
    if (s >= nseg) return;
    const SortSeg sg = segs[s];
    uint32_t carry = 0;
    for (uint32_t t0 = 0; t0 < sg.ntiles; t0 += 32) {
        const uint32_t t = t0 + lane_id();
        const uint32_t v = t < sg.ntiles ? tcount[sg.tile0 + t] : 0u;
        uint32_t tot;
        const uint32_t ex = warp_excl_scan(v, &tot);
        if (t < sg.ntiles) tpre[sg.tile0 + t] = carry + ex;
        carry += tot;
    }
}

// Number of right-side tuples at segment positions [0, p): the tile prefix plus
// the right tuples of p's tile before p (one warp counts them).
__device__ __forceinline__ uint32_t eright_before_warp(const uint32_t *tags, const SortSeg &sg, const uint32_t *tpre,
                                                       uint32_t p) {
    const uint32_t t = p / kSortTile, t0 = t * kSortTile;
    uint32_t c = 0;
    for (uint32_t i = t0 + lane_id(); i < p; i += 32) c += tags[sg.off + i] & 1u;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xFFFFFFFFu, c, o);
    return tpre[sg.tile0 + t] + c;
}

// Per sort tile: each tuple's count = other-side tuples before it in its key
// group, summed into its batch's counter.
__global__ void __launch_bounds__(kAttrThreads)
eattr_kernel(const SortView *__restrict__ view, const SortSeg *__restrict__ segs,
             const uint32_t *__restrict__ tile_seg, const ESegMeta *__restrict__ meta, const uint32_t *__restrict__ tpre,
             unsigned long long *__restrict__ counts) {
    extern __shared__ __align__(16) uint8_t attr_smem[];
    unsigned long long *tc = reinterpret_cast<unsigned long long *>(attr_smem);   // kTagSmem batch counters
    uint32_t *sk = reinterpret_cast<uint32_t *>(tc + kTagSmem);                   // the tile's keys
    uint32_t *rloc = sk + kSortTile;        // right tuples before each position inside the tile
    int32_t *gst = reinterpret_cast<int32_t *>(rloc + kSortTile);                  // group start inside the tile, or -1
    __shared__ uint32_t warp_tot[kAttrThreads / 32];
    __shared__ uint32_t g0_s, r0_s;
    const uint32_t *__restrict__ keys = view->keys;   // the sorted keys and their tags
    const uint32_t *__restrict__ tags = view->vals;
    const uint32_t s = find_seg(tile_seg, blockIdx.x);
    const SortSeg sg = segs[s];
    const ESegMeta m = meta[s];
    const uint32_t base = (blockIdx.x - sg.tile0) * kSortTile;
    if (base >= sg.n) return;   // whole CTA
    const uint32_t n = min(kSortTile, sg.n - base);
    const bool smem_tags = m.tag_n <= kTagSmem;
    if (smem_tags)
        for (uint32_t i = threadIdx.x; i < m.tag_n; i += blockDim.x) tc[i] = 0;
    // thread t owns positions [t * kAttrPer, (t + 1) * kAttrPer) of the tile
    const uint32_t p0 = threadIdx.x * kAttrPer;
    uint32_t myr = 0, tg[kAttrPer];
#pragma unroll
    for (int q = 0; q < (int)kAttrPer; q++) {
        const uint32_t p = p0 + q;
        const bool valid = p < n;
        const uint32_t k = valid ? keys[sg.off + base + p] : 0xFFFFFFFFu;
        tg[q] = valid ? tags[sg.off + base + p] : 0u;
        sk[p] = k;
        myr += valid ? (tg[q] & 1u) : 0u;
    }
    uint32_t tot;
    const uint32_t ex = warp_excl_scan(myr, &tot);
    if (lane_id() == 31) warp_tot[warp_id()] = ex + myr;
    SJBG_BARRIER();
    if (warp_id() == 0) {
        const uint32_t x = lane_id() < blockDim.x / 32 ? warp_tot[lane_id()] : 0u;
        uint32_t tt;
        const uint32_t e = warp_excl_scan(x, &tt);   // all 32 lanes
        if (lane_id() < blockDim.x / 32) warp_tot[lane_id()] = e;
    }
    SJBG_BARRIER();
    uint32_t run = warp_tot[warp_id()] + ex;
    int32_t last = -1;
#pragma unroll
    for (int q = 0; q < (int)kAttrPer; q++) {
        const uint32_t p = p0 + q;
        rloc[p] = run;
        run += (p < n) ? (tg[q] & 1u) : 0u;
        // a group starts at p when the previous position (this tile or the one before) holds another key
        const uint32_t prevk = p ? sk[p - 1] : (base ? keys[sg.off + base - 1] : ~sk[0]);
        const bool head = p < n && (base + p == 0 || prevk != sk[p]);
        if (head) last = (int32_t)p;
        gst[p] = last;   // partial: only this thread's run so far
    }
    // block-wide max-scan of group starts: carry the last start of earlier threads
    {
        int32_t mine = last, incl = mine;
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane_id() >= (uint32_t)o) incl = max(incl, y);
        }
        __shared__ int32_t wmax[kAttrThreads / 32];
        if (lane_id() == 31) wmax[warp_id()] = incl;
        SJBG_BARRIER();
        int32_t carry = -1;
        for (uint32_t q = 0; q < warp_id(); q++) carry = max(carry, wmax[q]);
        int32_t before = __shfl_up_sync(0xFFFFFFFFu, incl, 1);
        if (lane_id() == 0) before = -1;
        before = max(before, carry);
#pragma unroll
        for (int q = 0; q < (int)kAttrPer; q++) {
            const uint32_t p = p0 + q;
            if (gst[p] < 0) gst[p] = before;
        }
    }
    // the tile's first group may have started in an earlier tile: find its start
    if (threadIdx.x == 0) g0_s = 0xFFFFFFFFu;
    SJBG_BARRIER();
    if (warp_id() == 0 && gst[0] < 0) {
        const uint32_t k0 = sk[0];
        uint32_t lo = 0, hi = base;   // first position in [0, base] whose key is >= k0
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (keys[sg.off + mid] < k0) lo = mid + 1; else hi = mid;
        }
        const uint32_t r = eright_before_warp(tags, sg, tpre, lo);
        if (lane_id() == 0) { g0_s = lo; r0_s = r; }
    }
    SJBG_BARRIER();
    const uint32_t tile_r = tpre[blockIdx.x];
#pragma unroll
    for (int q = 0; q < (int)kAttrPer; q++) {
        const uint32_t p = p0 + q;
        if (p >= n) break;
        const uint32_t gp = base + p;   // segment position
        uint32_t gs, rg;
        if (gst[p] >= 0) {
            gs = base + (uint32_t)gst[p];
            rg = tile_r + rloc[gst[p]];
        } else {
            gs = g0_s;
            rg = r0_s;
        }
        const uint32_t r_before = tile_r + rloc[p] - rg;            // right tuples before p in its group
        const uint32_t l_before = (gp - gs) - r_before;              // left tuples before p in its group
        const uint32_t c = (tg[q] & 1u) ? l_before : r_before;
        if (!c) continue;
        if (smem_tags) atomicAdd(&tc[tg[q] - m.tag_lo], (unsigned long long)c);
        else atomicAdd(&counts[tg[q]], (unsigned long long)c);
    }
    if (smem_tags) {
        SJBG_BARRIER();
        for (uint32_t i = threadIdx.x; i < m.tag_n; i += blockDim.x)
            if (tc[i]) atomicAdd(&counts[m.tag_lo + i], tc[i]);
    }
}

struct ERunWin {
    uint64_t l0, l1, r0, r1;   // batch ranges [l0, l1) and [r0, r1)
};

// Windows of the recorded stream under the reference's close rule.
static std::vector<ERunWin> erun_windows(uint64_t n_batches, uint64_t B, uint64_t W) {
    std::vector<ERunWin> wins;
    ERunWin cur{0, 0, 0, 0};
    uint64_t tot[2] = {0, 0};
    bool open = false;
    for (uint64_t b = 0; b < n_batches; b++) {
        for (int side = 0; side < 2; side++) {
            if (tot[0] >= W || tot[1] >= W) {
                wins.push_back(cur);
                tot[0] = tot[1] = 0;
                open = false;
            }
            if (!open) {
                cur = ERunWin{b + (side == 1 ? 1 : 0), b + (side == 1 ? 1 : 0), b, b};
                open = true;
            }
            if (side == 0) cur.l1 = b + 1;
            else cur.r1 = b + 1;
            tot[side] += B;
        }
    }
    if (open) wins.push_back(cur);
    return wins;
}

int hj_lazy_batch(sjbg_handle *h, const sjbg_tuple *dL, const sjbg_tuple *dR, const WinHost *wins, uint32_t n,
                  sjbg_pair *dPairs, WinAcc *acc, bool enumerate, uint32_t *part_used);

// Whole recorded stream; dCounts (2 * n_batches) and dWin (one entry per
// window, then the status word) are device arrays zeroed here.  Returns the
// number of windows in *n_windows.
int eager_run_batched(sjbg_handle *h, const sjbg_tuple *dl, const sjbg_tuple *dr, uint64_t n_batches, bool enumerate,
                      unsigned long long *dCounts, WinAcc *dWin, uint32_t *n_windows) {
    const uint64_t B = h->cfg.batch_size, W = h->cfg.window_size;
    const std::vector<ERunWin> ew = erun_windows(n_batches, B, W);
    const uint32_t nw = (uint32_t)ew.size();
    *n_windows = nw;
    SJBG_CK(h, cudaMemsetAsync(dCounts, 0, 8 * std::max<uint64_t>(2 * n_batches, 1), h->stream));
    SJBG_CK(h, cudaMemsetAsync(dWin, 0, sizeof(WinAcc) * (nw + 1), h->stream));
    if (nw == 0) return SJBG_OK;
    if (B * n_batches >= 0x7FFFFFFFull) return fail(h, SJBG_E_CAPACITY, "eager streams are limited to 2^31 tuples");

    if (h->cfg.algorithm == SJBG_ALG_NLJ) {
        const uint32_t lt = nlj_left_tile();
        std::vector<ERunItem> items;
        for (uint32_t w = 0; w < nw; w++)
            for (uint64_t i = ew[w].l0; i < ew[w].l1; i++)
                for (uint64_t j = ew[w].r0; j < ew[w].r1; j++) {
                    const uint32_t dest = i > j ? (uint32_t)(2 * i) : (uint32_t)(2 * j + 1);
                    for (uint64_t l0 = 0; l0 < B; l0 += lt)
                        items.push_back(ERunItem{w, (uint32_t)i, (uint32_t)j, dest, (uint32_t)l0, {0, 0, 0}});
                }
        return eager_nlj_blocks(h, dl, dr, B, items.data(), (uint32_t)items.size(), dWin, dCounts, enumerate);
    }

    // ---- window totals: the lazy join of each window's tuples
    std::vector<WinHost> wh(nw);
    for (uint32_t w = 0; w < nw; w++)
        wh[w] = WinHost{ew[w].l0 * B, (ew[w].l1 - ew[w].l0) * B, ew[w].r0 * B, (ew[w].r1 - ew[w].r0) * B, 0, 0};

    // ---- batch counts: one segment per window, its batches in arrival order
    std::vector<uint64_t> lens(nw), srcs(nw, 0);
    for (uint32_t w = 0; w < nw; w++) lens[w] = wh[w].n_left + wh[w].n_right;
    SortPlan plan = sort_plan(lens.data(), srcs.data(), nw);
    std::vector<ESegMeta> meta(nw);
    std::vector<EGather> gat;
    for (uint32_t w = 0; w < nw; w++) {
        const ERunWin &x = ew[w];
        const uint64_t lo = std::min(x.l0, x.r0), hi = std::max(x.l1, x.r1);
        meta[w] = ESegMeta{(uint32_t)(2 * lo), (uint32_t)(2 * (hi - lo))};
        uint64_t pos = plan.segs[w].off;
        for (uint64_t b = lo; b < hi; b++) {   // arrival order: left batch b, then right batch b
            if (b >= x.l0 && b < x.l1) { gat.push_back(EGather{pos, (uint32_t)b, 0}); pos += B; }
            if (b >= x.r0 && b < x.r1) { gat.push_back(EGather{pos, (uint32_t)b, 1}); pos += B; }
        }
    }
    const size_t segB = sizeof(SortSeg) * nw, metaB = sizeof(ESegMeta) * nw, gatB = sizeof(EGather) * gat.size();
    const size_t upB = segB + metaB + gatB;
    uint8_t *hst = static_cast<uint8_t *>(pinned_get(h, 2, upB));
    uint8_t *dev = static_cast<uint8_t *>(ws_get(h, WS_EAGER_META, upB + 16));
    uint32_t *k0 = static_cast<uint32_t *>(ws_get(h, WS_EAGER_K0, sizeof(uint32_t) * plan.elems));
    uint32_t *t0 = static_cast<uint32_t *>(ws_get(h, WS_EAGER_V0, sizeof(uint32_t) * plan.elems));
    uint32_t *k1 = static_cast<uint32_t *>(ws_get(h, WS_EAGER_K1, sizeof(uint32_t) * plan.elems));
    uint32_t *t1 = static_cast<uint32_t *>(ws_get(h, WS_EAGER_V1, sizeof(uint32_t) * plan.elems));
    uint32_t *tcnt = static_cast<uint32_t *>(ws_get(h, WS_EAGER_TILES, sizeof(uint32_t) * 2 * std::max(plan.tiles, 1u)));
    if (!hst || !dev || !k0 || !t0 || !k1 || !t1 || !tcnt) return fail(h, SJBG_E_NOMEM, "eager run buffers");
    std::memcpy(hst, plan.segs.data(), segB);
    std::memcpy(hst + segB, meta.data(), metaB);
    std::memcpy(hst + segB + metaB, gat.data(), gatB);
    if (int rc = stage_copy(h, dev, hst, upB)) return rc;
    const SortSeg *dSegs = reinterpret_cast<const SortSeg *>(dev);
    const ESegMeta *dMeta = reinterpret_cast<const ESegMeta *>(dev + segB);
    const EGather *dGat = reinterpret_cast<const EGather *>(dev + segB + metaB);
    if (int rc_map = sort_tile_map(h, plan, dSegs)) return rc_map;
    SJBG_CK(h, launch(h, "erun_gather", egather_kernel, dim3((uint32_t)gat.size()), dim3(256), 0, dl, dr, dGat,
                      (uint32_t)B, k0, t0));
    const SortView *view = nullptr;
    int rc = radix_sort_segments(h, plan, dSegs, k0, t0, k1, t1, reinterpret_cast<uint32_t *>(&dWin[nw].info), &view);
    if (rc) return rc;
    uint32_t *tpre = tcnt + std::max(plan.tiles, 1u);
    SJBG_CK(h, launch(h, "erun_tile_count", etile_count_kernel, dim3(plan.tiles), dim3(256), 0, view, dSegs,
                      plan.tile_seg, tcnt));
    SJBG_CK(h, launch(h, "erun_tile_scan", etile_scan_kernel, dim3(nw), dim3(32), 0, dSegs, nw,
                      (const uint32_t *)tcnt, tpre));
    allow_big_smem(eattr_kernel, kAttrSmem);
    SJBG_CK(h, launch(h, "erun_attribute", eattr_kernel, dim3(plan.tiles), dim3(kAttrThreads), kAttrSmem,
                      view, dSegs, plan.tile_seg, dMeta, (const uint32_t *)tpre, dCounts));

    uint32_t pu = 0;
    if (h->cfg.algorithm == SJBG_ALG_SMJ) return smj_lazy_batch(h, dl, dr, wh.data(), nw, nullptr, dWin, enumerate);
    return hj_lazy_batch(h, dl, dr, wh.data(), nw, nullptr, dWin, enumerate, &pu);
}

}  // namespace sjbg
