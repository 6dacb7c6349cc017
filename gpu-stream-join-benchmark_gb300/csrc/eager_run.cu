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
// Hash and sort-merge joins: the batch counts come from one stable sort per
// window: the window's keys in arrival order are sorted (sort.cu) with each
// tuple's arrival position as payload, so each key group lists its tuples in
// arrival order and a tuple's count is the number of other-side tuples before
// it in its group, which a segmented scan over the sorted window gives.
// Sort-merge without pair enumeration takes the window totals from the same
// pass (count = the sum of those counts, prod = the same pairs weighted by
// fr * gs); otherwise they come from the lazy join of the windows (hj.cu /
// smj.cu).
#include <algorithm>
#include <cstring>
#include <vector>

#include "eager.cuh"
#include "sort.cuh"

namespace sjbg {

// ---------------------------------------------------------------- sort-based batch counts
constexpr uint32_t kAttrThreads = 256;
constexpr uint32_t kAttrPer = kSortTile / kAttrThreads;   // 16 consecutive positions per thread
constexpr uint32_t kTagSmem = 4096;                       // batch counters kept in shared memory

// Per window (one sort segment).
struct ESegMeta {
    uint32_t tag_lo, tag_n;   // the batch-counter range its tags fall in
    uint32_t first_tag;       // arrival tag (2 * batch + side) of the window's first batch
    uint32_t pad_;
};

// One copy item: batch `batch` of side `side` -> buffer positions [dst, dst + B),
// which are positions [rel, rel + B) of its window's segment.
struct EGather {
    uint64_t dst;
    uint32_t batch, side, rel, pad_;
};

// The sort's payload is a tuple's position in its window's arrival-ordered
// segment.  A window holds consecutive arrival tags (the close rule is checked
// before every batch, in arrival order), so the position names the tuple:
// tag = the window's first tag + position / B, index in the batch = position % B.
struct ETup {
    uint32_t tag, val;
};

__device__ __forceinline__ ETup etuple(uint32_t rel, uint32_t first_tag, const sjbg_tuple *__restrict__ L,
                                       const sjbg_tuple *__restrict__ R, uint32_t B, bool need_val) {
    const uint32_t slot = rel / B;
    const uint32_t tag = first_tag + slot;
    uint32_t v = 0;
    if (need_val) {
        const sjbg_tuple *src = (tag & 1u) ? R : L;
        v = __ldg(&src[(uint64_t)(tag >> 1) * B + (rel - slot * B)].val);
    }
    return ETup{tag, v};
}

__global__ void __launch_bounds__(256)
egather_kernel(const sjbg_tuple *__restrict__ L, const sjbg_tuple *__restrict__ R, const EGather *__restrict__ items,
               uint32_t B, uint32_t *__restrict__ keys, uint32_t *__restrict__ rels, uint32_t *__restrict__ kmax) {
    const EGather it = items[blockIdx.x];
    const sjbg_tuple *src = (it.side ? R : L) + (uint64_t)it.batch * B;
    uint32_t m = 0;
    for (uint32_t i = threadIdx.x; i < B; i += blockDim.x) {
        const uint32_t k = __ldg(reinterpret_cast<const uint32_t *>(src + i));
        keys[it.dst + i] = k;
        rels[it.dst + i] = it.rel + i;
        m = max(m, k);
    }
    block_key_max(m, kmax);   // the sort's key range
}

// Sums over a run of a window's sorted tuples: left and right tuples, and the
// sums of fr over the left ones and of gs over the right ones (the weights
// exist only when the window's totals are formed here, kW).
struct ESum {
    uint32_t nl, nr;
    unsigned long long wl, wr;
};

__device__ __forceinline__ ESum esum_zero() { return ESum{0u, 0u, 0ull, 0ull}; }

__device__ __forceinline__ void esum_add(ESum &a, const ESum &b) {
    a.nl += b.nl;
    a.nr += b.nr;
    a.wl += b.wl;
    a.wr += b.wr;
}

template <bool kW>
__device__ __forceinline__ void esum_item(ESum &a, const ETup &e) {
    if (e.tag & 1u) {
        a.nr++;
        if (kW) a.wr += sjbg_gs(e.val);
    } else {
        a.nl++;
        if (kW) a.wl += sjbg_fr(e.val);
    }
}

template <bool kW>
__device__ __forceinline__ ESum esum_shfl_up(const ESum &a, uint32_t o) {
    ESum y = esum_zero();
    y.nl = __shfl_up_sync(0xFFFFFFFFu, a.nl, o);
    y.nr = __shfl_up_sync(0xFFFFFFFFu, a.nr, o);
    if (kW) {
        y.wl = __shfl_up_sync(0xFFFFFFFFu, a.wl, o);
        y.wr = __shfl_up_sync(0xFFFFFFFFu, a.wr, o);
    }
    return y;
}

template <bool kW>
__device__ __forceinline__ ESum esum_warp_sum(ESum a) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a.nl += __shfl_xor_sync(0xFFFFFFFFu, a.nl, o);
        a.nr += __shfl_xor_sync(0xFFFFFFFFu, a.nr, o);
        if (kW) {
            a.wl += __shfl_xor_sync(0xFFFFFFFFu, a.wl, o);
            a.wr += __shfl_xor_sync(0xFFFFFFFFu, a.wr, o);
        }
    }
    return a;
}

// A sort tile's sums, then (in place) their exclusive prefix within the segment.
struct ETileSum {
    unsigned long long nl, nr, wl, wr;
};

template <bool kW>
__global__ void __launch_bounds__(256)
etile_sum_kernel(const SortView *__restrict__ view, const SortSeg *__restrict__ segs,
                 const uint32_t *__restrict__ tile_seg, const ESegMeta *__restrict__ meta,
                 const sjbg_tuple *__restrict__ L, const sjbg_tuple *__restrict__ R, uint32_t B,
                 ETileSum *__restrict__ tsum) {
    const uint32_t *__restrict__ rels = view->vals;
    const uint32_t s = find_seg(tile_seg, blockIdx.x);
    const SortSeg sg = segs[s];
    const uint32_t first = meta[s].first_tag;
    const uint32_t base = (blockIdx.x - sg.tile0) * kSortTile;
    // all 16 positions' loads first, then their gathers, then the sums
    constexpr uint32_t kPer = kSortTile / 256;
    uint32_t rl[kPer];
#pragma unroll
    for (uint32_t q = 0; q < kPer; q++) {
        const uint32_t i = base + threadIdx.x + q * 256;
        rl[q] = i < sg.n ? rels[sg.off + i] : 0u;
    }
    ETup e[kPer];
#pragma unroll
    for (uint32_t q = 0; q < kPer; q++) e[q] = etuple(rl[q], first, L, R, B, kW);
    ESum a = esum_zero();
#pragma unroll
    for (uint32_t q = 0; q < kPer; q++)
        if (base + threadIdx.x + q * 256 < sg.n) esum_item<kW>(a, e[q]);
    a = esum_warp_sum<kW>(a);
    __shared__ ESum part[8];
    if (lane_id() == 0) part[warp_id()] = a;
    SJBG_BARRIER();
    if (threadIdx.x == 0) {
        ESum t = esum_zero();
        for (uint32_t q = 0; q < blockDim.x / 32; q++) esum_add(t, part[q]);
        tsum[blockIdx.x] = ETileSum{t.nl, t.nr, t.wl, t.wr};
    }
}

// One warp per segment: its tiles' sums become their exclusive prefix.  Each
// lane sums a run of consecutive tiles (independent loads), the lane sums get
// a warp scan, and each lane writes its run's prefixes.
__global__ void etile_scan_kernel(const SortSeg *__restrict__ segs, uint32_t nseg, ETileSum *__restrict__ t) {
    const uint32_t s = blockIdx.x;
    if (s >= nseg) return;
    const SortSeg sg = segs[s];
    ETileSum *ts = t + sg.tile0;
    const uint32_t nt = sg.ntiles, per = (nt + 31) >> 5;
    const uint32_t a = min(nt, lane_id() * per), b = min(nt, a + per);
    unsigned long long x[4] = {0, 0, 0, 0};
    for (uint32_t i = a; i < b; i++) {
        const ETileSum v = ts[i];
        x[0] += v.nl;
        x[1] += v.nr;
        x[2] += v.wl;
        x[3] += v.wr;
    }
    unsigned long long run[4];
#pragma unroll
    for (int f = 0; f < 4; f++) {
        unsigned long long inc = x[f];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long u = __shfl_up_sync(0xFFFFFFFFu, inc, o);
            if (lane_id() >= (uint32_t)o) inc += u;
        }
        run[f] = inc - x[f];
    }
    for (uint32_t i = a; i < b; i++) {
        const ETileSum v = ts[i];
        ts[i] = ETileSum{run[0], run[1], run[2], run[3]};
        run[0] += v.nl;
        run[1] += v.nr;
        run[2] += v.wl;
        run[3] += v.wr;
    }
}

// Sums over the part of a tile's first key group that lies before the tile
// (zero when the tile starts a group).  Called by one whole warp.  The group
// start is looked for among the 32 positions before the tile first; a longer
// group is found by binary search and summed from the tile prefix of the tile
// it starts in, counting from the nearer end of that tile.
template <bool kW>
__device__ ESum efirst_group_carry(const uint32_t *__restrict__ keys, const uint32_t *__restrict__ rels,
                                   const SortSeg &sg, uint32_t first_tag, const ETileSum *__restrict__ tpre,
                                   uint32_t tile, uint32_t base, const sjbg_tuple *__restrict__ L,
                                   const sjbg_tuple *__restrict__ R, uint32_t B) {
    ESum c = esum_zero();
    if (base == 0) return c;
    const uint32_t *__restrict__ ks = keys + sg.off;
    const uint32_t *__restrict__ rs = rels + sg.off;
    const uint32_t k0 = ks[base];
    if (ks[base - 1] != k0) return c;
    const uint32_t lane = lane_id();
    const bool in = lane < base && ks[base - 1 - lane] == k0;
    const uint32_t out = __ballot_sync(0xFFFFFFFFu, !in);
    if (out) {
        const uint32_t len = __ffs(out) - 1;   // group positions before the tile
        if (lane < len) esum_item<kW>(c, etuple(rs[base - 1 - lane], first_tag, L, R, B, kW));
        return esum_warp_sum<kW>(c);
    }
    uint32_t lo = 0, hi = base - 32;   // first position whose key is >= k0
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (ks[mid] < k0) lo = mid + 1; else hi = mid;
    }
    const uint32_t g0 = lo, t0 = g0 / kSortTile, a0 = t0 * kSortTile;
    const bool fwd = g0 - a0 <= a0 + kSortTile - g0;
    const uint32_t i0 = fwd ? a0 : g0, i1 = fwd ? g0 : a0 + kSortTile;   // inside tile t0, all valid
    ESum part = esum_zero();
    for (uint32_t i = i0 + lane; i < i1; i += 32) esum_item<kW>(part, etuple(rs[i], first_tag, L, R, B, kW));
    part = esum_warp_sum<kW>(part);
    const ETileSum at = tpre[sg.tile0 + t0 + (fwd ? 0u : 1u)];   // sums before tile t0 (or t0 + 1 <= this tile)
    const ETileSum cur = tpre[tile];                              // sums before this tile
    // group part before the tile = S(base) - S(g0), S(g0) = at + part (forward) or at - part
    c.nl = (uint32_t)(cur.nl - at.nl);
    c.nr = (uint32_t)(cur.nr - at.nr);
    c.wl = cur.wl - at.wl;
    c.wr = cur.wr - at.wr;
    if (fwd) {
        c.nl -= part.nl;
        c.nr -= part.nr;
        c.wl -= part.wl;
        c.wr -= part.wr;
    } else {
        esum_add(c, part);
    }
    return c;
}

// Per sort tile: each tuple's count = other-side tuples before it in its key
// group, summed into its batch's counter.  Running sums over the key groups
// come from a segmented scan of the tile (per thread over its 16 positions,
// then over threads and warps), continued from the group's part in earlier
// tiles.  With kW the tile also adds the window's totals: count = all those
// counts (each pair is counted once, by its later tuple), prod = the same
// pairs weighted by fr(left) * gs(right).
template <bool kW>
__global__ void __launch_bounds__(kAttrThreads)
eattr_kernel(const SortView *__restrict__ view, const SortSeg *__restrict__ segs,
             const uint32_t *__restrict__ tile_seg, const ESegMeta *__restrict__ meta,
             const ETileSum *__restrict__ tpre, const sjbg_tuple *__restrict__ L, const sjbg_tuple *__restrict__ R,
             uint32_t B, unsigned long long *__restrict__ counts, WinAcc *__restrict__ acc) {
    __shared__ unsigned long long tc[kTagSmem];   // batch counters of the window
    __shared__ uint32_t wflag[kAttrThreads / 32];
    __shared__ ESum wsum[kAttrThreads / 32];
    __shared__ ESum carry0;
    const uint32_t *__restrict__ keys = view->keys;   // the sorted keys and their positions
    const uint32_t *__restrict__ rels = view->vals;
    const uint32_t s = find_seg(tile_seg, blockIdx.x);
    const SortSeg sg = segs[s];
    const ESegMeta m = meta[s];
    const uint32_t base = (blockIdx.x - sg.tile0) * kSortTile;
    if (base >= sg.n) return;   // whole CTA
    const uint32_t n = min(kSortTile, sg.n - base);
    const bool smem_tags = m.tag_n <= kTagSmem;
    if (smem_tags)
        for (uint32_t i = threadIdx.x; i < m.tag_n; i += blockDim.x) tc[i] = 0;
    // thread t owns positions [t * 16, t * 16 + 16) of the tile; segments start on
    // tile boundaries, so a full run is four aligned 16-byte loads per array
    const uint32_t p0 = threadIdx.x * kAttrPer;
    const uint64_t g = sg.off + base + p0;
    uint32_t k[kAttrPer], tg[kAttrPer], vl[kAttrPer];
    if (p0 + kAttrPer <= n) {
#pragma unroll
        for (int q = 0; q < (int)kAttrPer; q += 4) {
            const uint4 a = *reinterpret_cast<const uint4 *>(keys + g + q);
            const uint4 b = *reinterpret_cast<const uint4 *>(rels + g + q);
            k[q] = a.x; k[q + 1] = a.y; k[q + 2] = a.z; k[q + 3] = a.w;
            tg[q] = b.x; tg[q + 1] = b.y; tg[q + 2] = b.z; tg[q + 3] = b.w;
        }
    } else {
#pragma unroll
        for (int q = 0; q < (int)kAttrPer; q++) {
            const bool valid = p0 + q < n;
            k[q] = valid ? keys[g + q] : 0u;
            tg[q] = valid ? rels[g + q] : 0u;
        }
    }
    const uint32_t prev = p0 < n ? (base + p0 ? keys[g - 1] : ~k[0]) : 0u;
    // pass 1: group heads, and this thread's sums since its last head
    uint32_t heads = 0, anyh = 0;
    ESum run = esum_zero();
#pragma unroll
    for (int q = 0; q < (int)kAttrPer; q++) {
        vl[q] = 0;
        if (p0 + q < n) {
            const ETup e = etuple(tg[q], m.first_tag, L, R, B, kW);
            tg[q] = e.tag;
            vl[q] = e.val;
            if (k[q] != (q ? k[q - 1] : prev)) {
                heads |= 1u << q;
                run = esum_zero();
                anyh = 1;
            }
            esum_item<kW>(run, e);
        }
    }
    // segmented scan over the threads: (flag, sums) (+) (flag', sums') =
    // (flag | flag', flag' ? sums' : sums + sums')
    uint32_t f = anyh;
    ESum a = run;
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
        const uint32_t fy = __shfl_up_sync(0xFFFFFFFFu, f, o);
        const ESum y = esum_shfl_up<kW>(a, o);
        if (lane_id() >= o) {
            if (!f) esum_add(a, y);
            f |= fy;
        }
    }
    uint32_t ef = __shfl_up_sync(0xFFFFFFFFu, f, 1);
    ESum ea = esum_shfl_up<kW>(a, 1);
    if (lane_id() == 0) {
        ef = 0;
        ea = esum_zero();
    }
    if (lane_id() == 31) {
        wflag[warp_id()] = f;
        wsum[warp_id()] = a;
    }
    if (warp_id() == 0) {
        const ESum c = efirst_group_carry<kW>(keys, rels, sg, m.first_tag, tpre, blockIdx.x, base, L, R, B);
        if (lane_id() == 0) carry0 = c;
    }
    SJBG_BARRIER();
    uint32_t cf = 0;
    ESum r = esum_zero();
    for (uint32_t q = 0; q < warp_id(); q++) {
        if (wflag[q]) {
            r = wsum[q];
            cf = 1;
        } else {
            esum_add(r, wsum[q]);
        }
    }
    if (ef) r = ea; else esum_add(r, ea);
    if (!(cf | ef)) esum_add(r, carry0);   // the thread's first group began before the tile
    // pass 2: counts and weighted pairs against the group's earlier tuples
    unsigned long long cnt = 0, prod = 0;
#pragma unroll
    for (int q = 0; q < (int)kAttrPer; q++) {
        if (p0 + q < n) {
            if ((heads >> q) & 1u) r = esum_zero();
            const bool right = tg[q] & 1u;
            const uint32_t c = right ? r.nl : r.nr;
            if (kW) {
                const unsigned long long w = right ? sjbg_gs(vl[q]) : sjbg_fr(vl[q]);
                prod += w * (right ? r.wl : r.wr);
                if (right) r.wr += w; else r.wl += w;
            }
            if (right) r.nr++; else r.nl++;
            cnt += c;
            if (c) {
                if (smem_tags) atomicAdd(&tc[tg[q] - m.tag_lo], (unsigned long long)c);
                else atomicAdd(&counts[tg[q]], (unsigned long long)c);
            }
        }
    }
    if (kW) flush_acc(&acc[s], cnt, 0ull, prod);
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
        // a window opens with left batch l0 (r0 == l0) or with right batch r0 (l0 == r0 + 1)
        const uint32_t first = x.l0 <= x.r0 ? (uint32_t)(2 * x.l0) : (uint32_t)(2 * x.r0 + 1);
        meta[w] = ESegMeta{(uint32_t)(2 * lo), (uint32_t)(2 * (hi - lo)), first, 0};
        const uint64_t off = plan.segs[w].off;
        uint64_t pos = off;
        for (uint64_t b = lo; b < hi; b++) {   // arrival order: left batch b, then right batch b
            for (uint32_t side = 0; side < 2; side++) {
                if (b < (side ? x.r0 : x.l0) || b >= (side ? x.r1 : x.l1)) continue;
                gat.push_back(EGather{pos, (uint32_t)b, side, (uint32_t)(pos - off), 0});
                pos += B;
            }
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
    ETileSum *tpre = static_cast<ETileSum *>(ws_get(h, WS_EAGER_TILES, sizeof(ETileSum) * std::max(plan.tiles, 1u)));
    if (!hst || !dev || !k0 || !t0 || !k1 || !t1 || !tpre) return fail(h, SJBG_E_NOMEM, "eager run buffers");
    std::memcpy(hst, plan.segs.data(), segB);
    std::memcpy(hst + segB, meta.data(), metaB);
    std::memcpy(hst + segB + metaB, gat.data(), gatB);
    if (int rc = stage_copy(h, dev, hst, upB)) return rc;
    const SortSeg *dSegs = reinterpret_cast<const SortSeg *>(dev);
    const ESegMeta *dMeta = reinterpret_cast<const ESegMeta *>(dev + segB);
    const EGather *dGat = reinterpret_cast<const EGather *>(dev + segB + metaB);
    if (int rc_map = sort_tile_map(h, plan, dSegs)) return rc_map;
    uint32_t *kmax = nullptr;
    if (int rc_max = sort_key_max(h, &kmax)) return rc_max;
    SJBG_CK(h, launch(h, "erun_gather", egather_kernel, dim3((uint32_t)gat.size()), dim3(256), 0, dl, dr, dGat,
                      (uint32_t)B, k0, t0, kmax));
    const SortView *view = nullptr;
    int rc = radix_sort_segments(h, plan, dSegs, k0, t0, k1, t1, reinterpret_cast<uint32_t *>(&dWin[nw].info), &view,
                                 kmax);
    if (rc) return rc;
    // sort-merge without pair enumeration: the attribution also forms the window
    // totals (the sorted window is the merge of its two sides); otherwise the
    // lazy join of the windows forms them
    const bool totals = h->cfg.algorithm == SJBG_ALG_SMJ && !enumerate;
    const uint32_t uB = (uint32_t)B;
    if (totals)
        SJBG_CK(h, launch(h, "erun_tile_sum", etile_sum_kernel<true>, dim3(plan.tiles), dim3(256), 0, view, dSegs,
                          plan.tile_seg, dMeta, dl, dr, uB, tpre));
    else
        SJBG_CK(h, launch(h, "erun_tile_sum", etile_sum_kernel<false>, dim3(plan.tiles), dim3(256), 0, view, dSegs,
                          plan.tile_seg, dMeta, dl, dr, uB, tpre));
    SJBG_CK(h, launch(h, "erun_tile_scan", etile_scan_kernel, dim3(nw), dim3(32), 0, dSegs, nw, tpre));
    if (totals) {
        SJBG_CK(h, launch(h, "erun_attribute", eattr_kernel<true>, dim3(plan.tiles), dim3(kAttrThreads), 0, view,
                          dSegs, plan.tile_seg, dMeta, (const ETileSum *)tpre, dl, dr, uB, dCounts, dWin));
        return SJBG_OK;
    }
    SJBG_CK(h, launch(h, "erun_attribute", eattr_kernel<false>, dim3(plan.tiles), dim3(kAttrThreads), 0, view,
                      dSegs, plan.tile_seg, dMeta, (const ETileSum *)tpre, dl, dr, uB, dCounts, dWin));

    uint32_t pu = 0;
    if (h->cfg.algorithm == SJBG_ALG_SMJ) return smj_lazy_batch(h, dl, dr, wh.data(), nw, nullptr, dWin, enumerate);
    return hj_lazy_batch(h, dl, dr, wh.data(), nw, nullptr, dWin, enumerate, &pu);
}

}  // namespace sjbg
