// sort.cu - segmented LSD radix sort (8-bit digits) of (key, val) pairs and
// segmented prefix sums, for the sort-merge join (sm_103a).
//
// One pass = three launches over all segments of a batch:
//   rs_upsweep    per 4096-key tile: digit histogram (one shared atomic per key)
//   rs_scan       per segment: each digit's tile counts scanned over the tiles
//                 (a warp per digit), the digit totals scanned into per-digit
//                 starts, so tile t's digit d lands after all smaller digits
//                 and after digit d of tiles < t (stability)
//   rs_downsweep  per tile: the tile's keys and vals are staged in shared
//                 memory by TMA bulk copies (cp.async.bulk, mbarrier with a
//                 bounded wait); stable ranks come from warp-private digit
//                 counters and each lane's digit peers (nine ballots: faster
//                 than __match_any_sync); the tile is reordered in shared
//                 memory and written as contiguous per-digit runs.
// Every per-tile kernel finds its segment in the plan's tile map (one load).
// The reference's GPU sort-merge join uses a counting sort by key with
// unstable atomics instead (src/sjb/windowing/lazy/executor/GPU/GPU_SMJ.cu:19-32).
#include <algorithm>
#include <cstring>
#include <vector>

#include "sort.cuh"

namespace sjbg {

constexpr int kSortThreads = 512;
constexpr int kSortWarps = kSortThreads / 32;
constexpr uint32_t kDigits = 256;

SortPlan sort_plan(const uint64_t *n, const uint64_t *src, uint32_t k) {
    SortPlan p;
    p.segs.resize(k);
    uint64_t off = 0;
    uint32_t tiles = 0;
    for (uint32_t s = 0; s < k; s++) {
        const uint64_t padded = (n[s] + 1 + kSortTile - 1) / kSortTile * kSortTile;
        p.segs[s] = SortSeg{off, src[s], (uint32_t)n[s], tiles, (uint32_t)(padded / kSortTile), 0};
        off += padded;
        tiles += (uint32_t)(padded / kSortTile);
    }
    p.tiles = tiles;
    p.elems = off;
    return p;
}

// ------------------------------------------------------------------ TMA bulk staging
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// 1-D bulk copy global -> shared (16-byte aligned addresses, size multiple of 16).
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// Bounded wait on phase `parity`; false when it gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    for (uint32_t it = 0; it < (1u << 26); it++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// ------------------------------------------------------------------ kernels
// Under graph capture every pass is launched and the largest key (written on
// the device by sort_max) decides: a pass whose digit is zero in every key is
// the identity permutation and is skipped by all its kernels.  kmax == nullptr:
// the host chose the passes.
__device__ __forceinline__ bool pass_is_identity(const uint32_t *kmax, uint32_t shift) {
    return kmax != nullptr && shift != 0 && (*kmax >> shift) == 0;
}

// Points the view at the buffer pair the last pass wrote: after an even
// number of passes the input pair, after an odd number the scratch pair.
// kmax == nullptr: the host's pass count `passes` ran; else the first pass and
// every pass whose digit is not zero in the largest key did.
__global__ void sort_view_kernel(SortView *view, const uint32_t *keys, const uint32_t *vals, const uint32_t *keys2,
                                 const uint32_t *vals2, const uint32_t *__restrict__ kmax, uint32_t passes) {
    uint32_t ran = passes;
    if (kmax) {
        const uint32_t m = *kmax;
        ran = 1;
        for (uint32_t shift = 8; shift < 32; shift += 8) ran += (m >> shift) != 0;
    }
    view->keys = (ran & 1u) ? keys2 : keys;
    view->vals = (ran & 1u) ? vals2 : vals;
}
// Lanes of the warp holding the same 9-bit digit (256 = no element): one
// ballot per bit, each lane keeping the lanes that agree with it on that bit.
__device__ __forceinline__ unsigned digit_peers(uint32_t d) {
    unsigned peers = 0xFFFFFFFFu;
#pragma unroll
    for (int b = 0; b < 9; b++) {
        const bool bit = (d >> b) & 1u;
        const unsigned m = __ballot_sync(0xFFFFFFFFu, bit);
        peers &= bit ? m : ~m;
    }
    return peers;
}

// Segments [0, split) read srcA, the others srcB.
__global__ void __launch_bounds__(256)
sort_extract_kernel(const sjbg_tuple *__restrict__ srcA, const sjbg_tuple *__restrict__ srcB, uint32_t split,
                    const SortSeg *__restrict__ segs, const uint32_t *__restrict__ tile_seg, uint32_t *__restrict__ keys,
                    uint32_t *__restrict__ vals, uint32_t *__restrict__ kmax) {
    const uint32_t s = find_seg(tile_seg, blockIdx.x);
    const SortSeg sg = segs[s];
    const sjbg_tuple *src = s < split ? srcA : srcB;
    const uint32_t base = (blockIdx.x - sg.tile0) * kSortTile;
    uint32_t m = 0;
    for (uint32_t i = threadIdx.x; i < kSortTile; i += blockDim.x) {
        const uint32_t li = base + i;
        uint32_t k = 0xFFFFFFFFu, v = 0;
        if (li < sg.n) {
            const uint2 t = __ldg(reinterpret_cast<const uint2 *>(src + sg.src + li));
            k = t.x;
            v = t.y;
            m = max(m, k);
        }
        keys[sg.off + li] = k;
        vals[sg.off + li] = v;
    }
    if (kmax) block_key_max(m, kmax);
}

__global__ void __launch_bounds__(256)
sort_max_kernel(const uint32_t *__restrict__ keys, const SortSeg *__restrict__ segs, const uint32_t *__restrict__ tile_seg,
                uint32_t *__restrict__ out) {
    const uint32_t s = find_seg(tile_seg, blockIdx.x);
    const SortSeg sg = segs[s];
    const uint32_t base = (blockIdx.x - sg.tile0) * kSortTile;
    uint32_t m = 0;
    for (uint32_t i = threadIdx.x; i < kSortTile; i += blockDim.x)
        if (base + i < sg.n) m = max(m, keys[sg.off + base + i]);
    block_key_max(m, out);
}

// counts block of segment s: counts[tile0 * 256 + d * ntiles + t_local]
__global__ void __launch_bounds__(256)
rs_upsweep_kernel(const uint32_t *__restrict__ keys, const SortSeg *__restrict__ segs,
                  const uint32_t *__restrict__ tile_seg, uint32_t shift, uint32_t *__restrict__ counts,
                  const uint32_t *__restrict__ kmax) {
    if (pass_is_identity(kmax, shift)) return;   // whole grid
    __shared__ uint32_t hist[kDigits];
    const uint32_t s = find_seg(tile_seg, blockIdx.x);
    const SortSeg sg = segs[s];
    const uint32_t tl = blockIdx.x - sg.tile0;
    const uint32_t base = tl * kSortTile;
    hist[threadIdx.x] = 0;
    SJBG_BARRIER();
    const uint4 *k4 = reinterpret_cast<const uint4 *>(keys + sg.off + base);
    constexpr int kPer = kSortTile / 4 / 256;   // 4 vectors per thread
    uint4 v[kPer];
#pragma unroll
    for (int q = 0; q < kPer; q++) v[q] = __ldg(k4 + threadIdx.x + q * 256);
#pragma unroll
    for (int q = 0; q < kPer; q++) {
        const uint32_t e0 = base + 4 * (threadIdx.x + q * 256);
        const uint32_t kk[4] = {v[q].x, v[q].y, v[q].z, v[q].w};
#pragma unroll
        for (int c = 0; c < 4; c++) {
            const bool valid = e0 + c < sg.n;
            const uint32_t d = valid ? (kk[c] >> shift) & 0xFFu : 0u;
            if (valid) atomicAdd(&hist[d], 1u);   // one shared atomic per key: faster than combining a warp's equal digits first
        }
    }
    SJBG_BARRIER();
    counts[(uint64_t)sg.tile0 * kDigits + (uint64_t)threadIdx.x * sg.ntiles + tl] = hist[threadIdx.x];
}

// Grid (segments, G): CTA (s, g) scans digits [g * 256 / G, (g + 1) * 256 / G)
// of segment s, 256 / (8 G) consecutive digits per warp.  Each digit's tile
// counts (contiguous: the block is digit-major) get an exclusive scan over the
// tiles in place.  A warp walks its (digit, 32-tile chunk) items eight at a
// time, the eight loads issued before the eight scans, so few and many tiles
// per segment both keep loads in flight.  The digit totals go to dtot; the
// segment's last CTA to finish (a counter per segment, reset by that CTA for
// the next pass) scans them into digoff[segment][digit].  Tile t's digit d
// starts at digoff[d] + counts[d][t]: after every smaller digit of the
// segment and after digit d of the tiles before t (stability).  Segments hold
// at least one tile.
__global__ void __launch_bounds__(256)
rs_scan_kernel(uint32_t *__restrict__ counts, const SortSeg *__restrict__ segs, uint32_t *__restrict__ digoff,
               uint32_t *__restrict__ dtot, uint32_t *__restrict__ done, uint32_t shift,
               const uint32_t *__restrict__ kmax) {
    if (pass_is_identity(kmax, shift)) return;   // whole grid
    __shared__ uint32_t last;
    const uint32_t s = blockIdx.x, G = gridDim.y;
    const SortSeg sg = segs[s];
    uint32_t *c = counts + (uint64_t)sg.tile0 * kDigits;
    const uint32_t nt = sg.ntiles, lane = lane_id();
    const uint32_t pw = kDigits / (G * (blockDim.x >> 5));                  // digits per warp
    const uint32_t d0 = blockIdx.y * (kDigits / G) + warp_id() * pw;        // the warp's first digit
    const uint32_t nch = (nt + 31) >> 5, items = pw * nch;
    uint32_t carry = 0;
    for (uint32_t i0 = 0; i0 < items; i0 += 8) {
        uint32_t v[8];
#pragma unroll
        for (uint32_t j = 0; j < 8; j++) {
            const uint32_t i = i0 + j, row = i / nch, t = (i - row * nch) * 32 + lane;
            v[j] = (i < items && t < nt) ? c[(uint64_t)(d0 + row) * nt + t] : 0u;
        }
#pragma unroll
        for (uint32_t j = 0; j < 8; j++) {
            const uint32_t i = i0 + j;
            if (i >= items) break;   // uniform over the warp
            const uint32_t row = i / nch, ch = i - row * nch, t = ch * 32 + lane;
            uint32_t tot;
            const uint32_t ex = warp_excl_scan(v[j], &tot);
            if (t < nt) c[(uint64_t)(d0 + row) * nt + t] = carry + ex;
            carry += tot;
            if (ch == nch - 1) {
                if (lane == 0) dtot[(uint64_t)s * kDigits + d0 + row] = carry;
                carry = 0;
            }
        }
    }
    if (G > 1) {
        __threadfence();
        SJBG_BARRIER();
        if (threadIdx.x == 0) last = atomicAdd(&done[s], 1u) == G - 1;
        SJBG_BARRIER();
        if (!last) return;
        __threadfence();
        if (threadIdx.x == 0) done[s] = 0;
    } else {
        SJBG_BARRIER();
    }
    if (warp_id() == 0) {
        constexpr uint32_t kPer = kDigits / 32;
        uint32_t a[kPer], sum = 0;
#pragma unroll
        for (uint32_t q = 0; q < kPer; q++) {
            a[q] = __ldcg(&dtot[(uint64_t)s * kDigits + lane * kPer + q]);
            sum += a[q];
        }
        uint32_t tot;
        uint32_t run = warp_excl_scan(sum, &tot);
        uint32_t *dw = digoff + (uint64_t)s * kDigits;
#pragma unroll
        for (uint32_t q = 0; q < kPer; q++) {
            dw[lane * kPer + q] = run;
            run += a[q];
        }
    }
}

struct DownSmem {
    uint32_t in_keys[kSortTile];
    uint32_t in_vals[kSortTile];
    uint16_t perm[kSortTile];                  // tile position of the p-th element in sorted order
    uint32_t wcnt[kSortWarps][kDigits + 1];   // per-warp digit counters (+1: invalid slots)
    uint32_t loc[kDigits];                     // tile-local digit offsets
    uint32_t gofs[kDigits];                    // global digit offsets of this tile
    uint32_t warp_tot[32];
    uint64_t bar;
};

// Three CTAs per SM: the reorder keeps a 16-bit permutation instead of a
// second copy of the tile's keys and vals (58 KB of shared memory per CTA).
__global__ void __launch_bounds__(kSortThreads, 3)
rs_downsweep_kernel(const uint32_t *__restrict__ keys, const uint32_t *__restrict__ vals,
                    uint32_t *__restrict__ keys_out, uint32_t *__restrict__ vals_out,
                    const SortSeg *__restrict__ segs, const uint32_t *__restrict__ tile_seg, uint32_t shift,
                    const uint32_t *__restrict__ counts, const uint32_t *__restrict__ digoff,
                    uint32_t *__restrict__ status, const uint32_t *__restrict__ kmax) {
    if (pass_is_identity(kmax, shift)) return;   // whole grid
    extern __shared__ __align__(128) uint8_t smem_raw[];
    DownSmem &sm = *reinterpret_cast<DownSmem *>(smem_raw);
    const uint32_t s = find_seg(tile_seg, blockIdx.x);
    const SortSeg sg = segs[s];
    const uint32_t tl = blockIdx.x - sg.tile0;
    const uint32_t base = tl * kSortTile;
    const uint32_t n = sg.n > base ? min(kSortTile, sg.n - base) : 0u;
    const uint32_t w = warp_id(), lane = lane_id();

    if (threadIdx.x == 0) mbar_init(&sm.bar, 1);
    for (uint32_t i = threadIdx.x; i < kSortWarps * (kDigits + 1); i += kSortThreads) (&sm.wcnt[0][0])[i] = 0;
    SJBG_BARRIER();
    if (threadIdx.x == 0) {
        mbar_expect_tx(&sm.bar, 2 * kSortTile * 4);
        bulk_g2s(sm.in_keys, keys + sg.off + base, kSortTile * 4, &sm.bar);
        bulk_g2s(sm.in_vals, vals + sg.off + base, kSortTile * 4, &sm.bar);
    }
    if (threadIdx.x < kDigits)
        sm.gofs[threadIdx.x] = digoff[(uint64_t)s * kDigits + threadIdx.x] +
                               counts[(uint64_t)sg.tile0 * kDigits + (uint64_t)threadIdx.x * sg.ntiles + tl];
    // every thread waits (bounded); the block leaves together if any gave up
    const bool arrived = mbar_wait(&sm.bar, 0);
    if (!__syncthreads_and(arrived)) {
        if (threadIdx.x == 0) atomicOr(status, kErrTimeout);
        return;
    }

    // stable warp-local ranks: warp w owns tile positions [w*256, w*256+256),
    // item k of lane l is position w*256 + k*32 + l (k-major = tile order)
    constexpr int kItems = kSortTile / kSortThreads;   // 8
    uint32_t rank[kItems], dig[kItems];
    const unsigned lt_mask = (1u << lane) - 1u;
#pragma unroll
    for (int k = 0; k < kItems; k++) {
        const uint32_t pos = w * (kSortTile / kSortWarps) + k * 32 + lane;
        const uint32_t d = pos < n ? (sm.in_keys[pos] >> shift) & 0xFFu : kDigits;
        const unsigned peers = digit_peers(d);
        const uint32_t cur = sm.wcnt[w][d];
        __syncwarp();
        rank[k] = cur + __popc(peers & lt_mask);
        dig[k] = d;
        if (lane == (uint32_t)(__ffs(peers) - 1)) sm.wcnt[w][d] = cur + __popc(peers);
        __syncwarp();
    }
    SJBG_BARRIER();
    // per digit: exclusive scan over warps, tile total in `loc`
    if (threadIdx.x < kDigits) {
        uint32_t run = 0;
        for (int ww = 0; ww < kSortWarps; ww++) {
            const uint32_t c = sm.wcnt[ww][threadIdx.x];
            sm.wcnt[ww][threadIdx.x] = run;
            run += c;
        }
        sm.loc[threadIdx.x] = run;
    }
    SJBG_BARRIER();
    // exclusive scan of the 256 digit totals (8 warps x 32 digits)
    if (threadIdx.x < kDigits) {
        const uint32_t x = sm.loc[threadIdx.x];
        uint32_t tot;
        const uint32_t ex = warp_excl_scan(x, &tot);
        if (lane == 31) sm.warp_tot[w] = ex + x;
        __syncwarp();
        sm.loc[threadIdx.x] = ex;   // partial; warp offsets added below
    }
    SJBG_BARRIER();
    if (threadIdx.x < kDigits) {
        uint32_t add = 0;
        for (uint32_t ww = 0; ww < w; ww++) add += sm.warp_tot[ww];
        sm.loc[threadIdx.x] += add;
    }
    SJBG_BARRIER();
#pragma unroll
    for (int k = 0; k < kItems; k++) {
        const uint32_t pos = w * (kSortTile / kSortWarps) + k * 32 + lane;
        if (pos < n) {
            const uint32_t d = dig[k];
            const uint32_t p = sm.loc[d] + sm.wcnt[w][d] + rank[k];
            sm.perm[p] = (uint16_t)pos;
        }
    }
    SJBG_BARRIER();
    for (uint32_t j = threadIdx.x; j < n; j += kSortThreads) {
        const uint32_t q = sm.perm[j];
        const uint32_t k = sm.in_keys[q];
        const uint32_t d = (k >> shift) & 0xFFu;
        const uint64_t dst = sg.off + sm.gofs[d] + (j - sm.loc[d]);
        keys_out[dst] = k;
        vals_out[dst] = sm.in_vals[q];
    }
}

// ---- segmented exclusive prefix of fr(val): tile sums, per-segment scan of the
// ---- tile sums, per-tile scan plus offset
__global__ void __launch_bounds__(256)
fr_tile_sum_kernel(const SortView *__restrict__ view, const SortSeg *__restrict__ segs,
                   const uint32_t *__restrict__ tile_seg, unsigned long long *__restrict__ tsum) {
    const uint32_t *__restrict__ vals = view->vals;
    __shared__ unsigned long long ws[8];
    const uint32_t s = find_seg(tile_seg, blockIdx.x);
    const SortSeg sg = segs[s];
    const uint32_t base = (blockIdx.x - sg.tile0) * kSortTile;
    unsigned long long acc = 0;
    for (uint32_t i = threadIdx.x; i < kSortTile; i += blockDim.x)
        if (base + i < sg.n) acc += sjbg_fr(vals[sg.off + base + i]);
    acc = warp_sum_u64(acc);
    if (lane_id() == 0) ws[warp_id()] = acc;
    SJBG_BARRIER();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int i = 0; i < 8; i++) t += ws[i];
        tsum[blockIdx.x] = t;
    }
}

__global__ void fr_seg_scan_kernel(unsigned long long *__restrict__ tsum, const SortSeg *__restrict__ segs) {
    const SortSeg sg = segs[blockIdx.x];
    if (threadIdx.x == 0) {
        unsigned long long run = 0;
        for (uint32_t t = 0; t < sg.ntiles; t++) {
            const unsigned long long v = tsum[sg.tile0 + t];
            tsum[sg.tile0 + t] = run;
            run += v;
        }
    }
}

__global__ void __launch_bounds__(256)
fr_tile_scan_kernel(const SortView *__restrict__ view, const SortSeg *__restrict__ segs,
                    const uint32_t *__restrict__ tile_seg, const unsigned long long *__restrict__ tsum,
                    unsigned long long *__restrict__ out) {
    const uint32_t *__restrict__ vals = view->vals;
    // warp w owns the tile's elements [w * 512, (w + 1) * 512), 32 consecutive
    // ones per round: coalesced loads and stores, fr computed once per element
    constexpr uint32_t kWarps = 8, kChunk = kSortTile / kWarps, kRounds = kChunk / 32;   // 256 threads
    __shared__ unsigned long long wtot[kWarps];
    const uint32_t s = find_seg(tile_seg, blockIdx.x);
    const SortSeg sg = segs[s];
    const uint32_t base = (blockIdx.x - sg.tile0) * kSortTile;
    const uint32_t w = warp_id(), lane = lane_id();
    const uint32_t c0 = base + w * kChunk;
    unsigned long long f[kRounds], tot = 0;
#pragma unroll
    for (uint32_t r = 0; r < kRounds; r++) {
        const uint32_t li = c0 + 32 * r + lane;
        f[r] = li < sg.n ? sjbg_fr(vals[sg.off + li]) : 0ull;
        tot += f[r];
    }
    tot = warp_sum_u64(tot);
    if (lane == 0) wtot[w] = tot;
    SJBG_BARRIER();
    unsigned long long run = tsum[blockIdx.x];
    for (uint32_t ww = 0; ww < w; ww++) run += wtot[ww];
#pragma unroll
    for (uint32_t r = 0; r < kRounds; r++) {
        unsigned long long x = f[r];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        const uint32_t li = c0 + 32 * r + lane;
        if (li <= sg.n) out[sg.off + li] = run + x - f[r];   // positions 0..n inclusive
        run += __shfl_sync(0xFFFFFFFFu, x, 31);
    }
}

__global__ void __launch_bounds__(256) sort_tile_map_kernel(const SortSeg *__restrict__ segs, uint32_t *__restrict__ map) {
    const SortSeg sg = segs[blockIdx.x];
    for (uint32_t t = threadIdx.x; t < sg.ntiles; t += blockDim.x) map[sg.tile0 + t] = blockIdx.x;
}

// ------------------------------------------------------------------ host drivers
int sort_tile_map(sjbg_handle *h, SortPlan &plan, const SortSeg *dSegs) {
    uint32_t *map = static_cast<uint32_t *>(ws_get(h, WS_SORT_MAP, sizeof(uint32_t) * std::max(plan.tiles, 1u)));
    if (!map) return fail(h, SJBG_E_NOMEM, "sort tile map");
    if (!plan.segs.empty())
        SJBG_CK(h, launch(h, "sort_tile_map", sort_tile_map_kernel, dim3((uint32_t)plan.segs.size()), dim3(256), 0,
                          dSegs, map));
    plan.tile_seg = map;
    return SJBG_OK;
}

int sort_key_max(sjbg_handle *h, uint32_t **kmax) {
    *kmax = static_cast<uint32_t *>(ws_get(h, WS_STATUS, 64));
    if (!*kmax) return fail(h, SJBG_E_NOMEM, "sort buffers");
    SJBG_CK(h, cudaMemsetAsync(*kmax, 0, 64, h->stream));
    return SJBG_OK;
}

int sort_extract(sjbg_handle *h, const sjbg_tuple *srcA, const sjbg_tuple *srcB, uint32_t split, const SortPlan &plan,
                 const SortSeg *dSegs, uint32_t *keys, uint32_t *vals, uint32_t *kmax) {
    SJBG_CK(h, launch(h, "sort_extract", sort_extract_kernel, dim3(plan.tiles), dim3(256), 0, srcA, srcB, split, dSegs,
                      plan.tile_seg, keys, vals, kmax));
    return SJBG_OK;
}

int radix_sort_segments(sjbg_handle *h, const SortPlan &plan, const SortSeg *dSegs, uint32_t *keys, uint32_t *vals,
                        uint32_t *keys2, uint32_t *vals2, uint32_t *status, const SortView **view, uint32_t *kmax) {
    const uint32_t nseg = (uint32_t)plan.segs.size();
    uint32_t *dMax = kmax;
    if (!dMax)
        if (int rc = sort_key_max(h, &dMax)) return rc;
    // per tile and digit: the digit's count, then its start among the segment's tiles;
    // per segment and digit: the digit's start in the segment
    // then per segment and digit the digit's total, and per segment a finished-CTA counter
    uint32_t *counts =
        static_cast<uint32_t *>(ws_get(h, WS_SORT_HIST, sizeof(uint32_t) * (kDigits * (plan.tiles + 2 * nseg) + nseg)));
    SortView *dView = static_cast<SortView *>(ws_get(h, WS_SORT_VIEW, sizeof(SortView)));
    if (!counts || !dView) return fail(h, SJBG_E_NOMEM, "sort buffers");
    if (!kmax)
        SJBG_CK(h, launch(h, "sort_max", sort_max_kernel, dim3(plan.tiles), dim3(256), 0, (const uint32_t *)keys, dSegs,
                          plan.tile_seg, dMax));
    // all four passes are launched and each skips itself on the device when its
    // digit is zero in every key: no read-back of the key range, no host wait,
    // and the same launches under graph capture
    const uint32_t passes = 4;
    const uint32_t *dkmax = dMax;
    uint32_t *digoff = counts + (size_t)kDigits * plan.tiles;
    uint32_t *dtot = digoff + (size_t)kDigits * nseg;
    uint32_t *done = dtot + (size_t)kDigits * nseg;
    SJBG_CK(h, cudaMemsetAsync(done, 0, sizeof(uint32_t) * nseg, h->stream));
    // CTAs per segment: as many as keep the scan within about one wave of 256-thread CTAs
    uint32_t G = 1;
    while (G < 32 && (uint64_t)nseg * G * 2 <= 1216) G *= 2;
    const size_t smem = sizeof(DownSmem);
    allow_big_smem(rs_downsweep_kernel, smem);
    uint32_t *kin = keys, *vin = vals, *kout = keys2, *vout = vals2;
    for (uint32_t p = 0; p < passes; p++) {
        const uint32_t shift = 8 * p;
        SJBG_CK(h, launch(h, "rs_upsweep", rs_upsweep_kernel, dim3(plan.tiles), dim3(256), 0, (const uint32_t *)kin,
                          dSegs, plan.tile_seg, shift, counts, dkmax));
        SJBG_CK(h, launch(h, "rs_scan", rs_scan_kernel, dim3(nseg, G), dim3(256), 0, counts, dSegs, digoff, dtot, done,
                          shift, dkmax));
        SJBG_CK(h, launch(h, "rs_downsweep", rs_downsweep_kernel, dim3(plan.tiles), dim3(kSortThreads), smem,
                          (const uint32_t *)kin, (const uint32_t *)vin, kout, vout, dSegs, plan.tile_seg, shift,
                          (const uint32_t *)counts, (const uint32_t *)digoff, status, dkmax));
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
    // no copy home: the consumers read the result where the last pass left it
    SJBG_CK(h, launch(h, "sort_view", sort_view_kernel, dim3(1), dim3(1), 0, dView, (const uint32_t *)keys,
                      (const uint32_t *)vals, (const uint32_t *)keys2, (const uint32_t *)vals2, dkmax, passes));
    *view = dView;
    return SJBG_OK;
}

int segmented_fr_prefix(sjbg_handle *h, const SortPlan &plan, uint32_t nseg, const SortSeg *dSegs,
                        const SortView *view, unsigned long long *out) {
    if (nseg == 0) return SJBG_OK;
    // the first nseg segments: their tiles are [0, tile0 of segment nseg)
    const uint32_t tiles = nseg < plan.segs.size() ? plan.segs[nseg].tile0 : plan.tiles;
    unsigned long long *tsum = static_cast<unsigned long long *>(ws_get(h, WS_AUX3, sizeof(unsigned long long) * tiles));
    if (!tsum) return fail(h, SJBG_E_NOMEM, "prefix buffers");
    SJBG_CK(h, launch(h, "fr_tile_sum", fr_tile_sum_kernel, dim3(tiles), dim3(256), 0, view, dSegs, plan.tile_seg, tsum));
    SJBG_CK(h, launch(h, "fr_seg_scan", fr_seg_scan_kernel, dim3(nseg), dim3(32), 0, tsum, dSegs));
    SJBG_CK(h, launch(h, "fr_tile_scan", fr_tile_scan_kernel, dim3(tiles), dim3(256), 0, view, dSegs, plan.tile_seg,
                      (const unsigned long long *)tsum, out));
    return SJBG_OK;
}

}  // namespace sjbg
