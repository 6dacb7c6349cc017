// learned.cu - learned key-CDF partitioner: sampling, least-squares fit and
// model check (no reference counterpart).
//
// Per window, on the device:
//   1. sample      rate * (|L|+|R|) keys at jittered strided positions of both
//                  sides; per-window min/max key.
//   2. count       equal-width histogram of the sample over kBins key bins and
//                  exact per-key sample counts in a per-window hash table.
//   3. heavy       keys whose sample count exceeds one bucket's fair share
//                  become candidates.
//   4. fit         (one CTA per window) the top kMaxHeavy candidates are made
//                  heavy and removed from the histogram; the light CDF at the
//                  bin edges is fitted by least squares: a root line routes
//                  points to `leaves` leaves, each leaf gets its own line
//                  (centred sums, two passes); lo/hi clamps make it monotone.
//   5. check       (inference) the model buckets the light sample; if the
//                  largest predicted bucket exceeds overflow_bound times the
//                  mean, the window falls back to radix partitioning.
#include <algorithm>
#include <cstring>
#include <vector>

#include "learned.cuh"
#include "runtime.h"

namespace sjbg {

constexpr uint32_t kBins = 1u << 16;     // histogram bins of the fit
constexpr uint32_t kCandMax = 2048;       // heavy candidates kept per window
constexpr uint32_t kSampleThreads = 256;
constexpr uint32_t kPredStride = 1u << 14;  // predicted-bucket counters per window (max buckets)

struct SampleWin {
    uint64_t left_off, n_left, right_off, n_right;
    uint32_t m;            // samples (even)
    uint32_t table_log2;   // per-window sample count table
    uint64_t table_off;    // first slot of this window's table
    uint32_t thresh;       // heavy candidate threshold (sample count)
    uint32_t log2_buckets;
};

struct SampleScratch {
    uint32_t kmin, kmax;   // sample key range
    uint32_t n_cand;
    uint32_t cut;          // candidates have a sample count >= cut
    uint32_t cls[32];      // candidate keys per count class floor(log2(count))
};

__device__ __forceinline__ uint32_t sample_key(const SampleWin &s, const sjbg_tuple *L, const sjbg_tuple *R, uint32_t i) {
    const bool right = i & 1u;
    const uint64_t n = right ? s.n_right : s.n_left;
    const uint64_t half = s.m >> 1;
    const uint64_t j = i >> 1;
    const uint64_t stride = n / half;   // >= 1 by construction of m
    uint64_t idx = j * stride + (stride > 1 ? sjbg_mix64(0x5A17ull + i) % stride : 0);
    if (idx >= n) idx = n - 1;
    return right ? R[s.right_off + idx].key : L[s.left_off + idx].key;
}

__global__ void __launch_bounds__(kSampleThreads)
sample_minmax_kernel(const sjbg_tuple *L, const sjbg_tuple *R, const SampleWin *wins, SampleScratch *scr) {
    const uint32_t w = blockIdx.y;
    const SampleWin s = wins[w];
    uint32_t lo = 0xFFFFFFFFu, hi = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < s.m; i += gridDim.x * blockDim.x) {
        uint32_t k = sample_key(s, L, R, i);
        lo = min(lo, k);
        hi = max(hi, k);
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xFFFFFFFFu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xFFFFFFFFu, hi, o));
    }
    if (lane_id() == 0) {
        atomicMin(&scr[w].kmin, lo);
        atomicMax(&scr[w].kmax, hi);
    }
}

__device__ __forceinline__ float key_x(uint32_t key, float kmin, float inv) {
    return fminf(fmaxf(((float)key - kmin) * inv, 0.0f), 1.0f);
}
__device__ __forceinline__ void model_range(const SampleScratch &sc, float *kmin, float *inv) {
    *kmin = (float)sc.kmin;
    float range = (float)sc.kmax - (float)sc.kmin;
    *inv = range > 0.0f ? 1.0f / range : 0.0f;
}
__device__ __forceinline__ uint32_t bin_of(float x) {
    uint32_t b = (uint32_t)(x * (float)kBins);
    return b < kBins ? b : kBins - 1;
}

// Sample histogram + exact sample counts (table slot = key << 32 | count).
__global__ void __launch_bounds__(kSampleThreads)
sample_count_kernel(const sjbg_tuple *L, const sjbg_tuple *R, const SampleWin *wins, const SampleScratch *scr,
                    uint32_t *hist, unsigned long long *table) {
    const uint32_t w = blockIdx.y;
    const SampleWin s = wins[w];
    float kmin, inv;
    model_range(scr[w], &kmin, &inv);
    uint32_t *hw = hist + (uint64_t)w * kBins;
    unsigned long long *tw = table + s.table_off;
    const uint32_t mask = (1u << s.table_log2) - 1;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < s.m; i += gridDim.x * blockDim.x) {
        const uint32_t k = sample_key(s, L, R, i);
        atomicAdd(&hw[bin_of(key_x(k, kmin, inv))], 1u);
        uint32_t slot = slot_hash(k, s.table_log2);
        for (uint32_t p = 0; p <= mask; p++) {
            unsigned long long cur = tw[slot];
            if (cur == 0ull) {
                unsigned long long prev = atomicCAS(&tw[slot], 0ull, ((unsigned long long)k << 32) | 1ull);
                if (prev == 0ull) break;
                cur = prev;
            }
            if ((uint32_t)(cur >> 32) == k) {
                atomicAdd(&tw[slot], 1ull);
                break;
            }
            slot = (slot + 1) & mask;
        }
    }
}

// Candidates per count class, so that the candidate cut keeps the heaviest keys.
__global__ void __launch_bounds__(kSampleThreads)
heavy_classes_kernel(const SampleWin *wins, const unsigned long long *table, SampleScratch *scr) {
    const uint32_t w = blockIdx.y;
    const SampleWin s = wins[w];
    const unsigned long long *tw = table + s.table_off;
    const uint32_t slots = 1u << s.table_log2;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < slots; i += gridDim.x * blockDim.x) {
        const unsigned long long v = tw[i];
        const uint32_t c = (uint32_t)v;
        if (v && c >= s.thresh) atomicAdd(&scr[w].cls[31 - __clz(c)], 1u);
    }
}

// The smallest count class boundary 2^k (>= thresh) above which at most
// kCandMax keys lie: every key counted more often than any dropped key is kept.
__device__ __forceinline__ uint32_t candidate_cut(const SampleScratch &sc, uint32_t thresh) {
    uint32_t acc = 0;
    for (int k = 31; k >= 0; k--) {
        acc += sc.cls[k];
        if (acc > kCandMax) return max(thresh, k == 31 ? 0xFFFFFFFFu : (1u << (k + 1)));
    }
    return thresh;
}

__global__ void __launch_bounds__(kSampleThreads)
heavy_candidates_kernel(const SampleWin *wins, const unsigned long long *table, SampleScratch *scr,
                        unsigned long long *cand) {
    const uint32_t w = blockIdx.y;
    const SampleWin s = wins[w];
    const unsigned long long *tw = table + s.table_off;
    const uint32_t slots = 1u << s.table_log2;
    const uint32_t cut = candidate_cut(scr[w], s.thresh);
    if (blockIdx.x == 0 && threadIdx.x == 0) scr[w].cut = cut;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < slots; i += gridDim.x * blockDim.x) {
        const unsigned long long v = tw[i];
        const uint32_t c = (uint32_t)v;
        if (v && c >= cut) {
            uint32_t pos = atomicAdd(&scr[w].n_cand, 1u);
            // candidates sort by count descending, then key: (count << 32 | ~key)
            if (pos < kCandMax) cand[(uint64_t)w * kCandMax + pos] = ((unsigned long long)c << 32) | (~(uint32_t)(v >> 32));
        }
    }
}

// One CTA (1024 threads) per window.
__global__ void __launch_bounds__(1024)
learned_fit_kernel(const SampleWin *wins, SampleScratch *scr, uint32_t *hist, unsigned long long *cand,
                   LearnedModel *models, uint32_t leaves, uint32_t max_heavy, float bound) {
    __shared__ unsigned long long sc[kCandMax];
    __shared__ float ls[kMaxLeaves][5];           // n, sum x, sum y, sum dx*dy, sum dx*dx
    __shared__ float lmin[kMaxLeaves], lmax[kMaxLeaves];
    __shared__ uint32_t warp_tot[32];
    __shared__ double rootsum[4];
    __shared__ uint32_t n_heavy_s, light_total_s, log2_eff_s, compact_s;
    const uint32_t w = blockIdx.x;
    const SampleWin s = wins[w];
    LearnedModel &M = models[w];
    uint32_t *hw = hist + (uint64_t)w * kBins;
    float kmin, inv;
    model_range(scr[w], &kmin, &inv);

    // ---- heavy keys: bitonic sort of the candidates (descending), keep the top
    const uint32_t nc = min(scr[w].n_cand, kCandMax);
    for (uint32_t i = threadIdx.x; i < kCandMax; i += blockDim.x) sc[i] = i < nc ? cand[(uint64_t)w * kCandMax + i] : 0ull;
    SJBG_BARRIER();
    for (uint32_t k = 2; k <= kCandMax; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = threadIdx.x; i < kCandMax; i += blockDim.x) {
                const uint32_t p = i ^ j;
                if (p > i) {
                    const bool desc = (i & k) == 0;
                    const unsigned long long a = sc[i], b = sc[p];
                    if (desc ? (a < b) : (a > b)) { sc[i] = b; sc[p] = a; }
                }
            }
            SJBG_BARRIER();
        }
    }
    if (threadIdx.x == 0) {
        // largest first, a candidate is heavy while its sampled count exceeds an
        // eighth of one bucket's share of the mass that is still light
        const uint64_t P = 1ull << s.log2_buckets;
        uint64_t light = s.m;
        uint32_t h = 0;
        const uint32_t lim = min(nc, max_heavy);
        while (h < lim) {
            const uint64_t c = sc[h] >> 32;
            if (c * 8 * P <= light) break;
            light -= c;
            h++;
        }
        n_heavy_s = h;
        // fan-out for the light keys only: about as many light tuples per
        // bucket as the window's plan has tuples per bucket
        uint32_t lg = s.log2_buckets;
        while (lg > 0 && ((uint64_t)s.m << (lg - 1)) >= (light << s.log2_buckets)) lg--;
        // the largest light key must stay well inside the overflow bound
        const uint64_t c1 = h < nc ? (sc[h] >> 32) : (uint64_t)scr[w].cut;
        while (lg > 0 && 2.0 * (double)c1 * (double)(1ull << lg) > (double)bound * (double)light) lg--;
        log2_eff_s = lg;
        // when at most half of the sample is light, the counting pass also
        // writes the light tuples out compacted, and only those are re-read
        compact_s = (h > 0 && 2 * light <= s.m) ? 1u : 0u;
    }
    SJBG_BARRIER();
    const uint32_t nh = n_heavy_s;
    for (uint32_t h = threadIdx.x; h < nh; h += blockDim.x) {
        const uint32_t key = ~(uint32_t)sc[h];
        const uint32_t c = (uint32_t)(sc[h] >> 32);
        M.heavy_keys[h] = key;
        atomicSub(&hw[bin_of(key_x(key, kmin, inv))], c);   // light histogram only
    }
    SJBG_BARRIER();
    heavy_set_build(M.heavy_set, M.heavy_keys, nh);

    // ---- light CDF at bin upper edges: in-place exclusive scan, then cdf_j = incl_j / total
    const uint32_t per = kBins / blockDim.x;   // 64
    const uint32_t b0 = threadIdx.x * per;
    uint32_t loc = 0;
    for (uint32_t i = 0; i < per; i++) loc += hw[b0 + i];
    uint32_t tot;
    const uint32_t ex = warp_excl_scan(loc, &tot);
    if (lane_id() == 31) warp_tot[warp_id()] = ex + loc;
    SJBG_BARRIER();
    if (warp_id() == 0) {
        uint32_t x = warp_tot[lane_id()], tt;
        const uint32_t e = warp_excl_scan(x, &tt);
        warp_tot[lane_id()] = e;
        if (lane_id() == 31) light_total_s = e + x;
    }
    SJBG_BARRIER();
    const uint32_t total = light_total_s;
    uint32_t run = warp_tot[warp_id()] + ex;
    for (uint32_t i = 0; i < per; i++) {
        run += hw[b0 + i];
        hw[b0 + i] = run;   // inclusive count at the bin's upper edge
    }
    if (threadIdx.x < kMaxLeaves) {
        for (int q = 0; q < 5; q++) ls[threadIdx.x][q] = 0.0f;
        lmin[threadIdx.x] = 2.0f;
        lmax[threadIdx.x] = -1.0f;
    }
    if (threadIdx.x < 4) rootsum[threadIdx.x] = 0.0;
    SJBG_BARRIER();
    const float invt = total ? 1.0f / (float)total : 0.0f;

    // ---- root line y = a x + b over all bin points (x_j = (j+1)/kBins, y_j = cdf_j)
    double sx = 0, sy = 0, sxx = 0, sxy = 0;
    for (uint32_t i = 0; i < per; i++) {
        const uint32_t j = b0 + i;
        const double x = (double)(j + 1) / kBins, y = (double)hw[j] * invt;
        sx += x; sy += y; sxx += x * x; sxy += x * y;
    }
    for (int o = 16; o > 0; o >>= 1) {
        sx += __shfl_xor_sync(0xFFFFFFFFu, sx, o);
        sy += __shfl_xor_sync(0xFFFFFFFFu, sy, o);
        sxx += __shfl_xor_sync(0xFFFFFFFFu, sxx, o);
        sxy += __shfl_xor_sync(0xFFFFFFFFu, sxy, o);
    }
    if (lane_id() == 0) {
        atomicAdd(&rootsum[0], sx);
        atomicAdd(&rootsum[1], sy);
        atomicAdd(&rootsum[2], sxx);
        atomicAdd(&rootsum[3], sxy);
    }
    SJBG_BARRIER();
    const double nn = kBins;
    const double den = nn * rootsum[2] - rootsum[0] * rootsum[0];
    double ra = den != 0.0 ? (nn * rootsum[3] - rootsum[0] * rootsum[1]) / den : 1.0;
    if (!(ra > 0.0)) ra = 1.0;   // the root must increase with the key
    const double rb = (rootsum[1] - ra * rootsum[0]) / nn;
    const float root_a = (float)ra, root_b = (float)rb;
    auto leaf_of = [&](float x) {
        int l = (int)floorf((root_a * x + root_b) * (float)leaves);
        return min(max(l, 0), (int)leaves - 1);
    };

    // ---- leaf lines, pass 1: counts and means; pass 2: centred products
    // a thread's bins are consecutive, so they fall into one or two leaves:
    // sums are kept in registers per run of equal leaves and flushed on change
    {
        int cur = -1;
        float c0 = 0.f, c1 = 0.f, c2 = 0.f, mn = 2.f, mxv = -1.f;
        for (uint32_t i = 0; i <= per; i++) {
            int l = -1;
            float x = 0.f, y = 0.f;
            if (i < per) {
                const uint32_t j = b0 + i;
                x = (float)(j + 1) / kBins;
                y = (float)hw[j] * invt;
                l = leaf_of(x);
            }
            if (l != cur) {
                if (cur >= 0) {
                    atomicAdd(&ls[cur][0], c0);
                    atomicAdd(&ls[cur][1], c1);
                    atomicAdd(&ls[cur][2], c2);
                    atomicMin(reinterpret_cast<int *>(&lmin[cur]), __float_as_int(mn));  // y >= 0: int order == float order
                    atomicMax(reinterpret_cast<int *>(&lmax[cur]), __float_as_int(mxv));
                }
                cur = l;
                c0 = c1 = c2 = 0.f;
                mn = 2.f;
                mxv = -1.f;
            }
            if (l >= 0) {
                c0 += 1.f; c1 += x; c2 += y;
                mn = fminf(mn, y);
                mxv = fmaxf(mxv, y);
            }
        }
    }
    SJBG_BARRIER();
    {
        int cur = -1;
        float sxy = 0.f, sxx = 0.f, mx = 0.f, my = 0.f;
        for (uint32_t i = 0; i <= per; i++) {
            int l = -1;
            float x = 0.f, y = 0.f;
            if (i < per) {
                const uint32_t j = b0 + i;
                x = (float)(j + 1) / kBins;
                y = (float)hw[j] * invt;
                l = leaf_of(x);
            }
            if (l != cur) {
                if (cur >= 0) {
                    atomicAdd(&ls[cur][3], sxy);
                    atomicAdd(&ls[cur][4], sxx);
                }
                cur = l;
                sxy = sxx = 0.f;
                if (l >= 0) {
                    mx = ls[l][1] / ls[l][0];
                    my = ls[l][2] / ls[l][0];
                }
            }
            if (l >= 0) {
                const float dx = x - mx, dy = y - my;
                sxy += dx * dy;
                sxx += dx * dx;
            }
        }
    }
    SJBG_BARRIER();
    if (threadIdx.x == 0) {
        // monotone clamps: empty leaves inherit the previous upper bound
        float prev = 0.0f;
        for (uint32_t l = 0; l < leaves; l++) {
            const float n = ls[l][0];
            float lo, hi, slope, mx, my;
            if (n < 1.0f) {
                lo = hi = prev; slope = 0.0f; mx = 0.0f; my = prev;
            } else {
                mx = ls[l][1] / n; my = ls[l][2] / n;
                slope = ls[l][4] > 0.0f ? ls[l][3] / ls[l][4] : 0.0f;
                if (!(slope >= 0.0f)) slope = 0.0f;
                // the leaf owns the CDF range from the previous leaf's top to its own
                // largest sampled value: contiguous, non-overlapping, increasing ranges
                lo = prev;
                hi = fmaxf(lmax[l], lo);
            }
            M.slope[l] = slope; M.mean_x[l] = mx; M.mean_y[l] = my; M.lo[l] = lo; M.hi[l] = hi;
            prev = hi;
        }
        M.kmin = kmin; M.inv_range = inv; M.root_a = root_a; M.root_b = root_b;
        M.leaves = leaves; M.log2_buckets = log2_eff_s; M.fallback = (total == 0 && nh == 0) ? 1u : 0u; M.n_heavy = nh;
        M.compact = compact_s;
    }
}

// Inference on the sample: predicted bucket sizes of the light keys.
__global__ void __launch_bounds__(kSampleThreads)
learned_check_kernel(const sjbg_tuple *L, const sjbg_tuple *R, const SampleWin *wins, const LearnedModel *models,
                     uint32_t *pred) {
    __shared__ HeavySet hs;
    __shared__ LearnedCore core;
    const uint32_t w = blockIdx.y;
    const SampleWin s = wins[w];
    const LearnedModel *m = &models[w];
    if (m->fallback) return;   // whole CTA
    heavy_set_load(hs, m);
    copy_to_smem(&core, m, sizeof(LearnedCore));
    uint32_t *pw = pred + (uint64_t)w * kPredStride;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < s.m; i += gridDim.x * blockDim.x) {
        const uint32_t k = sample_key(s, L, R, i);
        if (heavy_find(hs, k) != kHeavyBucket) continue;
        atomicAdd(&pw[learned_bucket(core, k)], 1u);
    }
}

// One CTA per window: worst predicted bucket vs the mean -> fallback flag.
__global__ void __launch_bounds__(1024)
learned_overflow_kernel(const SampleWin *wins, LearnedModel *models, const uint32_t *pred, float bound) {
    __shared__ uint32_t mx_s, sum_s;
    const uint32_t w = blockIdx.x;
    LearnedModel &M = models[w];
    if (M.fallback) return;
    if (threadIdx.x == 0) { mx_s = 0; sum_s = 0; }
    SJBG_BARRIER();
    const uint32_t P = 1u << M.log2_buckets;
    const uint32_t *pw = pred + (uint64_t)w * kPredStride;
    uint32_t mx = 0, sm = 0;
    for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) { mx = max(mx, pw[i]); sm += pw[i]; }
    atomicMax(&mx_s, mx);
    atomicAdd(&sum_s, sm);
    SJBG_BARRIER();
    if (threadIdx.x == 0) {
        const float mean = (float)sum_s / (float)P;
        // a window whose light sample is too small to judge keeps its model
        if (sum_s >= 4 * P && (float)mx_s > bound * mean) M.fallback = 1u;
    }
}

__global__ void set_model_kernel(WinPlan *plan, uint32_t n) {
    uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w < n) plan[w].model = w;
}

uint32_t learned_log2_buckets(sjbg_handle *h, uint64_t n_left) {
    if (h->cfg.radix_bits) return h->cfg.radix_bits;
    uint32_t b = 0;
    while (((uint64_t)h->tune.bucket_target << b) < n_left) b++;
    return b;
}

int learned_prepare(sjbg_handle *h, const sjbg_tuple *dL, const sjbg_tuple *dR, const WinPlan *plan, uint32_t n,
                    WinPlan *dPlan, const LearnedModel **dModels, bool allow_heavy) {
    const float rate = h->cfg.sample_rate > 0.0f ? h->cfg.sample_rate : 0.01f;
    const float bound = h->cfg.overflow_bound > 0.0f ? h->cfg.overflow_bound : 8.0f;
    const uint32_t leaves = h->cfg.learned_leaves ? std::min(h->cfg.learned_leaves, kMaxLeaves) : kMaxLeaves;
    std::vector<SampleWin> sw(n);
    uint64_t table_total = 0;
    uint32_t max_m = 0;
    for (uint32_t w = 0; w < n; w++) {
        const WinPlan &p = plan[w];
        SampleWin &s = sw[w];
        s.left_off = p.left_off; s.n_left = p.n_left; s.right_off = p.right_off; s.n_right = p.n_right;
        const uint64_t nmin = std::min(p.n_left, p.n_right);
        uint64_t m = (uint64_t)((double)rate * (double)(p.n_left + p.n_right));
        m = std::max<uint64_t>(m, 64);
        m = std::min<uint64_t>(m, 2 * nmin);   // at most one sample per tuple
        m &= ~1ull;
        if (nmin == 0) m = 0;
        s.m = (uint32_t)m;
        uint32_t lg = 6;
        while (((uint64_t)1 << lg) < 2 * m) lg++;
        s.table_log2 = lg;
        s.table_off = table_total;
        table_total += (uint64_t)1 << lg;
        s.log2_buckets = p.log2_buckets;
        const uint64_t P = (uint64_t)1 << p.log2_buckets;
        // heavy candidates: keys sampled at least max(4, m / 64P) times; the fit
        // keeps those that exceed an eighth of a bucket of the remaining light mass
        s.thresh = (uint32_t)std::max<uint64_t>(4, m / (64 * P));
        max_m = std::max(max_m, s.m);
    }
    const size_t swB = sizeof(SampleWin) * n, scB = sizeof(SampleScratch) * n;
    const size_t histB = sizeof(uint32_t) * (size_t)kBins * n, tabB = sizeof(unsigned long long) * table_total;
    const size_t candB = sizeof(unsigned long long) * (size_t)kCandMax * n, predB = sizeof(uint32_t) * (size_t)n * kPredStride;
    uint8_t *hst = static_cast<uint8_t *>(pinned_get(h, 1, swB + scB));
    uint8_t *dsmall = static_cast<uint8_t *>(ws_get(h, WS_SAMPLE, swB + scB));
    uint32_t *dHist = static_cast<uint32_t *>(ws_get(h, WS_AUX0, histB + predB));
    unsigned long long *dTab = static_cast<unsigned long long *>(ws_get(h, WS_AUX1, tabB));
    unsigned long long *dCand = static_cast<unsigned long long *>(ws_get(h, WS_AUX2, candB));
    LearnedModel *dM = static_cast<LearnedModel *>(ws_get(h, WS_MODEL, sizeof(LearnedModel) * n));
    if (!hst || !dsmall || !dHist || !dTab || !dCand || !dM) return fail(h, SJBG_E_NOMEM, "learned partitioner buffers");
    uint32_t *dPred = dHist + (size_t)kBins * n;
    std::memcpy(hst, sw.data(), swB);
    SampleScratch init;
    std::memset(&init, 0, sizeof(init));
    init.kmin = 0xFFFFFFFFu;
    std::vector<SampleScratch> scr(n, init);
    std::memcpy(hst + swB, scr.data(), scB);
    if (int rc_up = stage_copy(h, dsmall, hst, swB + scB)) return rc_up;
    SJBG_CK(h, cudaMemsetAsync(dHist, 0, histB + predB, h->stream));
    SJBG_CK(h, cudaMemsetAsync(dTab, 0, tabB, h->stream));
    const SampleWin *dSw = reinterpret_cast<const SampleWin *>(dsmall);
    SampleScratch *dScr = reinterpret_cast<SampleScratch *>(dsmall + swB);

    const uint32_t bx = std::max<uint32_t>(1, std::min<uint32_t>(64, (max_m + 4095) / 4096));
    const dim3 g(bx, n);
    SJBG_CK(h, launch(h, "learned_sample", sample_minmax_kernel, g, dim3(kSampleThreads), 0, dL, dR, dSw, dScr));
    SJBG_CK(h, launch(h, "learned_count", sample_count_kernel, g, dim3(kSampleThreads), 0, dL, dR, dSw,
                      (const SampleScratch *)dScr, dHist, dTab));
    const uint32_t tx = std::max<uint32_t>(1, std::min<uint32_t>(64, (uint32_t)((table_total / n + 4095) / 4096)));
    SJBG_CK(h, launch(h, "learned_classes", heavy_classes_kernel, dim3(tx, n), dim3(kSampleThreads), 0, dSw,
                      (const unsigned long long *)dTab, dScr));
    SJBG_CK(h, launch(h, "learned_heavy", heavy_candidates_kernel, dim3(tx, n), dim3(kSampleThreads), 0, dSw,
                      (const unsigned long long *)dTab, dScr, dCand));
    SJBG_CK(h, launch(h, "learned_fit", learned_fit_kernel, dim3(n), dim3(1024), 0, dSw, dScr, dHist, dCand, dM, leaves,
                      allow_heavy ? kMaxHeavy : 0u, bound));
    SJBG_CK(h, launch(h, "learned_check", learned_check_kernel, g, dim3(kSampleThreads), 0, dL, dR, dSw,
                      (const LearnedModel *)dM, dPred));
    SJBG_CK(h, launch(h, "learned_overflow", learned_overflow_kernel, dim3(n), dim3(1024), 0, dSw, dM,
                      (const uint32_t *)dPred, bound));
    SJBG_CK(h, launch(h, "learned_set_model", set_model_kernel, dim3((n + 255) / 256), dim3(256), 0, dPlan, n));
    *dModels = dM;
    return SJBG_OK;
}

}  // namespace sjbg
