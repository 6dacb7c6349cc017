// nlj.cu - lazy nested-loop join (sm_103a).
//
// Replaces the reference's lazy GPU nested-loop family
// (src/sjb/windowing/lazy/executor/GPU/GPU_NLJ.cu:28-145 and its NoOutput /
// CountKernel / EstimatedSelectivity / Bitmap variants; one thread per pair
// with atomicAggInc, CudaUtils.cuh:8-14), whose matching rule is the lazy
// CPU_NLJ's (src/sjb/windowing/lazy/executor/CPU/CPU_NLJ.cpp:11-32): every
// (left, right) pair of the window is compared.
//
// Design: each thread keeps kLReg left keys in registers; the CTA streams the
// window's right side through shared memory in chunks of kChunk keys (SoA:
// keys and vals, extracted from the 16-byte tuples with vector loads).  The
// hot loop reads four right keys with one 128-bit shared load (a broadcast)
// and folds key equality into one predicate per thread (p |= a == b); every
// 64 right keys the warp votes (__any_sync) and only a warp that saw a match
// re-walks those 64 keys exactly: count, prod and xor checksums, and the
// (left.val, right.val) pairs appended with one atomic per warp
// (__ballot_sync/__popc-style warp aggregation of the reference's atomicAggInc).
#include <algorithm>
#include <cstring>
#include <vector>

#include "nlj.cuh"

namespace sjbg {

struct NljItem {
    uint32_t win, l0, r0, pad;
};

template <bool kEnum, bool kPairs>
__global__ void __launch_bounds__(kNljThreads)
nlj_kernel(const sjbg_tuple *__restrict__ L, const sjbg_tuple *__restrict__ R, const WinPlan *__restrict__ wins,
           const NljItem *__restrict__ items, WinAcc *__restrict__ acc, sjbg_pair *__restrict__ pairs) {
    const NljItem it = items[blockIdx.x];
    const WinPlan wp = wins[it.win];
    nlj_block<kEnum, kPairs>(L + wp.left_off, (uint32_t)wp.n_left, R + wp.right_off, (uint32_t)wp.n_right, it.l0, it.r0,
                             &acc[it.win], nullptr, kPairs ? pairs + wp.pairs_off : nullptr, kPairs ? wp.pairs_cap : 0);
}

// Eager form: one window given by scalar arguments (no uploaded plan, so it
// can be captured in a CUDA graph); blockIdx.x = left tile, blockIdx.y = right split.
template <bool kEnum, bool kPairs>
__global__ void __launch_bounds__(kNljThreads)
nlj_pair_kernel(const sjbg_tuple *__restrict__ L, uint32_t nL, const sjbg_tuple *__restrict__ R, uint32_t nR,
                uint32_t rsplit, WinAcc *acc, unsigned long long *batch_count, sjbg_pair *pairs, uint64_t pairs_cap) {
    nlj_block<kEnum, kPairs>(L, nL, R, nR, blockIdx.x * kLTile, blockIdx.y * rsplit, acc, batch_count, pairs,
                             pairs_cap, rsplit);
}

int nlj_pair_launch(sjbg_handle *h, const sjbg_tuple *L, uint64_t nL, const sjbg_tuple *R, uint64_t nR, WinAcc *acc,
                    unsigned long long *batch_count, sjbg_pair *pairs, uint64_t pairs_cap, bool enumerate) {
    if (nL == 0 || nR == 0) return SJBG_OK;
    // split the right side finely enough that the grid covers every SM twice
    const uint32_t lt = (uint32_t)((nL + kLTile - 1) / kLTile);
    uint32_t rsplit = kRSplit;
    while (rsplit > kChunk && (uint64_t)lt * ((nR + rsplit - 1) / rsplit) < 2ull * h->num_sms) rsplit >>= 1;
    const dim3 grid(lt, (uint32_t)((nR + rsplit - 1) / rsplit));
    if (pairs)
        SJBG_CK(h, launch(h, "eager_nlj_pairs", nlj_pair_kernel<true, true>, grid, dim3(kNljThreads), 0, L,
                          (uint32_t)nL, R, (uint32_t)nR, rsplit, acc, batch_count, pairs, pairs_cap));
    else if (enumerate)
        SJBG_CK(h, launch(h, "eager_nlj_xor", nlj_pair_kernel<true, false>, grid, dim3(kNljThreads), 0, L,
                          (uint32_t)nL, R, (uint32_t)nR, rsplit, acc, batch_count, pairs, pairs_cap));
    else
        SJBG_CK(h, launch(h, "eager_nlj_count", nlj_pair_kernel<false, false>, grid, dim3(kNljThreads), 0, L,
                          (uint32_t)nL, R, (uint32_t)nR, rsplit, acc, batch_count, pairs, pairs_cap));
    return SJBG_OK;
}

// Recorded eager streams (eager_run.cu): one CTA per (window, left batch,
// right batch, left tile); the block pair's matches go to the later batch's
// counter and its checksums to the window.
uint32_t nlj_left_tile() { return kLTile; }

template <bool kEnum>
__global__ void __launch_bounds__(kNljThreads)
eager_nlj_blocks_kernel(const sjbg_tuple *__restrict__ L, const sjbg_tuple *__restrict__ R, uint32_t B,
                        const ERunItem *__restrict__ items, WinAcc *__restrict__ acc,
                        unsigned long long *__restrict__ counts) {
    const ERunItem it = items[blockIdx.x];
    nlj_block<kEnum, false>(L + (uint64_t)it.lb * B, B, R + (uint64_t)it.rb * B, B, it.l0, 0, &acc[it.win],
                            &counts[it.dest], nullptr, 0, B);
}

int eager_nlj_blocks(sjbg_handle *h, const sjbg_tuple *dl, const sjbg_tuple *dr, uint64_t B, const ERunItem *items,
                     uint32_t n_items, WinAcc *acc, unsigned long long *counts, bool enumerate) {
    if (n_items == 0) return SJBG_OK;
    if (B >= 0xFFFFFFFFull) return fail(h, SJBG_E_CAPACITY, "eager batches are limited to 2^32 tuples");
    const size_t itB = sizeof(ERunItem) * n_items;
    uint8_t *hst = static_cast<uint8_t *>(pinned_get(h, 2, itB));
    uint8_t *dev = static_cast<uint8_t *>(ws_get(h, WS_EAGER_META, itB));
    if (!hst || !dev) return fail(h, SJBG_E_NOMEM, "eager run plan");
    std::memcpy(hst, items, itB);
    if (int rc = stage_copy(h, dev, hst, itB)) return rc;
    const ERunItem *dItems = reinterpret_cast<const ERunItem *>(dev);
    if (enumerate)
        SJBG_CK(h, launch(h, "erun_nlj_xor", eager_nlj_blocks_kernel<true>, dim3(n_items), dim3(kNljThreads), 0, dl,
                          dr, (uint32_t)B, dItems, acc, counts));
    else
        SJBG_CK(h, launch(h, "erun_nlj_count", eager_nlj_blocks_kernel<false>, dim3(n_items), dim3(kNljThreads), 0,
                          dl, dr, (uint32_t)B, dItems, acc, counts));
    return SJBG_OK;
}

int nlj_lazy_batch(sjbg_handle *h, const sjbg_tuple *dL, const sjbg_tuple *dR, const WinHost *wins, uint32_t n,
                   sjbg_pair *dPairs, WinAcc *acc, bool enumerate) {
    if (n == 0) return SJBG_OK;
    std::vector<WinPlan> plan(n);
    std::vector<NljItem> items;
    for (uint32_t w = 0; w < n; w++) {
        const WinHost &wh = wins[w];
        if (wh.n_left >= 0xFFFFFFFFull || wh.n_right >= 0xFFFFFFFFull)
            return fail(h, SJBG_E_CAPACITY, "nested-loop windows are limited to 2^32 tuples per side");
        WinPlan &p = plan[w];
        std::memset(&p, 0, sizeof(p));
        p.left_off = wh.left_off; p.n_left = wh.n_left; p.right_off = wh.right_off; p.n_right = wh.n_right;
        p.pairs_off = wh.pairs_off; p.pairs_cap = dPairs ? wh.pairs_cap : 0;
        p.model = 0xFFFFFFFFu;
        for (uint64_t l0 = 0; l0 < wh.n_left; l0 += kLTile)
            for (uint64_t r0 = 0; r0 < wh.n_right; r0 += kRSplit) items.push_back({w, (uint32_t)l0, (uint32_t)r0, 0});
    }
    if (items.empty()) return SJBG_OK;
    const size_t planB = sizeof(WinPlan) * n, itB = sizeof(NljItem) * items.size();
    uint8_t *hst = static_cast<uint8_t *>(pinned_get(h, 0, planB + itB));
    uint8_t *dev = static_cast<uint8_t *>(ws_get(h, WS_WIN_PLAN, planB + itB));
    if (!hst || !dev) return fail(h, SJBG_E_NOMEM, "nested-loop plan");
    std::memcpy(hst, plan.data(), planB);
    std::memcpy(hst + planB, items.data(), itB);
    if (int rc_up = stage_copy(h, dev, hst, planB + itB)) return rc_up;
    const WinPlan *dPlan = reinterpret_cast<const WinPlan *>(dev);
    const NljItem *dItems = reinterpret_cast<const NljItem *>(dev + planB);
    const dim3 grid((uint32_t)items.size());
    if (dPairs)
        SJBG_CK(h, launch(h, "nlj_pairs", nlj_kernel<true, true>, grid, dim3(kNljThreads), 0, dL, dR, dPlan, dItems,
                          acc, dPairs));
    else if (enumerate)
        SJBG_CK(h, launch(h, "nlj_xor", nlj_kernel<true, false>, grid, dim3(kNljThreads), 0, dL, dR, dPlan, dItems,
                          acc, dPairs));
    else
        SJBG_CK(h, launch(h, "nlj_count", nlj_kernel<false, false>, grid, dim3(kNljThreads), 0, dL, dR, dPlan, dItems,
                          acc, dPairs));
    return SJBG_OK;
}

}  // namespace sjbg
