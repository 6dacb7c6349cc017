// eager.cu - eager (per-batch) joins (sm_103a).
//
// Replaces the reference's eager executors behind
// Windowing::Eager::Executor::BaseEagerExecutor
// (include/sjb/windowing/eager/executor/BaseEagerExecutor.hpp:16-20):
// eager CPU_HJ (src/sjb/windowing/eager/executor/CPU/CPU_HJ.cpp:35-82), eager
// GPU_HJ / GPU_HJ_Atomic (eager/executor/GPU/GPU_HJ.cu:33-183), GPU_NLJ /
// GPU_NLJ_BM (GPU_NLJ.cu:10-102) and the uncompiled GPU_SMJ specification
// (GPU_SMJ.cu:37-317).  Each incoming batch joins the other side's state of
// the current window and is then added to its own side's state, so a pair is
// counted once, by the later of its two batches.
//
// State per side (device): the side's tuples in arrival order, plus
//   HJ   an open-addressing table keyed by key: {count, sum of the side's pair
//        hash, head of a chain of tuple indices}; probing gives count and
//        prod in O(1) per tuple, the chain gives the pairs;
//   NLJ  nothing more: the batch is compared with every tuple of the other
//        side (nlj.cu's register-blocked block routine);
//   SMJ  the side's tuples sorted by key and prefix sums of its pair hash;
//        a batch is sorted by one CTA (bitonic, shared memory), probed by
//        binary search into the other side's sorted run, then merged into
//        its own run (each element's output rank = own index + rank in the
//        other input), and the prefix sums are recomputed.
// These per-batch kernels serve sjbg_eager_execute (the reference's
// per-batch interface); sjbg_eager_run, which has the whole recorded stream,
// computes the same results in a few launches (eager_run.cu).
#include <algorithm>
#include <cstring>
#include <vector>

#include "eager_dev.cuh"

namespace sjbg {

int nlj_pair_launch(sjbg_handle *h, const sjbg_tuple *L, uint64_t nL, const sjbg_tuple *R, uint64_t nR, WinAcc *acc,
                    unsigned long long *batch_count, sjbg_pair *pairs, uint64_t pairs_cap, bool enumerate);

constexpr uint32_t kPrefixTile = 4096;

EagerState::~EagerState() {
    pk.reset();   // the persistent kernel (if any) has returned before its buffers go
    for (void *p : allocs) cudaFree(p);
}

// ---------------------------------------------------------------- hash join
template <bool kEnum, bool kPairs>
__global__ void __launch_bounds__(256)
eager_hj_kernel(const sjbg_tuple *__restrict__ batch, uint32_t n, uint32_t base, int side, ETab own, ETab oth,
                const sjbg_tuple *__restrict__ oth_tuples, uint32_t oth_n, WinAcc *acc, unsigned long long *bcount,
                sjbg_pair *__restrict__ pairs, uint64_t pcap) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < n;
    uint32_t key = 0, val = 0;
    if (valid) {
        const uint2 t = *reinterpret_cast<const uint2 *>(batch + i);
        key = t.x;
        val = t.y;
    }
    eager_hj_step<kEnum, kPairs>(valid, key, val, base + i, side, own, oth, oth_tuples, oth_n, acc, bcount, pairs,
                                 pcap);
}

// ---------------------------------------------------------------- sort-merge join
// One CTA sorts n <= kEagerMaxSortBatch (key, val) pairs (bitonic on key<<32|val).
__global__ void __launch_bounds__(1024)
eager_sort_batch_kernel(const sjbg_tuple *__restrict__ batch, uint32_t n, uint32_t *__restrict__ out_keys,
                        uint32_t *__restrict__ out_vals) {
    extern __shared__ unsigned long long sv[];
    uint32_t P = 1;
    while (P < n) P <<= 1;
    for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
        if (i < n) {
            const uint2 t = *reinterpret_cast<const uint2 *>(batch + i);
            sv[i] = ((unsigned long long)t.x << 32) | t.y;
        } else {
            sv[i] = ~0ull;
        }
    }
    SJBG_BARRIER();
    for (uint32_t k = 2; k <= P; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
                const uint32_t p = i ^ j;
                if (p > i) {
                    const bool up = (i & k) == 0;
                    const unsigned long long a = sv[i], b = sv[p];
                    if (up ? (a > b) : (a < b)) { sv[i] = b; sv[p] = a; }
                }
            }
            SJBG_BARRIER();
        }
    }
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        out_keys[i] = (uint32_t)(sv[i] >> 32);
        out_vals[i] = (uint32_t)sv[i];
    }
}

template <bool kEnum, bool kPairs>
__global__ void __launch_bounds__(256)
eager_smj_probe_kernel(const uint32_t *__restrict__ bkeys, const uint32_t *__restrict__ bvals, uint32_t n, int side,
                       const uint32_t *__restrict__ okeys, const uint32_t *__restrict__ ovals,
                       const unsigned long long *__restrict__ oF, uint32_t on, WinAcc *acc, unsigned long long *bcount,
                       sjbg_pair *__restrict__ pairs, uint64_t pcap) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t lo = 0, hi = 0, val = 0;
    unsigned long long count = 0, xr = 0, prod = 0;
    if (i < n) {
        const uint32_t key = bkeys[i];
        val = bvals[i];
        lo = lower_bound_u32(okeys, on, key);
        hi = lo < on && okeys[lo] == key ? upper_bound_u32(okeys, on, key) : lo;
        count = hi - lo;
        prod = own_hash(side, val) * (oF[hi] - oF[lo]);
        if (kEnum)
            for (uint32_t a = lo; a < hi; a++)
                xr ^= side == 0 ? sjbg_pair_hash(val, ovals[a]) : sjbg_pair_hash(ovals[a], val);
    }
    if (kPairs) {
        const uint32_t mine = hi - lo;
        uint32_t tot;
        const uint32_t ex = warp_excl_scan(mine, &tot);
        unsigned long long b = 0;
        if (lane_id() == 0 && tot) b = atomicAdd(&acc->npairs, (unsigned long long)tot);
        b = __shfl_sync(0xFFFFFFFFu, b, 0) + ex;
        for (uint32_t a = lo; a < hi; a++, b++)
            if (b < pcap) pairs[b] = side == 0 ? sjbg_pair{val, ovals[a]} : sjbg_pair{ovals[a], val};
    }
    flush_batch(acc, bcount, count, xr, prod);
}

// Merge the sorted run A (na) with the sorted batch B (nb) into out: equal
// keys keep A first; every element's output rank = own index + rank in the other input.
__global__ void __launch_bounds__(256)
eager_merge_kernel(const uint32_t *__restrict__ ak, const uint32_t *__restrict__ av, uint32_t na,
                   const uint32_t *__restrict__ bk, const uint32_t *__restrict__ bv, uint32_t nb,
                   uint32_t *__restrict__ ok, uint32_t *__restrict__ ov) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < na) {
        const uint32_t k = ak[t];
        const uint32_t p = t + lower_bound_u32(bk, nb, k);
        ok[p] = k;
        ov[p] = av[t];
    } else if (t < na + nb) {
        const uint32_t j = t - na;
        const uint32_t k = bk[j];
        const uint32_t p = j + upper_bound_u32(ak, na, k);
        ok[p] = k;
        ov[p] = bv[j];
    }
}

// Prefix sums of the side's pair hash over a sorted run: F[i] = sum over [0, i), i in [0, n].
__global__ void __launch_bounds__(256)
eager_prefix_tiles_kernel(const uint32_t *__restrict__ vals, uint32_t n, int side, unsigned long long *tsum) {
    __shared__ unsigned long long ws[8];
    const uint32_t base = blockIdx.x * kPrefixTile;
    unsigned long long acc = 0;
    for (uint32_t i = threadIdx.x; i < kPrefixTile; i += blockDim.x)
        if (base + i < n) acc += own_hash(side, vals[base + i]);
    acc = warp_sum_u64(acc);
    if (lane_id() == 0) ws[warp_id()] = acc;
    SJBG_BARRIER();
    if (threadIdx.x == 0) {
        unsigned long long s = 0;
        for (int i = 0; i < 8; i++) s += ws[i];
        tsum[blockIdx.x] = s;
    }
}

__global__ void eager_prefix_scan_kernel(unsigned long long *tsum, uint32_t tiles) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        unsigned long long run = 0;
        for (uint32_t t = 0; t < tiles; t++) {
            const unsigned long long v = tsum[t];
            tsum[t] = run;
            run += v;
        }
    }
}

__global__ void __launch_bounds__(256)
eager_prefix_apply_kernel(const uint32_t *__restrict__ vals, uint32_t n, int side,
                          const unsigned long long *__restrict__ tsum, unsigned long long *__restrict__ F) {
    __shared__ unsigned long long wsum[8];
    const uint32_t base = blockIdx.x * kPrefixTile;
    constexpr uint32_t kPer = kPrefixTile / 256;
    const uint32_t b0 = base + threadIdx.x * kPer;
    unsigned long long loc = 0;
    for (uint32_t i = 0; i < kPer; i++)
        if (b0 + i < n) loc += own_hash(side, vals[b0 + i]);
    unsigned long long x = loc;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane_id() >= (uint32_t)o) x += y;
    }
    if (lane_id() == 31) wsum[warp_id()] = x;
    SJBG_BARRIER();
    unsigned long long wofs = 0;
    for (uint32_t w = 0; w < warp_id(); w++) wofs += wsum[w];
    unsigned long long run = tsum[blockIdx.x] + wofs + x - loc;
    for (uint32_t i = 0; i < kPer; i++) {
        const uint32_t li = b0 + i;
        if (li <= n) F[li] = run;
        if (li < n) run += own_hash(side, vals[li]);
    }
}

// ---------------------------------------------------------------- host side
static void *ealloc(EagerState &st, size_t bytes) {
    void *p = nullptr;
    if (cudaMalloc(&p, bytes ? bytes : 16) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    st.allocs.push_back(p);
    return p;
}

int eager_init(sjbg_handle *h) {
    auto st = std::make_unique<EagerState>();
    const sjbg_config &c = h->cfg;
    if (c.algorithm == SJBG_ALG_SMJ && c.batch_size > kEagerMaxSortBatch)
        return fail(h, SJBG_E_UNSUPPORTED, "eager sort-merge batches are limited to 8192 tuples");
    st->cap = std::max(c.max_tuples_per_window, c.window_size) + c.batch_size;
    if (st->cap >= 0x7FFFFFFFull) return fail(h, SJBG_E_CAPACITY, "eager windows are limited to 2^31 tuples per side");
    uint32_t bits = 4;
    while ((1ull << bits) < 2 * st->cap) bits++;
    st->table_bits = bits;
    const uint64_t C = 1ull << bits;
    for (int s = 0; s < 2; s++) {
        EagerSide &S = st->side[s];
        S.tuples = static_cast<sjbg_tuple *>(ealloc(*st, sizeof(sjbg_tuple) * st->cap));
        if (!S.tuples) return fail(h, SJBG_E_NOMEM, "eager state");
        if (c.algorithm == SJBG_ALG_HJ) {
            S.tkeys = static_cast<uint32_t *>(ealloc(*st, 4 * (C + 1)));
            S.tcnt = static_cast<uint32_t *>(ealloc(*st, 4 * (C + 1)));
            S.thead = static_cast<uint32_t *>(ealloc(*st, 4 * (C + 1)));
            S.tsum = static_cast<unsigned long long *>(ealloc(*st, 8 * (C + 1)));
            S.next = static_cast<uint32_t *>(ealloc(*st, 4 * st->cap));
            if (!S.tkeys || !S.tcnt || !S.thead || !S.tsum || !S.next) return fail(h, SJBG_E_NOMEM, "eager tables");
        } else if (c.algorithm == SJBG_ALG_SMJ) {
            S.skeys = static_cast<uint32_t *>(ealloc(*st, 4 * st->cap));
            S.svals = static_cast<uint32_t *>(ealloc(*st, 4 * st->cap));
            S.skeys2 = static_cast<uint32_t *>(ealloc(*st, 4 * st->cap));
            S.svals2 = static_cast<uint32_t *>(ealloc(*st, 4 * st->cap));
            S.F = static_cast<unsigned long long *>(ealloc(*st, 8 * (st->cap + kPrefixTile)));
            if (!S.skeys || !S.svals || !S.skeys2 || !S.svals2 || !S.F) return fail(h, SJBG_E_NOMEM, "eager runs");
        }
    }
    if (c.algorithm == SJBG_ALG_SMJ) {
        st->sort_tmp = static_cast<uint32_t *>(ealloc(*st, 4 * 2 * kEagerMaxSortBatch));
        if (!st->sort_tmp) return fail(h, SJBG_E_NOMEM, "eager sort buffer");
    }
    st->acc = static_cast<WinAcc *>(ealloc(*st, sizeof(WinAcc)));
    st->batch_count = static_cast<unsigned long long *>(ealloc(*st, 64));
    if (!st->acc || !st->batch_count) return fail(h, SJBG_E_NOMEM, "eager accumulators");
    if (c.result_mode != SJBG_RESULT_NO_OUTPUT) {
        st->pairs_cap = 4 * st->cap;
        st->pairs = static_cast<sjbg_pair *>(ealloc(*st, sizeof(sjbg_pair) * st->pairs_cap));
        if (!st->pairs) return fail(h, SJBG_E_NOMEM, "eager pair buffer");
    }
    h->eager = std::move(st);
    return SJBG_OK;
}

static int eager_clear(sjbg_handle *h);

// Allocate and clear (fresh device memory holds no valid table, run or total).
int eager_init_and_clear(sjbg_handle *h) {
    int rc = eager_init(h);
    if (rc) return rc;
    rc = eager_clear(h);
    if (rc) return rc;
    SJBG_CK(h, cudaStreamSynchronize(h->stream));
    return SJBG_OK;
}

static bool eager_enumerates(const sjbg_handle *h) {
    return h->cfg.result_mode != SJBG_RESULT_NO_OUTPUT || (h->cfg.flags & SJBG_F_XOR);
}

// Reset both sides (asynchronous; BaseEagerExecutor::clearStates).
static int eager_clear(sjbg_handle *h) {
    EagerState &st = *h->eager;
    const uint64_t C = 1ull << st.table_bits;
    for (int s = 0; s < 2; s++) {
        EagerSide &S = st.side[s];
        S.n = 0;
        if (S.tkeys) {
            SJBG_CK(h, cudaMemsetAsync(S.tkeys, 0xFF, 4 * (C + 1), h->stream));
            SJBG_CK(h, cudaMemsetAsync(S.thead, 0xFF, 4 * (C + 1), h->stream));
            SJBG_CK(h, cudaMemsetAsync(S.tcnt, 0, 4 * (C + 1), h->stream));
            SJBG_CK(h, cudaMemsetAsync(S.tsum, 0, 8 * (C + 1), h->stream));
        }
        if (S.F) SJBG_CK(h, cudaMemsetAsync(S.F, 0, 8, h->stream));   // F[0] = 0 for an empty run
    }
    SJBG_CK(h, cudaMemsetAsync(st.acc, 0, sizeof(WinAcc), h->stream));
    return SJBG_OK;
}

// Enqueue one batch (no synchronisation); its matches are added to *count_slot.
static int eager_enqueue(sjbg_handle *h, const sjbg_tuple *batch, uint64_t n, int side, bool from_host,
                         unsigned long long *count_slot) {
    EagerState &st = *h->eager;
    EagerSide &S = st.side[side];
    EagerSide &O = st.side[1 - side];
    if (S.n + n > st.cap) return fail(h, SJBG_E_CAPACITY, "eager window exceeds its capacity (window_size + batch_size)");
    if (n == 0) return SJBG_OK;
    if (h->cfg.algorithm == SJBG_ALG_SMJ && n > kEagerMaxSortBatch)
        return fail(h, SJBG_E_UNSUPPORTED, "eager sort-merge batches are limited to 8192 tuples");
    sjbg_tuple *dst = S.tuples + S.n;
    SJBG_CK(h, cudaMemcpyAsync(dst, batch, sizeof(sjbg_tuple) * n,
                               from_host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, h->stream));
    const bool en = eager_enumerates(h);
    sjbg_pair *pairs = st.pairs;
    const uint32_t blocks = (uint32_t)((n + 255) / 256);
    switch (h->cfg.algorithm) {
        case SJBG_ALG_NLJ: {
            EagerSide &Ls = st.side[0], &Rs = st.side[1];
            const sjbg_tuple *L = side == 0 ? dst : Ls.tuples;
            const sjbg_tuple *R = side == 0 ? Rs.tuples : dst;
            const uint64_t nl = side == 0 ? n : Ls.n, nr = side == 0 ? Rs.n : n;
            int rc = nlj_pair_launch(h, L, nl, R, nr, st.acc, count_slot, pairs, st.pairs_cap, en);
            if (rc) return rc;
            break;
        }
        case SJBG_ALG_HJ: {
            const ETab own{S.tkeys, S.tcnt, S.thead, S.next, S.tsum, st.table_bits};
            const ETab oth{O.tkeys, O.tcnt, O.thead, O.next, O.tsum, st.table_bits};
            if (pairs)
                SJBG_CK(h, launch(h, "eager_hj_pairs", eager_hj_kernel<true, true>, dim3(blocks), dim3(256), 0,
                                  (const sjbg_tuple *)dst, (uint32_t)n, (uint32_t)S.n, side, own, oth,
                                  (const sjbg_tuple *)O.tuples, (uint32_t)O.n, st.acc, count_slot, pairs,
                                  st.pairs_cap));
            else if (en)
                SJBG_CK(h, launch(h, "eager_hj_xor", eager_hj_kernel<true, false>, dim3(blocks), dim3(256), 0,
                                  (const sjbg_tuple *)dst, (uint32_t)n, (uint32_t)S.n, side, own, oth,
                                  (const sjbg_tuple *)O.tuples, (uint32_t)O.n, st.acc, count_slot, pairs,
                                  st.pairs_cap));
            else
                SJBG_CK(h, launch(h, "eager_hj_count", eager_hj_kernel<false, false>, dim3(blocks), dim3(256), 0,
                                  (const sjbg_tuple *)dst, (uint32_t)n, (uint32_t)S.n, side, own, oth,
                                  (const sjbg_tuple *)O.tuples, (uint32_t)O.n, st.acc, count_slot, pairs,
                                  st.pairs_cap));
            break;
        }
        case SJBG_ALG_SMJ: {
            uint32_t *bk = st.sort_tmp, *bv = st.sort_tmp + kEagerMaxSortBatch;
            uint32_t P = 1;
            while (P < n) P <<= 1;
            allow_big_smem(eager_sort_batch_kernel, sizeof(unsigned long long) * kEagerMaxSortBatch);
            SJBG_CK(h, launch(h, "eager_sort_batch", eager_sort_batch_kernel, dim3(1), dim3(1024),
                              sizeof(unsigned long long) * P, (const sjbg_tuple *)dst, (uint32_t)n, bk, bv));
            if (pairs)
                SJBG_CK(h, launch(h, "eager_smj_probe_pairs", eager_smj_probe_kernel<true, true>, dim3(blocks),
                                  dim3(256), 0, (const uint32_t *)bk, (const uint32_t *)bv, (uint32_t)n, side,
                                  (const uint32_t *)O.skeys, (const uint32_t *)O.svals,
                                  (const unsigned long long *)O.F, (uint32_t)O.n, st.acc, count_slot, pairs,
                                  st.pairs_cap));
            else if (en)
                SJBG_CK(h, launch(h, "eager_smj_probe_xor", eager_smj_probe_kernel<true, false>, dim3(blocks),
                                  dim3(256), 0, (const uint32_t *)bk, (const uint32_t *)bv, (uint32_t)n, side,
                                  (const uint32_t *)O.skeys, (const uint32_t *)O.svals,
                                  (const unsigned long long *)O.F, (uint32_t)O.n, st.acc, count_slot, pairs,
                                  st.pairs_cap));
            else
                SJBG_CK(h, launch(h, "eager_smj_probe_count", eager_smj_probe_kernel<false, false>, dim3(blocks),
                                  dim3(256), 0, (const uint32_t *)bk, (const uint32_t *)bv, (uint32_t)n, side,
                                  (const uint32_t *)O.skeys, (const uint32_t *)O.svals,
                                  (const unsigned long long *)O.F, (uint32_t)O.n, st.acc, count_slot, pairs,
                                  st.pairs_cap));
            const uint32_t nt = (uint32_t)(S.n + n);
            SJBG_CK(h, launch(h, "eager_merge", eager_merge_kernel, dim3((nt + 255) / 256), dim3(256), 0,
                              (const uint32_t *)S.skeys, (const uint32_t *)S.svals, (uint32_t)S.n,
                              (const uint32_t *)bk, (const uint32_t *)bv, (uint32_t)n, S.skeys2, S.svals2));
            std::swap(S.skeys, S.skeys2);
            std::swap(S.svals, S.svals2);
            const uint32_t tiles = (nt + 1 + kPrefixTile - 1) / kPrefixTile;
            unsigned long long *tsum = static_cast<unsigned long long *>(ws_get(h, WS_AUX3, 8 * tiles));
            if (!tsum) return fail(h, SJBG_E_NOMEM, "eager prefix buffer");
            SJBG_CK(h, launch(h, "eager_prefix_tiles", eager_prefix_tiles_kernel, dim3(tiles), dim3(256), 0,
                              (const uint32_t *)S.svals, nt, side, tsum));
            SJBG_CK(h, launch(h, "eager_prefix_scan", eager_prefix_scan_kernel, dim3(1), dim3(32), 0, tsum, tiles));
            SJBG_CK(h, launch(h, "eager_prefix_apply", eager_prefix_apply_kernel, dim3(tiles), dim3(256), 0,
                              (const uint32_t *)S.svals, nt, side, (const unsigned long long *)tsum, S.F));
            break;
        }
        default:
            return fail(h, SJBG_E_UNSUPPORTED, "unknown algorithm");
    }
    S.n += n;
    return SJBG_OK;
}

static void fill_eager_result(const sjbg_handle *h, const WinAcc &a, sjbg_window_result *out) {
    std::memset(out, 0, sizeof(*out));
    out->count = a.count;
    out->prod_checksum = a.prod;
    if (eager_enumerates(h)) {
        out->xor_checksum = a.xr;
        out->flags |= SJBG_WR_XOR;
    }
    const uint64_t cap = h->eager->pairs_cap;
    out->n_pairs = h->eager->pairs ? std::min<uint64_t>(a.npairs, cap) : 0;
    if (h->eager->pairs && a.npairs > cap) out->flags |= SJBG_WR_PAIRS_TRUNCATED;
    out->partitioner_used = SJBG_PART_NONE;
}

static int eager_check(sjbg_handle *h) {
    if (!h) return SJBG_E_INVALID;
    if (h->cfg.progressiveness != SJBG_EAGER || !h->eager) return fail(h, SJBG_E_STATE, "eager call on a lazy handle");
    SJBG_CK(h, cudaSetDevice(h->device));
    return SJBG_OK;
}

static bool persistent(const sjbg_handle *h) { return (h->cfg.flags & SJBG_F_PERSISTENT) != 0; }

int eager_shutdown(sjbg_handle *h) {
    if (!h->eager || !h->eager->pk) return SJBG_OK;
    cudaSetDevice(h->device);
    return pk_stop(h, false);
}

}  // namespace sjbg

using namespace sjbg;

extern "C" {

int sjbg_eager_execute(sjbg_handle *h, const sjbg_tuple *batch, uint64_t n, int is_left, uint32_t mem,
                       uint64_t *match_count) {
    int rc = eager_check(h);
    if (rc) return rc;
    if ((n && !batch) || (mem != SJBG_MEM_HOST && mem != SJBG_MEM_DEVICE)) return fail(h, SJBG_E_INVALID, "bad batch");
    if (persistent(h)) return pk_execute(h, batch, n, is_left ? 0 : 1, mem == SJBG_MEM_HOST, match_count);
    EagerState &st = *h->eager;
    SJBG_CK(h, cudaMemsetAsync(st.batch_count, 0, 8, h->stream));
    rc = eager_enqueue(h, batch, n, is_left ? 0 : 1, mem == SJBG_MEM_HOST, st.batch_count);
    if (rc) return rc;
    unsigned long long *hc = static_cast<unsigned long long *>(pinned_get(h, 5, 64));
    if (!hc) return fail(h, SJBG_E_NOMEM, "count staging");
    SJBG_CK(h, cudaMemcpyAsync(hc, st.batch_count, 8, cudaMemcpyDeviceToHost, h->stream));
    SJBG_CK(h, cudaStreamSynchronize(h->stream));
    profile_collect(h);
    if (match_count) *match_count = hc[0];
    return SJBG_OK;
}

int sjbg_eager_clear_states(sjbg_handle *h) {
    int rc = eager_check(h);
    if (rc) return rc;
    if (persistent(h)) return pk_clear_states(h);
    rc = eager_clear(h);
    if (rc) return rc;
    SJBG_CK(h, cudaStreamSynchronize(h->stream));
    return SJBG_OK;
}

int sjbg_eager_window_result(sjbg_handle *h, sjbg_pair *pairs, uint64_t pairs_capacity, sjbg_window_result *out) {
    int rc = eager_check(h);
    if (rc) return rc;
    if (!out) return fail(h, SJBG_E_INVALID, "null result");
    if (persistent(h)) {   // the totals after every ticket posted so far
        WinAcc totals;
        if ((rc = pk_report(h, &totals))) return rc;
        fill_eager_result(h, totals, out);
    } else {
        WinAcc *ha = static_cast<WinAcc *>(pinned_get(h, 3, sizeof(WinAcc)));
        if (!ha) return fail(h, SJBG_E_NOMEM, "result staging");
        SJBG_CK(h, cudaMemcpyAsync(ha, h->eager->acc, sizeof(WinAcc), cudaMemcpyDeviceToHost, h->stream));
        SJBG_CK(h, cudaStreamSynchronize(h->stream));
        fill_eager_result(h, *ha, out);
    }
    if (pairs && h->eager->pairs) {
        const uint64_t np = std::min(out->n_pairs, pairs_capacity);
        if (np) {   // (on the handle's stream: a running persistent kernel does not block the copy)
            SJBG_CK(h, cudaMemcpyAsync(pairs, h->eager->pairs, sizeof(sjbg_pair) * np, cudaMemcpyDeviceToHost,
                                       h->stream));
            SJBG_CK(h, cudaStreamSynchronize(h->stream));
        }
        if (np < out->n_pairs) out->flags |= SJBG_WR_PAIRS_TRUNCATED;
        out->n_pairs = np;
    } else {
        out->n_pairs = 0;
    }
    return SJBG_OK;
}

int sjbg_eager_end_of_stream(sjbg_handle *h) {
    int rc = eager_check(h);
    if (rc) return rc;
    if (persistent(h) && (rc = pk_stop(h, false))) return rc;
    SJBG_CK(h, cudaStreamSynchronize(h->stream));
    return SJBG_OK;
}

int sjbg_eager_post(sjbg_handle *h, const sjbg_tuple *batch, uint64_t n, int is_left, uint32_t mem,
                    uint64_t *ticket) {
    int rc = eager_check(h);
    if (rc) return rc;
    if (!persistent(h)) return fail(h, SJBG_E_STATE, "sjbg_eager_post needs an SJBG_F_PERSISTENT handle");
    if ((n && !batch) || (mem != SJBG_MEM_HOST && mem != SJBG_MEM_DEVICE)) return fail(h, SJBG_E_INVALID, "bad batch");
    return pk_post_batch(h, batch, n, is_left ? 0 : 1, mem == SJBG_MEM_HOST, ticket);
}

int sjbg_eager_wait(sjbg_handle *h, uint64_t ticket, uint64_t *match_count) {
    int rc = eager_check(h);
    if (rc) return rc;
    if (!persistent(h)) return fail(h, SJBG_E_STATE, "sjbg_eager_wait needs an SJBG_F_PERSISTENT handle");
    return pk_wait_batch(h, ticket, match_count);
}

int sjbg_eager_pk_status(sjbg_handle *h, int *running, uint64_t *launches) {
    int rc = eager_check(h);
    if (rc) return rc;
    if (!persistent(h)) return fail(h, SJBG_E_STATE, "not an SJBG_F_PERSISTENT handle");
    return pk_status(h, running, launches);
}

int sjbg_eager_run(sjbg_handle *h, const sjbg_tuple *left, const sjbg_tuple *right, uint64_t n_batches, uint32_t mem,
                   uint64_t *batch_counts, sjbg_window_result *out, uint32_t n_windows_out) {
    int rc = eager_check(h);
    if (rc) return rc;
    if (n_batches && (!left || !right)) return fail(h, SJBG_E_INVALID, "null stream");
    // the whole-stream path replaces the window state a persistent kernel keeps
    if (persistent(h) && (rc = pk_stop(h, true))) return rc;
    const uint64_t B = h->cfg.batch_size;
    // host streams are copied to the device once
    const sjbg_tuple *dl = left, *dr = right;
    if (mem == SJBG_MEM_HOST && n_batches) {
        sjbg_tuple *sl = static_cast<sjbg_tuple *>(ws_get(h, WS_IN_LEFT, sizeof(sjbg_tuple) * B * n_batches));
        sjbg_tuple *sr = static_cast<sjbg_tuple *>(ws_get(h, WS_IN_RIGHT, sizeof(sjbg_tuple) * B * n_batches));
        if (!sl || !sr) return fail(h, SJBG_E_NOMEM, "stream staging");
        SJBG_CK(h, cudaMemcpyAsync(sl, left, sizeof(sjbg_tuple) * B * n_batches, cudaMemcpyHostToDevice, h->stream));
        SJBG_CK(h, cudaMemcpyAsync(sr, right, sizeof(sjbg_tuple) * B * n_batches, cudaMemcpyHostToDevice, h->stream));
        dl = sl;
        dr = sr;
    }
    unsigned long long *dCounts = static_cast<unsigned long long *>(ws_get(h, WS_AUX0, 8 * std::max<uint64_t>(2 * n_batches, 1)));
    WinAcc *dWin = static_cast<WinAcc *>(ws_get(h, WS_AUX1, sizeof(WinAcc) * (2 * n_batches + 3)));
    if (!dCounts || !dWin) return fail(h, SJBG_E_NOMEM, "eager run buffers");
    rc = eager_clear(h);
    if (rc) return rc;
    uint32_t windows = 0;
    rc = eager_run_batched(h, dl, dr, n_batches, eager_enumerates(h), dCounts, dWin, &windows);
    if (rc) return rc;
    std::vector<WinAcc> hw(windows + 1);
    if (batch_counts && n_batches)
        SJBG_CK(h, cudaMemcpyAsync(batch_counts, dCounts, 8 * 2 * n_batches, cudaMemcpyDeviceToHost, h->stream));
    SJBG_CK(h, cudaMemcpyAsync(hw.data(), dWin, sizeof(WinAcc) * (windows + 1), cudaMemcpyDeviceToHost, h->stream));
    SJBG_CK(h, cudaStreamSynchronize(h->stream));
    profile_collect(h);
    if (int se = device_status_error(h, hw[windows].info)) return se;
    for (uint32_t w = 0; w < windows && w < n_windows_out; w++) fill_eager_result(h, hw[w], &out[w]);
    for (uint32_t w = windows; w < n_windows_out; w++) {
        std::memset(&out[w], 0, sizeof(out[w]));
        out[w].status = SJBG_E_INVALID;   // no such window
    }
    return SJBG_OK;
}

}  // extern "C"
