// nlj.cuh - the nested-loop join's block routine, shared by the lazy and
// eager kernels (nlj.cu) and the persistent eager kernel (eager_pk.cu).
#pragma once

#include "eager.cuh"

namespace sjbg {

constexpr int kNljThreads = 256;
constexpr int kLReg = 8;                         // left keys per thread
constexpr uint32_t kLTile = kNljThreads * kLReg;  // left tuples per CTA
constexpr uint32_t kChunk = 2048;                // right tuples per shared-memory chunk
constexpr uint32_t kRSplit = 16384;              // right tuples per CTA
constexpr uint32_t kVote = 64;                   // right keys between warp votes

// Whether any of the thread's 8 left keys equals any of 4 right keys: the 32
// compares as PTX setp.eq with an OR into the predicate (one instruction per
// compare), in four independent chains (one per right key) merged at the end.
static_assert(kLReg == 8, "any_equal_8x4 compares 8 left keys");
__device__ __forceinline__ uint32_t any_equal_8x4(const uint32_t (&l)[kLReg], const uint4 k) {
    uint32_t hit;
    asm("{\n\t"
        ".reg .pred p0, p1, p2, p3;\n\t"
        "setp.eq.u32 p0, %1, %9;\n\t"
        "setp.eq.u32 p1, %1, %10;\n\t"
        "setp.eq.u32 p2, %1, %11;\n\t"
        "setp.eq.u32 p3, %1, %12;\n\t"
        "setp.eq.or.u32 p0, %2, %9, p0;\n\t"
        "setp.eq.or.u32 p1, %2, %10, p1;\n\t"
        "setp.eq.or.u32 p2, %2, %11, p2;\n\t"
        "setp.eq.or.u32 p3, %2, %12, p3;\n\t"
        "setp.eq.or.u32 p0, %3, %9, p0;\n\t"
        "setp.eq.or.u32 p1, %3, %10, p1;\n\t"
        "setp.eq.or.u32 p2, %3, %11, p2;\n\t"
        "setp.eq.or.u32 p3, %3, %12, p3;\n\t"
        "setp.eq.or.u32 p0, %4, %9, p0;\n\t"
        "setp.eq.or.u32 p1, %4, %10, p1;\n\t"
        "setp.eq.or.u32 p2, %4, %11, p2;\n\t"
        "setp.eq.or.u32 p3, %4, %12, p3;\n\t"
        "setp.eq.or.u32 p0, %5, %9, p0;\n\t"
        "setp.eq.or.u32 p1, %5, %10, p1;\n\t"
        "setp.eq.or.u32 p2, %5, %11, p2;\n\t"
        "setp.eq.or.u32 p3, %5, %12, p3;\n\t"
        "setp.eq.or.u32 p0, %6, %9, p0;\n\t"
        "setp.eq.or.u32 p1, %6, %10, p1;\n\t"
        "setp.eq.or.u32 p2, %6, %11, p2;\n\t"
        "setp.eq.or.u32 p3, %6, %12, p3;\n\t"
        "setp.eq.or.u32 p0, %7, %9, p0;\n\t"
        "setp.eq.or.u32 p1, %7, %10, p1;\n\t"
        "setp.eq.or.u32 p2, %7, %11, p2;\n\t"
        "setp.eq.or.u32 p3, %7, %12, p3;\n\t"
        "setp.eq.or.u32 p0, %8, %9, p0;\n\t"
        "setp.eq.or.u32 p1, %8, %10, p1;\n\t"
        "setp.eq.or.u32 p2, %8, %11, p2;\n\t"
        "setp.eq.or.u32 p3, %8, %12, p3;\n\t"
        "or.pred p0, p0, p1;\n\t"
        "or.pred p2, p2, p3;\n\t"
        "or.pred p0, p0, p2;\n\t"
        "selp.u32 %0, 1, 0, p0;\n\t"
        "}"
        : "=r"(hit)
        : "r"(l[0]), "r"(l[1]), "r"(l[2]), "r"(l[3]), "r"(l[4]), "r"(l[5]), "r"(l[6]), "r"(l[7]), "r"(k.x),
          "r"(k.y), "r"(k.z), "r"(k.w));
    return hit;
}

// Load of a (key, val) pair.  Kernels whose inputs do not change while they
// run read through the read-only path; the persistent eager kernel, whose
// tuple stores grow while it runs, uses plain (coherent) loads.
template <bool kCoherent>
__device__ __forceinline__ uint2 nlj_load(const sjbg_tuple *p) {
    if (kCoherent) return *reinterpret_cast<const uint2 *>(p);
    return __ldg(reinterpret_cast<const uint2 *>(p));
}

// One CTA's share of a window: left tuples [l0, l0 + kLTile) against right
// tuples [r0, r0 + kRSplit).  Adds count/xor/prod to *acc (and the count to
// *extra_count when given); pairs go to pout[0, pcap) via *npairs.
template <bool kEnum, bool kPairs, bool kCoherent = false>
__device__ __forceinline__ void nlj_block(const sjbg_tuple *__restrict__ Lw, uint32_t nL,
                                          const sjbg_tuple *__restrict__ Rw, uint32_t nR, uint32_t l0, uint32_t r0,
                                          WinAcc *acc, unsigned long long *extra_count, sjbg_pair *pout,
                                          uint64_t pcap, uint32_t rsplit = kRSplit) {
    __shared__ __align__(16) uint32_t rkeys[kChunk];
    __shared__ __align__(16) uint32_t rvals[kChunk];
    uint32_t lk[kLReg], lv[kLReg];
    uint32_t lvalid = 0;
    uint32_t fill = 0;
#pragma unroll
    for (int a = 0; a < kLReg; a++) {
        const uint32_t li = l0 + a * kNljThreads + threadIdx.x;
        if (li < nL) {
            const uint2 t = nlj_load<kCoherent>(Lw + li);
            lk[a] = t.x;
            lv[a] = t.y;
            lvalid |= 1u << a;
            fill = t.x;
        }
    }
#pragma unroll
    for (int a = 0; a < kLReg; a++)
        if (!((lvalid >> a) & 1u)) { lk[a] = fill; lv[a] = 0; }   // invalid slots only cause false alarms

    unsigned long long count = 0, xr = 0, prod = 0;
    const uint32_t r_end = min(nR, r0 + rsplit);
    for (uint32_t c0 = r0; c0 < r_end; c0 += kChunk) {
        const uint32_t m = min(kChunk, r_end - c0);
        const uint32_t mpad = (m + kVote - 1) / kVote * kVote;
        SJBG_BARRIER();
        for (uint32_t i = threadIdx.x; i < mpad; i += kNljThreads) {
            if (i < m) {
                const uint2 t = nlj_load<kCoherent>(Rw + c0 + i);
                rkeys[i] = t.x;
                rvals[i] = t.y;
            } else {
                rkeys[i] = lk[0];   // padding: bounds are re-checked in the exact path
                rvals[i] = 0;
            }
        }
        SJBG_BARRIER();
        const uint4 *rk4 = reinterpret_cast<const uint4 *>(rkeys);
        for (uint32_t r = 0; r < mpad; r += kVote) {
            bool p = false;
#pragma unroll 4
            for (uint32_t q = 0; q < kVote / 4; q++) {
                const uint4 k4 = rk4[(r >> 2) + q];
                p |= any_equal_8x4(lk, k4) != 0u;
            }
            if (!__any_sync(0xFFFFFFFFu, p)) continue;
            // exact path for this group of kVote right keys (warp-uniform)
            const uint32_t qe = min(r + kVote, m);
            uint32_t mine = 0;
            for (uint32_t q = r; q < qe; q++) {
                const uint32_t k = rkeys[q];
#pragma unroll
                for (int a = 0; a < kLReg; a++) {
                    if (((lvalid >> a) & 1u) && lk[a] == k) {
                        const uint32_t sv = rvals[q];
                        mine++;
                        prod += sjbg_fr(lv[a]) * sjbg_gs(sv);
                        if (kEnum) xr ^= sjbg_pair_hash(lv[a], sv);
                    }
                }
            }
            count += mine;
            if (kPairs) {
                uint32_t tot;
                const uint32_t ex = warp_excl_scan(mine, &tot);
                unsigned long long base = 0;
                if (lane_id() == 0 && tot) base = atomicAdd(&acc->npairs, (unsigned long long)tot);
                base = __shfl_sync(0xFFFFFFFFu, base, 0) + ex;
                for (uint32_t q = r; q < qe && mine; q++) {
                    const uint32_t k = rkeys[q];
#pragma unroll
                    for (int a = 0; a < kLReg; a++) {
                        if (((lvalid >> a) & 1u) && lk[a] == k) {
                            if (base < pcap) pout[base] = sjbg_pair{lv[a], rvals[q]};
                            base++;
                        }
                    }
                }
            }
        }
    }
    flush_acc(acc, count, xr, prod);
    if (extra_count) {
        const unsigned long long c = warp_sum_u64(count);
        if (lane_id() == 0 && c) atomicAdd(extra_count, c);
    }
}

}  // namespace sjbg
