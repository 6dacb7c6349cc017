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

// Which of 4 quads of right keys (16 keys at shared-memory address `rk`,
// 16-byte aligned) hold a key equal to one of the thread's 8 left keys: bit q
// of the result for quad q.  The 128 compares are PTX setp.eq with an OR into
// the predicate, one instruction per compare, in eight independent chains (two
// per quad: left keys 0-3 and 4-7), so the integer pipe sees about one
// instruction per compare; seven more form the mask.
static_assert(kLReg == 8, "quads_equal_8x16 compares 8 left keys");
__device__ __forceinline__ uint32_t quads_equal_8x16(const uint32_t (&l)[kLReg], uint32_t rk) {
    uint32_t m;
    asm volatile("{\n\t"
        ".reg .b32 a<16>, t;\n\t"
        ".reg .pred p<8>;\n\t"
        "ld.shared.v4.u32 {a0, a1, a2, a3}, [%9+0];\n\t"
        "ld.shared.v4.u32 {a4, a5, a6, a7}, [%9+16];\n\t"
        "ld.shared.v4.u32 {a8, a9, a10, a11}, [%9+32];\n\t"
        "ld.shared.v4.u32 {a12, a13, a14, a15}, [%9+48];\n\t"
        "setp.eq.u32 p0, %1, a0;\n\t"
        "setp.eq.u32 p1, %5, a0;\n\t"
        "setp.eq.u32 p2, %1, a4;\n\t"
        "setp.eq.u32 p3, %5, a4;\n\t"
        "setp.eq.u32 p4, %1, a8;\n\t"
        "setp.eq.u32 p5, %5, a8;\n\t"
        "setp.eq.u32 p6, %1, a12;\n\t"
        "setp.eq.u32 p7, %5, a12;\n\t"
        "setp.eq.or.u32 p0, %2, a0, p0;\n\t"
        "setp.eq.or.u32 p1, %6, a0, p1;\n\t"
        "setp.eq.or.u32 p2, %2, a4, p2;\n\t"
        "setp.eq.or.u32 p3, %6, a4, p3;\n\t"
        "setp.eq.or.u32 p4, %2, a8, p4;\n\t"
        "setp.eq.or.u32 p5, %6, a8, p5;\n\t"
        "setp.eq.or.u32 p6, %2, a12, p6;\n\t"
        "setp.eq.or.u32 p7, %6, a12, p7;\n\t"
        "setp.eq.or.u32 p0, %3, a0, p0;\n\t"
        "setp.eq.or.u32 p1, %7, a0, p1;\n\t"
        "setp.eq.or.u32 p2, %3, a4, p2;\n\t"
        "setp.eq.or.u32 p3, %7, a4, p3;\n\t"
        "setp.eq.or.u32 p4, %3, a8, p4;\n\t"
        "setp.eq.or.u32 p5, %7, a8, p5;\n\t"
        "setp.eq.or.u32 p6, %3, a12, p6;\n\t"
        "setp.eq.or.u32 p7, %7, a12, p7;\n\t"
        "setp.eq.or.u32 p0, %4, a0, p0;\n\t"
        "setp.eq.or.u32 p1, %8, a0, p1;\n\t"
        "setp.eq.or.u32 p2, %4, a4, p2;\n\t"
        "setp.eq.or.u32 p3, %8, a4, p3;\n\t"
        "setp.eq.or.u32 p4, %4, a8, p4;\n\t"
        "setp.eq.or.u32 p5, %8, a8, p5;\n\t"
        "setp.eq.or.u32 p6, %4, a12, p6;\n\t"
        "setp.eq.or.u32 p7, %8, a12, p7;\n\t"
        "setp.eq.or.u32 p0, %1, a1, p0;\n\t"
        "setp.eq.or.u32 p1, %5, a1, p1;\n\t"
        "setp.eq.or.u32 p2, %1, a5, p2;\n\t"
        "setp.eq.or.u32 p3, %5, a5, p3;\n\t"
        "setp.eq.or.u32 p4, %1, a9, p4;\n\t"
        "setp.eq.or.u32 p5, %5, a9, p5;\n\t"
        "setp.eq.or.u32 p6, %1, a13, p6;\n\t"
        "setp.eq.or.u32 p7, %5, a13, p7;\n\t"
        "setp.eq.or.u32 p0, %2, a1, p0;\n\t"
        "setp.eq.or.u32 p1, %6, a1, p1;\n\t"
        "setp.eq.or.u32 p2, %2, a5, p2;\n\t"
        "setp.eq.or.u32 p3, %6, a5, p3;\n\t"
        "setp.eq.or.u32 p4, %2, a9, p4;\n\t"
        "setp.eq.or.u32 p5, %6, a9, p5;\n\t"
        "setp.eq.or.u32 p6, %2, a13, p6;\n\t"
        "setp.eq.or.u32 p7, %6, a13, p7;\n\t"
        "setp.eq.or.u32 p0, %3, a1, p0;\n\t"
        "setp.eq.or.u32 p1, %7, a1, p1;\n\t"
        "setp.eq.or.u32 p2, %3, a5, p2;\n\t"
        "setp.eq.or.u32 p3, %7, a5, p3;\n\t"
        "setp.eq.or.u32 p4, %3, a9, p4;\n\t"
        "setp.eq.or.u32 p5, %7, a9, p5;\n\t"
        "setp.eq.or.u32 p6, %3, a13, p6;\n\t"
        "setp.eq.or.u32 p7, %7, a13, p7;\n\t"
        "setp.eq.or.u32 p0, %4, a1, p0;\n\t"
        "setp.eq.or.u32 p1, %8, a1, p1;\n\t"
        "setp.eq.or.u32 p2, %4, a5, p2;\n\t"
        "setp.eq.or.u32 p3, %8, a5, p3;\n\t"
        "setp.eq.or.u32 p4, %4, a9, p4;\n\t"
        "setp.eq.or.u32 p5, %8, a9, p5;\n\t"
        "setp.eq.or.u32 p6, %4, a13, p6;\n\t"
        "setp.eq.or.u32 p7, %8, a13, p7;\n\t"
        "setp.eq.or.u32 p0, %1, a2, p0;\n\t"
        "setp.eq.or.u32 p1, %5, a2, p1;\n\t"
        "setp.eq.or.u32 p2, %1, a6, p2;\n\t"
        "setp.eq.or.u32 p3, %5, a6, p3;\n\t"
        "setp.eq.or.u32 p4, %1, a10, p4;\n\t"
        "setp.eq.or.u32 p5, %5, a10, p5;\n\t"
        "setp.eq.or.u32 p6, %1, a14, p6;\n\t"
        "setp.eq.or.u32 p7, %5, a14, p7;\n\t"
        "setp.eq.or.u32 p0, %2, a2, p0;\n\t"
        "setp.eq.or.u32 p1, %6, a2, p1;\n\t"
        "setp.eq.or.u32 p2, %2, a6, p2;\n\t"
        "setp.eq.or.u32 p3, %6, a6, p3;\n\t"
        "setp.eq.or.u32 p4, %2, a10, p4;\n\t"
        "setp.eq.or.u32 p5, %6, a10, p5;\n\t"
        "setp.eq.or.u32 p6, %2, a14, p6;\n\t"
        "setp.eq.or.u32 p7, %6, a14, p7;\n\t"
        "setp.eq.or.u32 p0, %3, a2, p0;\n\t"
        "setp.eq.or.u32 p1, %7, a2, p1;\n\t"
        "setp.eq.or.u32 p2, %3, a6, p2;\n\t"
        "setp.eq.or.u32 p3, %7, a6, p3;\n\t"
        "setp.eq.or.u32 p4, %3, a10, p4;\n\t"
        "setp.eq.or.u32 p5, %7, a10, p5;\n\t"
        "setp.eq.or.u32 p6, %3, a14, p6;\n\t"
        "setp.eq.or.u32 p7, %7, a14, p7;\n\t"
        "setp.eq.or.u32 p0, %4, a2, p0;\n\t"
        "setp.eq.or.u32 p1, %8, a2, p1;\n\t"
        "setp.eq.or.u32 p2, %4, a6, p2;\n\t"
        "setp.eq.or.u32 p3, %8, a6, p3;\n\t"
        "setp.eq.or.u32 p4, %4, a10, p4;\n\t"
        "setp.eq.or.u32 p5, %8, a10, p5;\n\t"
        "setp.eq.or.u32 p6, %4, a14, p6;\n\t"
        "setp.eq.or.u32 p7, %8, a14, p7;\n\t"
        "setp.eq.or.u32 p0, %1, a3, p0;\n\t"
        "setp.eq.or.u32 p1, %5, a3, p1;\n\t"
        "setp.eq.or.u32 p2, %1, a7, p2;\n\t"
        "setp.eq.or.u32 p3, %5, a7, p3;\n\t"
        "setp.eq.or.u32 p4, %1, a11, p4;\n\t"
        "setp.eq.or.u32 p5, %5, a11, p5;\n\t"
        "setp.eq.or.u32 p6, %1, a15, p6;\n\t"
        "setp.eq.or.u32 p7, %5, a15, p7;\n\t"
        "setp.eq.or.u32 p0, %2, a3, p0;\n\t"
        "setp.eq.or.u32 p1, %6, a3, p1;\n\t"
        "setp.eq.or.u32 p2, %2, a7, p2;\n\t"
        "setp.eq.or.u32 p3, %6, a7, p3;\n\t"
        "setp.eq.or.u32 p4, %2, a11, p4;\n\t"
        "setp.eq.or.u32 p5, %6, a11, p5;\n\t"
        "setp.eq.or.u32 p6, %2, a15, p6;\n\t"
        "setp.eq.or.u32 p7, %6, a15, p7;\n\t"
        "setp.eq.or.u32 p0, %3, a3, p0;\n\t"
        "setp.eq.or.u32 p1, %7, a3, p1;\n\t"
        "setp.eq.or.u32 p2, %3, a7, p2;\n\t"
        "setp.eq.or.u32 p3, %7, a7, p3;\n\t"
        "setp.eq.or.u32 p4, %3, a11, p4;\n\t"
        "setp.eq.or.u32 p5, %7, a11, p5;\n\t"
        "setp.eq.or.u32 p6, %3, a15, p6;\n\t"
        "setp.eq.or.u32 p7, %7, a15, p7;\n\t"
        "setp.eq.or.u32 p0, %4, a3, p0;\n\t"
        "setp.eq.or.u32 p1, %8, a3, p1;\n\t"
        "setp.eq.or.u32 p2, %4, a7, p2;\n\t"
        "setp.eq.or.u32 p3, %8, a7, p3;\n\t"
        "setp.eq.or.u32 p4, %4, a11, p4;\n\t"
        "setp.eq.or.u32 p5, %8, a11, p5;\n\t"
        "setp.eq.or.u32 p6, %4, a15, p6;\n\t"
        "setp.eq.or.u32 p7, %8, a15, p7;\n\t"
        "or.pred p0, p0, p1;\n\t"
        "or.pred p2, p2, p3;\n\t"
        "or.pred p4, p4, p5;\n\t"
        "or.pred p6, p6, p7;\n\t"
        "selp.u32 %0, 1, 0, p0;\n\t"
        "selp.u32 t, 2, 0, p2;\n\t"
        "or.b32 %0, %0, t;\n\t"
        "selp.u32 t, 4, 0, p4;\n\t"
        "or.b32 %0, %0, t;\n\t"
        "selp.u32 t, 8, 0, p6;\n\t"
        "or.b32 %0, %0, t;\n\t"
        "}"
        : "=r"(m)
        : "r"(l[0]), "r"(l[1]), "r"(l[2]), "r"(l[3]), "r"(l[4]), "r"(l[5]), "r"(l[6]), "r"(l[7]), "r"(rk)
        : "memory");
    return m;
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
        const uint32_t rbase = (uint32_t)__cvta_generic_to_shared(rkeys);
        for (uint32_t r = 0; r < mpad; r += kVote) {
            // bit q: right keys r + 4q .. r + 4q + 3 hold a key equal to one of this lane's
            uint32_t hits = 0;
#pragma unroll
            for (uint32_t b = 0; b < kVote / 16; b++) hits |= quads_equal_8x16(lk, rbase + 4u * (r + 16u * b)) << (4u * b);
            if (!__any_sync(0xFFFFFFFFu, hits != 0u)) continue;
            // exact path (warp-uniform) over the quads that some lane matched
            const uint32_t quads = __reduce_or_sync(0xFFFFFFFFu, hits);
            uint32_t mine = 0;
            for (uint32_t qs = quads; qs; qs &= qs - 1) {
                const uint32_t q0 = r + 4u * (uint32_t)(__ffs(qs) - 1), qe = min(q0 + 4u, m);
                for (uint32_t q = q0; q < qe; q++) {
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
            }
            count += mine;
            if (kPairs) {
                uint32_t tot;
                const uint32_t ex = warp_excl_scan(mine, &tot);
                unsigned long long base = 0;
                if (lane_id() == 0 && tot) base = atomicAdd(&acc->npairs, (unsigned long long)tot);
                base = __shfl_sync(0xFFFFFFFFu, base, 0) + ex;
                for (uint32_t qs = quads; qs && mine; qs &= qs - 1) {
                    const uint32_t q0 = r + 4u * (uint32_t)(__ffs(qs) - 1), qe = min(q0 + 4u, m);
                    for (uint32_t q = q0; q < qe; q++) {
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
    }
    flush_acc(acc, count, xr, prod);
    if (extra_count) {
        const unsigned long long c = warp_sum_u64(count);
        if (lane_id() == 0 && c) atomicAdd(extra_count, c);
    }
}

}  // namespace sjbg
