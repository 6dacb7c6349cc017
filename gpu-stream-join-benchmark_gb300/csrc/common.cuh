// common.cuh - device-side helpers shared by the join kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/sjbg.h"
#include "sjbg_gen.h"

// Block barrier that first reconverges the calling warp: loops whose trip
// count differs between the lanes of a warp (retry loops on shared atomics
// in particular) must not reach __syncthreads() with the warp diverged.
#define SJBG_BARRIER()   \
    do {                 \
        __syncwarp();    \
        __syncthreads(); \
    } while (0)

namespace sjbg {

constexpr uint32_t kEmptyKey = 0xFFFFFFFFu;   // empty slot marker of shared-memory tables
constexpr int kWarp = 32;

// Device-side error bits, OR-ed into the handle's status word.
enum : uint32_t {
    kErrTableFull = 1u << 0,   // a table could not take a key (should be impossible by sizing)
    kErrTimeout = 1u << 1,     // a bounded wait gave up
    kErrBadWindow = 1u << 2,   // a window descriptor is inconsistent
    kErrQueue = 1u << 3,       // work queue overflow
};

// Per-window accumulators kept in device memory.
struct WinAcc {
    unsigned long long count;
    unsigned long long xr;
    unsigned long long prod;
    unsigned long long npairs;   // pairs produced (may exceed capacity)
    unsigned long long info;     // kInfo* bits | heavy keys << 32 (learned partitioning)
};

enum : unsigned long long { kInfoLearned = 1ull, kInfoFallback = 2ull, kInfoRadixByCost = 4ull };

// Per-window plan entry of a lazy batch, in device memory.
struct WinPlan {
    uint64_t left_off, n_left, right_off, n_right;
    uint64_t pairs_off, pairs_cap;
    uint32_t bucket_base;   // first global bucket id of this window
    uint32_t log2_buckets;  // buckets of this window = 1 << log2_buckets
    uint32_t model;         // learned partitioner model slot, or 0xFFFFFFFF for radix
    uint32_t two_level;     // hash join: partitioned in two passes (coarse runs, then fine buckets)
};

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ uint32_t warp_id() { return threadIdx.x >> 5; }

// Multiplicative slot hash of a key inside a table of 2^bits slots.
__device__ __forceinline__ uint32_t slot_hash(uint32_t key, uint32_t bits) {
    return (uint32_t)(((uint64_t)key * 0x9E3779B97F4A7C15ull) >> (64 - bits));
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
}
__device__ __forceinline__ unsigned long long warp_xor_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v ^= __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
}

// Add (count, xor, prod) of the calling block into a window accumulator:
// warp reduction, then one atomic per warp.
__device__ __forceinline__ void flush_acc(WinAcc *acc, unsigned long long count, unsigned long long xr,
                                          unsigned long long prod) {
    count = warp_sum_u64(count);
    xr = warp_xor_u64(xr);
    prod = warp_sum_u64(prod);
    if (lane_id() == 0) {
        if (count) atomicAdd(&acc->count, count);
        if (xr) atomicXor(&acc->xr, xr);
        if (prod) atomicAdd(&acc->prod, prod);
    }
}

// hi + the carry out of a + b (two instructions: add with carry-out, add with carry-in).
__device__ __forceinline__ uint32_t add_carry(uint32_t hi, uint32_t a, uint32_t b) {
    uint32_t r;
    asm("{\n\t.reg .u32 t;\n\tadd.cc.u32 t, %1, %2;\n\taddc.u32 %0, %3, 0;\n\t}" : "=r"(r) : "r"(a), "r"(b), "r"(hi));
    return r;
}

// Exclusive warp prefix sum of a 32-bit value.
__device__ __forceinline__ uint32_t warp_excl_scan(uint32_t v, uint32_t *total) {
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane_id() >= (uint32_t)o) x += y;
    }
    *total = __shfl_sync(0xFFFFFFFFu, x, 31);
    return x - v;
}

// Prefetch the 16-byte aligned part of [p, p + bytes) into L2 with one bulk
// request (at most 256 KiB; nothing outside the range is touched, no completion
// to wait for).
__device__ __forceinline__ void l2_prefetch_bulk(const void *p, size_t bytes) {
    const uintptr_t a = ((uintptr_t)p + 15) & ~(uintptr_t)15;
    uintptr_t e = ((uintptr_t)p + bytes) & ~(uintptr_t)15;
    if (e > a + (256u << 10)) e = a + (256u << 10);
    if (e > a)
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a), "r"((uint32_t)(e - a)) : "memory");
}

// Global nanosecond timer for bounded waits.
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

}  // namespace sjbg
