/*
 * sjbg_gen.h - deterministic, counter-based synthetic stream generator and the
 * pair hashes used by the join checksums.  Plain C99, usable from host C/C++
 * and (when compiled by nvcc) from device code, so that a tuple generated on
 * the GPU is bit-identical to the same tuple generated on the host.
 *
 * Stream tuples follow the reference's 16-byte Tuple {u32 key, u32 val,
 * u64 ts} (include/sjb/utils/Tuple.hpp:6-11).  Unlike the reference's
 * DataGenerator (src/sjb/utils/DataGenerator.cpp:63-70, which sets val = key
 * and draws keys with cuRAND), tuple i of a stream has val = (u32)i and
 * ts = i, so that a join result can name the (left index, right index) pair.
 *
 * Randomness: SplitMix64 (Steele, Lea, Flood, "Fast splittable pseudorandom
 * number generators", OOPSLA 2014) used as a counter-based generator:
 * draw i of stream `seed` is mix64(splitmix_state(seed) + (i+1) * gamma).
 *
 * Zipf keys: inverse-CDF lookup of a 64-bit uniform draw in a table of
 * 64-bit fixed-point cumulative probabilities (built on the host, see
 * sjbg_zipf_table_fill), so host and device sample identically with integer
 * arithmetic only.  Ranks are mapped to keys by a seeded bijection on the key
 * domain (a 4-round balanced Feistel network with cycle walking).
 */
#ifndef SJBG_GEN_H
#define SJBG_GEN_H

#include <stdint.h>
#include <math.h>

#if defined(__CUDACC__)
#define SJBG_HD __host__ __device__ __forceinline__
#else
#define SJBG_HD static inline
#endif

#define SJBG_GOLDEN_GAMMA 0x9E3779B97F4A7C15ull

/* SplitMix64 output function (the published finaliser). */
SJBG_HD uint64_t sjbg_mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* One SplitMix64 step from state x: advance by gamma, then mix. */
SJBG_HD uint64_t sjbg_splitmix64(uint64_t x) { return sjbg_mix64(x + SJBG_GOLDEN_GAMMA); }

/* Draw i of the stream identified by seed. */
SJBG_HD uint64_t sjbg_rand64(uint64_t seed, uint64_t i) {
    return sjbg_mix64(sjbg_splitmix64(seed) + (i + 1) * SJBG_GOLDEN_GAMMA);
}

/* High 64 bits of a 64x64 product (unbiased-enough range reduction). */
SJBG_HD uint64_t sjbg_mulhi64(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * (unsigned __int128)b) >> 64);
#endif
}

/* Uniform key in [0, domain) for draw i of stream seed. */
SJBG_HD uint32_t sjbg_uniform_key(uint64_t seed, uint64_t i, uint64_t domain) {
    return (uint32_t)sjbg_mulhi64(sjbg_rand64(seed, i), domain);
}

/* ---- pair hashes of the join checksums ------------------------------------
 * xor checksum  = XOR over matching pairs of sjbg_pair_hash(r, s)
 * prod checksum = sum over matching pairs of sjbg_fr(r) * sjbg_gs(s) mod 2^64
 *               = sum over keys k of (sum_{r in R_k} fr(r)) * (sum_{s in S_k} gs(s)),
 *   which is still a function of the exact pair multiset but costs O(|R|+|S|).
 * r and s are the val fields of the left (R) and right (S) tuples.
 *
 * fr and gs are computed once per tuple in the hash join's hot loops, so they
 * use a two-multiply mixer of 32-bit words instead of the 64-bit SplitMix64
 * finaliser: h1 = (x ^ k) * A (32x32 -> 64 bits; its low half is a bijection
 * of x), h2 = (lo(h1) ^ hi(h1) ^ c) * B, result = h1 ^ (h2 << 32) ^ (h2 >> 13),
 * forced odd.  A = 0x9E3779B1 and B = 0x85EBCA77 are the odd 32-bit
 * multipliers of Knuth's multiplicative hashing and of MurmurHash3's
 * finaliser; the side keys k (0x243F6A88 left, 0xB7E15162 right) are the
 * leading hex digits of pi and e.  The xor checksum keeps SplitMix64. */
SJBG_HD uint64_t sjbg_pair_hash(uint32_t r, uint32_t s) {
    return sjbg_splitmix64(((uint64_t)r << 32) | (uint64_t)s);
}
#define SJBG_FR_KEY 0x243F6A88u
#define SJBG_GS_KEY 0xB7E15162u
SJBG_HD uint64_t sjbg_mix32(uint32_t x, uint32_t k) {
    const uint64_t h1 = (uint64_t)(x ^ k) * 0x9E3779B1u;
    const uint64_t h2 = (uint64_t)((uint32_t)h1 ^ (uint32_t)(h1 >> 32) ^ 0x7F4A7C15u) * 0x85EBCA77u;
    return h1 ^ (h2 << 32) ^ (h2 >> 13);
}
SJBG_HD uint64_t sjbg_fr(uint32_t r) { return sjbg_mix32(r, SJBG_FR_KEY) | 1ull; }
SJBG_HD uint64_t sjbg_gs(uint32_t s) { return sjbg_mix32(s, SJBG_GS_KEY) | 1ull; }
/* fr (side 0) or gs (side 1), the side chosen by the key alone. */
SJBG_HD uint64_t sjbg_fside(uint32_t v, uint32_t side) {
    return sjbg_mix32(v, side ? SJBG_GS_KEY : SJBG_FR_KEY) | 1ull;
}

/* ---- seeded bijection on [0, domain) --------------------------------------
 * Balanced Feistel network on 2h bits (2h >= log2(domain), h >= 1), 4 rounds,
 * round function = mix64 of (half ^ round key) truncated to h bits; values
 * outside [0, domain) are walked through the permutation again (cycle walking),
 * which keeps the map a bijection on [0, domain). */
SJBG_HD uint32_t sjbg_perm_half_bits(uint64_t domain) {
    uint32_t bits = 0;
    while (bits < 64 && ((uint64_t)1 << bits) < domain) bits++;
    if (bits < 2) bits = 2;
    return (bits + 1) / 2;
}

SJBG_HD uint64_t sjbg_feistel(uint64_t x, uint32_t h, uint64_t seed) {
    const uint64_t mask = ((uint64_t)1 << h) - 1;
    uint64_t left = (x >> h) & mask, right = x & mask;
    for (uint32_t round = 0; round < 4; round++) {
        uint64_t f = sjbg_mix64(right ^ sjbg_splitmix64(seed + round)) & mask;
        uint64_t nl = right;
        right = left ^ f;
        left = nl;
    }
    return (left << h) | right;
}

SJBG_HD uint32_t sjbg_perm(uint64_t rank, uint64_t domain, uint64_t seed) {
    if (domain <= 1) return 0;
    uint32_t h = sjbg_perm_half_bits(domain);
    uint64_t x = rank;
    do { x = sjbg_feistel(x, h, seed); } while (x >= domain);
    return (uint32_t)x;
}

/* ---- Zipf ranks -------------------------------------------------------------
 * table[k] = floor(2^64 * P(rank <= k)) for rank k in [0, n), with P(rank = k)
 * proportional to (k+1)^-z; the last entry is saturated to 2^64-1.
 * A draw u maps to the smallest k with u < table[k]. */
SJBG_HD uint32_t sjbg_zipf_rank(const uint64_t *table, uint64_t n, uint64_t u) {
    uint64_t lo = 0, hi = n - 1;           /* answer in [lo, hi] */
    while (lo < hi) {
        uint64_t mid = lo + ((hi - lo) >> 1);
        if (u < table[mid]) hi = mid; else lo = mid + 1;
    }
    return (uint32_t)lo;
}

/* (the two functions below are plain static inline, i.e. host-only under nvcc) */
/* Host-only: fill the Zipf CDF table (n entries, exponent z >= 0).  Weights
 * are summed in IEEE double with Kahan compensation (no products inside the
 * sums, so FMA contraction cannot change the result between compilers). */
static inline void sjbg_zipf_table_fill(uint64_t *table, uint64_t n, double z) {
    double *w = (double *)table;               /* weights stored in place first */
    double total = 0.0, comp = 0.0;
    for (uint64_t k = 0; k < n; k++) {
        double x = pow((double)(k + 1), -z);
        w[k] = x;
        double y = x - comp, t = total + y;
        comp = (t - total) - y;
        total = t;
    }
    const double scale = 18446744073709551616.0; /* 2^64 */
    double run = 0.0;
    comp = 0.0;
    for (uint64_t k = 0; k < n; k++) {
        double x = w[k];
        double y = x - comp, t = run + y;
        comp = (t - run) - y;
        run = t;
        double v = (run / total) * scale;
        table[k] = (k + 1 == n || v >= scale) ? UINT64_MAX : (uint64_t)v;
    }
}

/* Host-only: log-uniform window length in [lo, hi] for window w. */
static inline uint64_t sjbg_log_uniform(uint64_t seed, uint64_t w, uint64_t lo, uint64_t hi) {
    double u = (double)(sjbg_rand64(seed, w) >> 11) * (1.0 / 9007199254740992.0);
    double v = exp2(log2((double)lo) + u * (log2((double)hi) - log2((double)lo)));
    uint64_t r = (uint64_t)v;
    if (r < lo) r = lo;
    if (r > hi) r = hi;
    return r;
}
#endif /* SJBG_GEN_H */
