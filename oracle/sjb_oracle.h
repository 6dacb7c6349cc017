/*
 * sjb_oracle.h - CPU oracle for the windowed stream-join path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: tests/, the
 * smoke() entry point and the CPU-baseline leg of bench.py may load it; the
 * product library (libsjbg.so) never links, loads or calls it.
 *
 * Contents
 *  - restatements of the reference's CPU joiners, returning what they return
 *    (the match count) and following their algorithm step by step so their
 *    timing is a fair CPU baseline:
 *        lazy CPU_HJ   src/sjb/windowing/lazy/executor/CPU/CPU_HJ.cpp:30-136
 *        lazy CPU_SMJ  src/sjb/windowing/lazy/executor/CPU/CPU_SMJ.cpp:23-139
 *        lazy CPU_NLJ  src/sjb/windowing/lazy/executor/CPU/CPU_NLJ.cpp:11-32
 *        eager CPU_HJ  src/sjb/windowing/eager/executor/CPU/CPU_HJ.cpp:27-82
 *          fed as Eager::CountBased does (include/sjb/windowing/eager/CountBased.cuh:36-72)
 *  - the result restatement (oracle_join): per window the match count, the
 *    xor and prod pair checksums and the sorted (left.val, right.val) pair
 *    list, by grouping both sides on key (the grouping of CPU_SMJ.cpp:103-125
 *    with the pair predicate of CPU_NLJ.cpp:18-27).
 *  - host generation of the synthetic streams (same generator header as the
 *    product, csrc/sjbg_gen.h).
 */
#ifndef SJB_ORACLE_H
#define SJB_ORACLE_H

#include <stdint.h>
#include "../include/sjbg.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_result {
    uint64_t count;
    uint64_t xor_checksum;
    uint64_t prod_checksum;
    uint64_t n_pairs;   /* pairs written (<= capacity) */
} oracle_result;

/* ---- generators ---- */
void oracle_gen_uniform(sjbg_tuple *out, uint64_t first, uint64_t n, uint64_t seed, uint64_t domain, int threads);
void oracle_zipf_table(uint64_t *table, uint64_t n, double z);
void oracle_gen_zipf(sjbg_tuple *out, uint64_t first, uint64_t n, uint64_t seed,
                     const uint64_t *table, uint64_t domain, uint64_t perm_seed, int threads);
uint32_t oracle_perm(uint64_t rank, uint64_t domain, uint64_t seed);
uint64_t oracle_log_uniform(uint64_t seed, uint64_t w, uint64_t lo, uint64_t hi);
uint64_t oracle_pair_hash(uint32_t r, uint32_t s);
uint64_t oracle_fr(uint32_t r);
uint64_t oracle_gs(uint32_t s);

/* ---- reference CPU joiners, restated (return 0 on success, -1 when a key
 *      is outside [0, distinct_keys), where the reference would index out of
 *      bounds) ---- */
int oracle_lazy_hj_count(const sjbg_tuple *left, uint64_t n_left, const sjbg_tuple *right, uint64_t n_right,
                         uint64_t distinct_keys, uint64_t batch_size, int probe_threads, uint64_t *count);
int oracle_lazy_smj_count(const sjbg_tuple *left, uint64_t n_left, const sjbg_tuple *right, uint64_t n_right,
                          uint64_t distinct_keys, int sort_threads, uint64_t *count);
uint64_t oracle_lazy_nlj_count(const sjbg_tuple *left, uint64_t n_left, const sjbg_tuple *right, uint64_t n_right);
/* Eager: n_batches left and right batches of batch_size tuples fed L0,R0,L1,R1,...
 * batch_counts (2*n_batches) receives each batch's matches in arrival order;
 * window_counts receives per-window totals (at most max_windows); returns the
 * number of windows seen, or -1 on bad arguments. */
int64_t oracle_eager_hj(const sjbg_tuple *left, const sjbg_tuple *right, uint64_t n_batches, uint64_t batch_size,
                        uint64_t window_size, uint64_t distinct_keys,
                        uint64_t *batch_counts, uint64_t *window_counts, uint64_t max_windows);

/* ---- result restatement ---- */
int oracle_join(const sjbg_tuple *left, uint64_t n_left, const sjbg_tuple *right, uint64_t n_right,
                int enumerate, sjbg_pair *pairs, uint64_t pairs_capacity, oracle_result *out);
/* Many windows (descriptors as in the C ABI); results[i] for window i. */
int oracle_join_windows(const sjbg_tuple *left, const sjbg_tuple *right, const sjbg_window_desc *windows,
                        uint32_t n_windows, int enumerate, sjbg_pair *pairs, oracle_result *results, int threads);

#ifdef __cplusplus
}
#endif
#endif
