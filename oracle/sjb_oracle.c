/*
 * sjb_oracle.c - CPU oracle (test infrastructure only; see sjb_oracle.h).
 *
 * Each function cites the reference lines it restates.  The restatements
 * keep the reference's data structures and loop order (so they can serve as
 * the timed CPU baseline) and differ only where noted:
 *  - counting loops of the form `for i in range: for j in range: count++`
 *    (CPU_SMJ.cpp:104-125) are written as count += n_i * n_j, which is what
 *    an optimising compiler emits for them;
 *  - TBB arenas become POSIX threads with the same work split.
 */
#define _GNU_SOURCE
#include "sjb_oracle.h"
#include "../gpu-stream-join-benchmark_gb300/csrc/sjbg_gen.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------- */
/* small thread helper                                                        */
/* ------------------------------------------------------------------------- */
typedef void (*range_fn)(void *ctx, uint64_t begin, uint64_t end, int tid);
typedef struct { range_fn fn; void *ctx; uint64_t b, e; int tid; } range_job;
static void *range_tramp(void *p) { range_job *j = (range_job *)p; j->fn(j->ctx, j->b, j->e, j->tid); return NULL; }

static void parallel_range(uint64_t n, int threads, range_fn fn, void *ctx) {
    if (threads < 1) threads = 1;
    if ((uint64_t)threads > n) threads = n ? (int)n : 1;
    if (threads == 1) { fn(ctx, 0, n, 0); return; }
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * threads);
    range_job *jobs = (range_job *)malloc(sizeof(range_job) * threads);
    for (int t = 0; t < threads; t++) {
        jobs[t].fn = fn; jobs[t].ctx = ctx; jobs[t].tid = t;
        jobs[t].b = n * (uint64_t)t / threads; jobs[t].e = n * (uint64_t)(t + 1) / threads;
        pthread_create(&th[t], NULL, range_tramp, &jobs[t]);
    }
    for (int t = 0; t < threads; t++) pthread_join(th[t], NULL);
    free(th); free(jobs);
}

/* ------------------------------------------------------------------------- */
/* generators                                                                 */
/* ------------------------------------------------------------------------- */
typedef struct { sjbg_tuple *out; uint64_t first, seed, domain, perm_seed; const uint64_t *table; } gen_ctx;

static void gen_uniform_range(void *p, uint64_t b, uint64_t e, int tid) {
    (void)tid;
    gen_ctx *c = (gen_ctx *)p;
    for (uint64_t i = b; i < e; i++) {
        uint64_t g = c->first + i;
        c->out[i].key = sjbg_uniform_key(c->seed, g, c->domain);
        c->out[i].val = (uint32_t)g;
        c->out[i].ts = g;
    }
}

void oracle_gen_uniform(sjbg_tuple *out, uint64_t first, uint64_t n, uint64_t seed, uint64_t domain, int threads) {
    gen_ctx c = {out, first, seed, domain, 0, NULL};
    parallel_range(n, threads, gen_uniform_range, &c);
}

void oracle_zipf_table(uint64_t *table, uint64_t n, double z) { sjbg_zipf_table_fill(table, n, z); }

static void gen_zipf_range(void *p, uint64_t b, uint64_t e, int tid) {
    (void)tid;
    gen_ctx *c = (gen_ctx *)p;
    for (uint64_t i = b; i < e; i++) {
        uint64_t g = c->first + i;
        uint32_t rank = sjbg_zipf_rank(c->table, c->domain, sjbg_rand64(c->seed, g));
        c->out[i].key = sjbg_perm(rank, c->domain, c->perm_seed);
        c->out[i].val = (uint32_t)g;
        c->out[i].ts = g;
    }
}

void oracle_gen_zipf(sjbg_tuple *out, uint64_t first, uint64_t n, uint64_t seed,
                     const uint64_t *table, uint64_t domain, uint64_t perm_seed, int threads) {
    gen_ctx c = {out, first, seed, domain, perm_seed, table};
    parallel_range(n, threads, gen_zipf_range, &c);
}

uint32_t oracle_perm(uint64_t rank, uint64_t domain, uint64_t seed) { return sjbg_perm(rank, domain, seed); }
uint64_t oracle_log_uniform(uint64_t seed, uint64_t w, uint64_t lo, uint64_t hi) { return sjbg_log_uniform(seed, w, lo, hi); }
uint64_t oracle_pair_hash(uint32_t r, uint32_t s) { return sjbg_pair_hash(r, s); }
uint64_t oracle_fr(uint32_t r) { return sjbg_fr(r); }
uint64_t oracle_gs(uint32_t s) { return sjbg_gs(s); }

/* ------------------------------------------------------------------------- */
/* lazy CPU_HJ  (src/sjb/windowing/lazy/executor/CPU/CPU_HJ.cpp:30-136)       */
/* ------------------------------------------------------------------------- */
typedef struct {
    const sjbg_tuple *right;
    const sjbg_tuple *store;
    const uint64_t *occupation, *prefix;
    uint64_t dk, batch;
    uint64_t *partial; /* per thread */
} hj_probe_ctx;

/* CPU_HJ::probe (CPU_HJ.cpp:101-119): scan bucket [prefix[h], prefix[h]+occ[h])
 * and count entries whose key equals the hash.  The probe side is split by
 * batches over the threads, as tbb::parallel_for_each over
 * rightIndexesToJoin does (CPU_HJ.cpp:54-65). */
static void hj_probe_range(void *p, uint64_t b, uint64_t e, int tid) {
    hj_probe_ctx *c = (hj_probe_ctx *)p;
    uint64_t count = 0;
    for (uint64_t batch = b; batch < e; batch++) {
        uint64_t lo = batch * c->batch, hi = lo + c->batch;
        for (uint64_t i = lo; i < hi; i++) {
            uint64_t h = c->right[i].key % c->dk;
            uint64_t occ = c->occupation[h], ps = c->prefix[h];
            for (uint64_t j = ps; j < ps + occ; j++) count += (h == c->store[j].key);
        }
    }
    c->partial[tid] = count;
}

int oracle_lazy_hj_count(const sjbg_tuple *left, uint64_t n_left, const sjbg_tuple *right, uint64_t n_right,
                         uint64_t distinct_keys, uint64_t batch_size, int probe_threads, uint64_t *count) {
    if (!distinct_keys) return -1;
    for (uint64_t i = 0; i < n_left; i++) if (left[i].key >= distinct_keys) return -1;
    for (uint64_t i = 0; i < n_right; i++) if (right[i].key >= distinct_keys) return -1;
    if (batch_size == 0) batch_size = n_left > n_right ? n_left : n_right;
    if (batch_size == 0) { *count = 0; return 0; }
    if (n_left % batch_size || n_right % batch_size) return -1; /* windows are whole batches */

    uint64_t *occupation = (uint64_t *)calloc(distinct_keys, sizeof(uint64_t));
    uint64_t *inserted = (uint64_t *)calloc(distinct_keys, sizeof(uint64_t));
    uint64_t *prefix = (uint64_t *)calloc(distinct_keys, sizeof(uint64_t));
    sjbg_tuple *store = (sjbg_tuple *)malloc(sizeof(sjbg_tuple) * (n_left ? n_left : 1));

    /* computePrefixSum per left batch (CPU_HJ.cpp:41-44,121-136): occupation
     * is indexed by key and the whole prefix array is recomputed per batch. */
    for (uint64_t b = 0; b < n_left; b += batch_size) {
        for (uint64_t i = b; i < b + batch_size; i++) occupation[left[i].key]++;
        uint64_t run = 0;
        for (uint64_t k = 0; k < distinct_keys; k++) { prefix[k] = run; run += occupation[k]; }
    }
    /* build (CPU_HJ.cpp:45-48,84-99): scatter to prefix[h] + inserted[h]. */
    for (uint64_t i = 0; i < n_left; i++) {
        uint64_t h = left[i].key % distinct_keys;
        store[prefix[h] + inserted[h]] = left[i];
        inserted[h]++;
    }
    /* probe (CPU_HJ.cpp:52-65). */
    int threads = probe_threads < 1 ? 1 : probe_threads;
    uint64_t *partial = (uint64_t *)calloc(threads, sizeof(uint64_t));
    hj_probe_ctx c = {right, store, occupation, prefix, distinct_keys, batch_size, partial};
    parallel_range(n_right / batch_size, threads, hj_probe_range, &c);
    uint64_t total = 0;
    for (int t = 0; t < threads; t++) total += partial[t];
    *count = total;
    free(partial); free(occupation); free(inserted); free(prefix); free(store);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* lazy CPU_SMJ (src/sjb/windowing/lazy/executor/CPU/CPU_SMJ.cpp:23-139)      */
/* ------------------------------------------------------------------------- */
static int cmp_tuple_key(const void *a, const void *b) {
    uint32_t x = ((const sjbg_tuple *)a)->key, y = ((const sjbg_tuple *)b)->key;
    return (x > y) - (x < y);
}

typedef struct { sjbg_tuple *buf; uint64_t n; int parts; } psort_ctx;
static void psort_chunk(void *p, uint64_t b, uint64_t e, int tid) {
    (void)e; (void)tid;
    psort_ctx *c = (psort_ctx *)p;
    uint64_t lo = c->n * b / c->parts, hi = c->n * (b + 1) / c->parts;
    qsort(c->buf + lo, hi - lo, sizeof(sjbg_tuple), cmp_tuple_key);
}
typedef struct { sjbg_tuple *src, *dst; uint64_t n; int parts, width; } pmerge_ctx;
static void pmerge_pair(void *p, uint64_t b, uint64_t e, int tid) {
    (void)tid;
    pmerge_ctx *c = (pmerge_ctx *)p;
    for (uint64_t m = b; m < e; m++) {
        int p0 = (int)m * 2 * c->width, p1 = p0 + c->width, p2 = p0 + 2 * c->width;
        if (p1 > c->parts) p1 = c->parts;
        if (p2 > c->parts) p2 = c->parts;
        uint64_t a = c->n * p0 / c->parts, am = c->n * p1 / c->parts, ae = c->n * p2 / c->parts;
        uint64_t i = a, j = am, o = a;
        while (i < am && j < ae) c->dst[o++] = (c->src[j].key < c->src[i].key) ? c->src[j++] : c->src[i++];
        while (i < am) c->dst[o++] = c->src[i++];
        while (j < ae) c->dst[o++] = c->src[j++];
    }
}

/* Parallel sort by key standing in for tbb::parallel_sort (CPU_SMJ.cpp:88-94):
 * sort `threads` chunks concurrently, then merge pairwise in parallel rounds. */
static void parallel_sort_by_key(sjbg_tuple *buf, uint64_t n, int threads) {
    if (threads <= 1 || n < 4096) { qsort(buf, n, sizeof(sjbg_tuple), cmp_tuple_key); return; }
    psort_ctx sc = {buf, n, threads};
    parallel_range(threads, threads, psort_chunk, &sc);
    sjbg_tuple *tmp = (sjbg_tuple *)malloc(sizeof(sjbg_tuple) * n);
    sjbg_tuple *src = buf, *dst = tmp;
    for (int width = 1; width < threads; width *= 2) {
        pmerge_ctx mc = {src, dst, n, threads, width};
        uint64_t merges = (threads + 2 * width - 1) / (2 * width);
        parallel_range(merges, threads, pmerge_pair, &mc);
        sjbg_tuple *t = src; src = dst; dst = t;
    }
    if (src != buf) memcpy(buf, src, sizeof(sjbg_tuple) * n);
    free(tmp);
}

int oracle_lazy_smj_count(const sjbg_tuple *left, uint64_t n_left, const sjbg_tuple *right, uint64_t n_right,
                          uint64_t distinct_keys, int sort_threads, uint64_t *count) {
    if (!distinct_keys) return -1;
    uint64_t *lh = (uint64_t *)calloc(distinct_keys, sizeof(uint64_t));
    uint64_t *rh = (uint64_t *)calloc(distinct_keys, sizeof(uint64_t));
    sjbg_tuple *lb = (sjbg_tuple *)malloc(sizeof(sjbg_tuple) * (n_left ? n_left : 1));
    sjbg_tuple *rb = (sjbg_tuple *)malloc(sizeof(sjbg_tuple) * (n_right ? n_right : 1));
    int bad = 0;
    /* histogram + copy to the local buffers (CPU_SMJ.cpp:41-66); the
     * reference copies val = key on the left side (:48), which the count
     * does not see. */
    for (uint64_t i = 0; i < n_left; i++) {
        if (left[i].key >= distinct_keys) { bad = 1; break; }
        lh[left[i].key]++;
        lb[i].key = left[i].key; lb[i].val = left[i].key; lb[i].ts = left[i].ts;
    }
    for (uint64_t i = 0; i < n_right && !bad; i++) {
        if (right[i].key >= distinct_keys) { bad = 1; break; }
        rh[right[i].key]++;
        rb[i] = right[i];
    }
    if (bad) { free(lh); free(rh); free(lb); free(rb); return -1; }
    /* prefix sums (CPU_SMJ.cpp:71-83) */
    uint64_t *lp = (uint64_t *)malloc(sizeof(uint64_t) * distinct_keys);
    uint64_t *rp = (uint64_t *)malloc(sizeof(uint64_t) * distinct_keys);
    uint64_t run = 0;
    for (uint64_t k = 0; k < distinct_keys; k++) { lp[k] = run; run += lh[k]; }
    run = 0;
    for (uint64_t k = 0; k < distinct_keys; k++) { rp[k] = run; run += rh[k]; }
    /* sort both relations by key (CPU_SMJ.cpp:88-94) */
    parallel_sort_by_key(lb, n_left, sort_threads);
    parallel_sort_by_key(rb, n_right, sort_threads);
    /* merge: per key, the cartesian product of its two runs (CPU_SMJ.cpp:99-125);
     * the last key's runs extend to the end of the buffers (:106-115). */
    uint64_t c = 0;
    for (uint64_t k = 0; k < distinct_keys; k++) {
        uint64_t le = (k + 1 == distinct_keys) ? n_left : lp[k + 1];
        uint64_t re = (k + 1 == distinct_keys) ? n_right : rp[k + 1];
        c += (le - lp[k]) * (re - rp[k]);
    }
    *count = c;
    free(lh); free(rh); free(lb); free(rb); free(lp); free(rp);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* lazy CPU_NLJ (src/sjb/windowing/lazy/executor/CPU/CPU_NLJ.cpp:11-32)       */
/* ------------------------------------------------------------------------- */
uint64_t oracle_lazy_nlj_count(const sjbg_tuple *left, uint64_t n_left, const sjbg_tuple *right, uint64_t n_right) {
    uint64_t counter = 0;
    for (uint64_t j = 0; j < n_left; j++)
        for (uint64_t l = 0; l < n_right; l++) counter += (left[j].key == right[l].key);
    return counter;
}

/* ------------------------------------------------------------------------- */
/* eager CPU_HJ + Eager::CountBased feeding                                   */
/* (src/sjb/windowing/eager/executor/CPU/CPU_HJ.cpp:27-82,                    */
/*  include/sjb/windowing/eager/CountBased.cuh:36-72, src/sjb/source/Source.cpp:20-28) */
/* ------------------------------------------------------------------------- */
typedef struct { uint64_t *head; uint64_t *next; uint32_t *keys; uint64_t n; } eager_side;
#define EAGER_NIL UINT64_MAX

static void eager_clear(eager_side *s, uint64_t dk) {   /* CPU_HJ::clearStates (:27-33) */
    for (uint64_t h = 0; h < dk; h++) s->head[h] = EAGER_NIL;
    s->n = 0;
}
/* CPU_HJ::build (:50-65): append each tuple to bucket key % numDistinctKeys. */
static void eager_build(eager_side *s, const sjbg_tuple *t, uint64_t n, uint64_t dk) {
    for (uint64_t i = 0; i < n; i++) {
        uint64_t h = t[i].key % dk;
        s->keys[s->n] = t[i].key;
        s->next[s->n] = s->head[h];
        s->head[h] = s->n;
        s->n++;
    }
}
/* CPU_HJ::probe (:67-82): compare keys inside the other side's bucket. */
static uint64_t eager_probe(const eager_side *s, const sjbg_tuple *t, uint64_t n, uint64_t dk) {
    uint64_t c = 0;
    for (uint64_t i = 0; i < n; i++) {
        uint64_t h = t[i].key % dk;
        for (uint64_t j = s->head[h]; j != EAGER_NIL; j = s->next[j]) c += (s->keys[j] == t[i].key);
    }
    return c;
}

int64_t oracle_eager_hj(const sjbg_tuple *left, const sjbg_tuple *right, uint64_t n_batches, uint64_t batch_size,
                        uint64_t window_size, uint64_t distinct_keys,
                        uint64_t *batch_counts, uint64_t *window_counts, uint64_t max_windows) {
    if (!batch_size || !window_size || !distinct_keys) return -1;
    /* A side holds at most window_size + batch_size - 1 tuples: the window
     * closes before a batch once either side has >= window_size
     * (CountBased.cuh:38-46). */
    uint64_t cap = window_size + batch_size;
    eager_side sides[2];
    for (int s = 0; s < 2; s++) {
        sides[s].head = (uint64_t *)malloc(sizeof(uint64_t) * distinct_keys);
        sides[s].next = (uint64_t *)malloc(sizeof(uint64_t) * cap);
        sides[s].keys = (uint32_t *)malloc(sizeof(uint32_t) * cap);
        eager_clear(&sides[s], distinct_keys);
    }
    uint64_t tot[2] = {0, 0};
    int64_t window = 0;
    uint64_t wsum = 0;
    for (uint64_t b = 0; b < n_batches; b++) {
        for (int side = 0; side < 2; side++) {          /* onIncomingLeft then onIncomingRight */
            if (tot[0] >= window_size || tot[1] >= window_size) {
                eager_clear(&sides[0], distinct_keys);
                eager_clear(&sides[1], distinct_keys);
                tot[0] = tot[1] = 0;
                if (window_counts && (uint64_t)window < max_windows) window_counts[window] = wsum;
                window++;
                wsum = 0;
            }
            const sjbg_tuple *batch = (side == 0 ? left : right) + b * batch_size;
            eager_build(&sides[side], batch, batch_size, distinct_keys);
            uint64_t c = eager_probe(&sides[1 - side], batch, batch_size, distinct_keys);
            if (batch_counts) batch_counts[2 * b + side] = c;
            wsum += c;
            tot[side] += batch_size;
        }
    }
    if (n_batches) {
        if (window_counts && (uint64_t)window < max_windows) window_counts[window] = wsum;
        window++;
    }
    for (int s = 0; s < 2; s++) { free(sides[s].head); free(sides[s].next); free(sides[s].keys); }
    return window;
}

/* ------------------------------------------------------------------------- */
/* result restatement                                                         */
/* ------------------------------------------------------------------------- */
static int cmp_u64(const void *a, const void *b) {
    uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return (x > y) - (x < y);
}

/* Group both sides on key (sorted (key, val) composites), then per common key
 * k: count += |L_k||R_k|, prod += (sum fr)(sum gs); when enumerating, every
 * pair contributes pair_hash to xor and is appended to the pair list, which is
 * finally sorted by (r, s). */
int oracle_join(const sjbg_tuple *left, uint64_t n_left, const sjbg_tuple *right, uint64_t n_right,
                int enumerate, sjbg_pair *pairs, uint64_t pairs_capacity, oracle_result *out) {
    uint64_t *l = (uint64_t *)malloc(sizeof(uint64_t) * (n_left ? n_left : 1));
    uint64_t *r = (uint64_t *)malloc(sizeof(uint64_t) * (n_right ? n_right : 1));
    if (!l || !r) { free(l); free(r); return -1; }
    for (uint64_t i = 0; i < n_left; i++) l[i] = ((uint64_t)left[i].key << 32) | left[i].val;
    for (uint64_t i = 0; i < n_right; i++) r[i] = ((uint64_t)right[i].key << 32) | right[i].val;
    qsort(l, n_left, sizeof(uint64_t), cmp_u64);
    qsort(r, n_right, sizeof(uint64_t), cmp_u64);
    uint64_t count = 0, xr = 0, prod = 0, np = 0;
    uint64_t i = 0, j = 0;
    while (i < n_left && j < n_right) {
        uint32_t kl = (uint32_t)(l[i] >> 32), kr = (uint32_t)(r[j] >> 32);
        if (kl < kr) { i++; continue; }
        if (kr < kl) { j++; continue; }
        uint64_t ie = i, je = j, sf = 0, sg = 0;
        while (ie < n_left && (uint32_t)(l[ie] >> 32) == kl) sf += sjbg_fr((uint32_t)l[ie++]);
        while (je < n_right && (uint32_t)(r[je] >> 32) == kl) sg += sjbg_gs((uint32_t)r[je++]);
        count += (ie - i) * (je - j);
        prod += sf * sg;
        if (enumerate) {
            for (uint64_t a = i; a < ie; a++)
                for (uint64_t b = j; b < je; b++) {
                    uint32_t rv = (uint32_t)l[a], sv = (uint32_t)r[b];
                    xr ^= sjbg_pair_hash(rv, sv);
                    if (pairs && np < pairs_capacity) { pairs[np].r = rv; pairs[np].s = sv; }
                    np++;
                }
        }
        i = ie; j = je;
    }
    if (pairs && enumerate) {
        uint64_t w = np < pairs_capacity ? np : pairs_capacity;
        uint64_t *tmp = (uint64_t *)malloc(sizeof(uint64_t) * (w ? w : 1));
        for (uint64_t k = 0; k < w; k++) tmp[k] = ((uint64_t)pairs[k].r << 32) | pairs[k].s;
        qsort(tmp, w, sizeof(uint64_t), cmp_u64);
        for (uint64_t k = 0; k < w; k++) { pairs[k].r = (uint32_t)(tmp[k] >> 32); pairs[k].s = (uint32_t)tmp[k]; }
        free(tmp);
        np = w;
    } else {
        np = 0;
    }
    out->count = count;
    out->xor_checksum = enumerate ? xr : 0;
    out->prod_checksum = prod;
    out->n_pairs = np;
    free(l); free(r);
    return 0;
}

typedef struct {
    const sjbg_tuple *left, *right;
    const sjbg_window_desc *w;
    int enumerate;
    sjbg_pair *pairs;
    oracle_result *res;
    int err;
} jw_ctx;

static void join_windows_range(void *p, uint64_t b, uint64_t e, int tid) {
    (void)tid;
    jw_ctx *c = (jw_ctx *)p;
    for (uint64_t k = b; k < e; k++) {
        const sjbg_window_desc *d = &c->w[k];
        sjbg_pair *pp = (c->pairs && d->pairs_capacity) ? c->pairs + d->pairs_offset : NULL;
        if (oracle_join(c->left + d->left_offset, d->n_left, c->right + d->right_offset, d->n_right,
                        c->enumerate, pp, d->pairs_capacity, &c->res[k]))
            c->err = 1;
    }
}

int oracle_join_windows(const sjbg_tuple *left, const sjbg_tuple *right, const sjbg_window_desc *windows,
                        uint32_t n_windows, int enumerate, sjbg_pair *pairs, oracle_result *results, int threads) {
    jw_ctx c = {left, right, windows, enumerate, pairs, results, 0};
    parallel_range(n_windows, threads, join_windows_range, &c);
    return c.err ? -1 : 0;
}
