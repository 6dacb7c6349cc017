// tune.cu - autotuner of the hash join's partitioning parameters.
//
// No reference counterpart.  For a batch shape (algorithm, partitioner,
// enumeration, log2 of the tuples and of the windows) not seen before, the
// candidate settings - left tuples per bucket (which sets the partition
// fan-out), persistent vs one-CTA-per-bucket joins and, for SJBG_PART_AUTO
// handles, one HBM table per window vs radix partitioning - are each run on the
// batch itself, timed with CUDA events, and the fastest is kept.  Decisions
// are persisted as JSON lines in $SJBG_TUNE_CACHE (default
// ~/.cache/sjbg_tune.json) and reloaded by later handles.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include <sys/stat.h>

#include "runtime.h"

namespace sjbg {

static std::string tune_path() {
    const char *p = std::getenv("SJBG_TUNE_CACHE");
    if (p && *p) return p;
    const char *home = std::getenv("HOME");
    return std::string(home && *home ? home : "/tmp") + "/.cache/sjbg_tune.json";
}

static void tune_load(sjbg_handle *h) {
    if (h->tune_loaded) return;
    h->tune_loaded = true;
    std::ifstream f(tune_path());
    std::string line;
    while (std::getline(f, line)) {
        char shape[256] = {0};
        unsigned target = 0, persistent = 0, part = 0;
        float ms = 0.f;
        if (std::sscanf(line.c_str(),
                        " {\"shape\": \"%255[^\"]\", \"bucket_target\": %u, \"persistent\": %u, \"partitioner\": %u, \"ms\": %f",
                        shape, &target, &persistent, &part, &ms) == 5 &&
            (target == 2048 || target == 4096 || target == 8192) && part <= SJBG_PART_LEARNED) {
            sjbg_handle::Tune t;
            t.bucket_target = target;
            t.persistent_join = persistent != 0;
            t.partitioner = part;
            t.ms = ms;
            h->tuned[shape] = t;
        }
    }
}

static void tune_save(const sjbg_handle *h) {
    const std::string path = tune_path();
    const size_t slash = path.find_last_of('/');
    if (slash != std::string::npos) {
        const std::string dir = path.substr(0, slash);
        for (size_t i = 1; i <= dir.size(); i++)   // create the cache directory, level by level
            if (i == dir.size() || dir[i] == '/') mkdir(dir.substr(0, i).c_str(), 0755);
    }
    std::ofstream f(path, std::ios::trunc);
    if (!f) return;   // a read-only home only loses the cache
    for (const auto &kv : h->tuned)
        f << "{\"shape\": \"" << kv.first << "\", \"bucket_target\": " << kv.second.bucket_target
          << ", \"persistent\": " << (kv.second.persistent_join ? 1 : 0) << ", \"partitioner\": "
          << kv.second.partitioner << ", \"ms\": " << kv.second.ms << "}\n";
}

static uint32_t log2u(uint64_t x) {
    uint32_t b = 0;
    while (x > 1) { x >>= 1; b++; }
    return b;
}

int autotune_lazy(sjbg_handle *h, const sjbg_tuple *dL, const sjbg_tuple *dR, const WinHost *wins, uint32_t n,
                  bool enumerate) {
    if (h->cfg.algorithm != SJBG_ALG_HJ || n == 0) return SJBG_OK;   // only the hash join has tunables
    if (std::getenv("SJBG_BUCKET_TARGET") || std::getenv("SJBG_PERSISTENT_JOIN")) return SJBG_OK;   // pinned by the user
    tune_load(h);
    uint64_t total = 0;
    for (uint32_t w = 0; w < n; w++) total += wins[w].n_left + wins[w].n_right;
    char key[160];
    std::snprintf(key, sizeof(key), "hj-part%u-enum%d-t%u-w%u-sm%d", h->cfg.partitioner, enumerate ? 1 : 0,
                  log2u(total), log2u(n), h->num_sms);
    auto it = h->tuned.find(key);
    if (it != h->tuned.end()) {
        h->tune = it->second;
        return SJBG_OK;
    }
    WinAcc *hAcc = static_cast<WinAcc *>(pinned_get(h, 3, sizeof(WinAcc) * (n + 1)));
    if (!hAcc) return fail(h, SJBG_E_NOMEM, "tuner staging");
    cudaEvent_t e0 = event_get(h), e1 = event_get(h);
    sjbg_handle::Tune best;
    best.ms = 1e30f;
    // partitioners tried: the configured one, or for SJBG_PART_AUTO the HBM
    // table and radix partitioning
    std::vector<uint32_t> parts;
    if (h->cfg.partitioner == SJBG_PART_AUTO) parts = {SJBG_PART_NONE, SJBG_PART_RADIX};
    else parts = {0u};
    for (uint32_t part : parts)
    for (uint32_t target : {2048u, 4096u, 8192u}) {
        for (bool persistent : {false, true}) {
            if (enumerate && persistent) continue;   // chain-building joins run one CTA per bucket
            if (part == SJBG_PART_NONE && (target != 4096u || !persistent)) continue;   // no buckets to tune
            h->tune.partitioner = part;
            h->tune.bucket_target = target;
            h->tune.persistent_join = persistent;
            uint32_t pu;
            int rc = run_lazy_device(h, dL, dR, wins, n, nullptr, hAcc, &pu);   // warm-up (sizes buffers)
            if (rc) return rc;
            SJBG_CK(h, cudaStreamSynchronize(h->stream));
            SJBG_CK(h, cudaEventRecord(e0, h->stream));
            rc = run_lazy_device(h, dL, dR, wins, n, nullptr, hAcc, &pu);
            if (rc) return rc;
            SJBG_CK(h, cudaEventRecord(e1, h->stream));
            SJBG_CK(h, cudaStreamSynchronize(h->stream));
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best.ms) {
                best = h->tune;
                best.ms = ms;
            }
        }
    }
    profile_collect(h);
    h->event_pool.push_back(e0);
    h->event_pool.push_back(e1);
    h->tune = best;
    h->tuned[key] = best;
    tune_save(h);
    return SJBG_OK;
}

}  // namespace sjbg
