// ref_wrap.cpp - C entry points around the reference's own CPU joiner classes
// (test infrastructure of the oracle only).
//
// Built by oracle/Makefile together with the reference's unmodified sources
//   src/sjb/windowing/lazy/executor/CPU/CPU_HJ.cpp
//   src/sjb/windowing/lazy/executor/CPU/CPU_SMJ.cpp
//   src/sjb/windowing/lazy/executor/CPU/CPU_NLJ.cpp
//   src/sjb/windowing/eager/executor/CPU/CPU_HJ.cpp
// into oracle/_ref/libsjbref.so.  It is used to pin the C restatement in
// sjb_oracle.c and to produce the golden fixtures under tests/golden/.
#include <cstdint>
#include <cstring>
#include <memory>
#include <new>
#include <vector>

#include <sjb/sink/Sink.h>
#include <sjb/utils/Tuple.hpp>
#include <sjb/windowing/eager/executor/CPU/CPU_HJ.hpp>
#include <sjb/windowing/lazy/executor/CPU/CPU_HJ.hpp>
#include <sjb/windowing/lazy/executor/CPU/CPU_NLJ.hpp>
#include <sjb/windowing/lazy/executor/CPU/CPU_SMJ.hpp>

namespace {
// The CPU joiners take a Sink& but never touch it (they return their count in
// ExecutionStatistic / as the return value).  Sink's constructor allocates
// pinned memory through the CUDA runtime, so an unconstructed, suitably
// aligned block stands in for it.
alignas(Sink) unsigned char g_sink_storage[sizeof(Sink)];
Sink &dummy_sink() { return *reinterpret_cast<Sink *>(g_sink_storage); }

std::vector<uint64_t> batch_offsets(uint64_t n, uint64_t batch) {
    std::vector<uint64_t> v;
    for (uint64_t o = 0; o + batch <= n; o += batch) v.push_back(o);
    return v;
}
}  // namespace

extern "C" {

// Lazy CPU_HJ::execute on one window laid out as whole batches.
int ref_lazy_hj_count(const Tuple *left, uint64_t n_left, const Tuple *right, uint64_t n_right,
                      uint64_t distinct_keys, uint64_t batch_size, uint64_t probe_threads, uint64_t *count) {
    if (!batch_size || n_left % batch_size || n_right % batch_size) return -1;
    Windowing::Lazy::Executor::CPU_HJ joiner(distinct_keys, batch_size, probe_threads, n_left);
    auto es = joiner.execute(const_cast<Tuple *>(left), const_cast<Tuple *>(right),
                             batch_offsets(n_left, batch_size), batch_offsets(n_right, batch_size), dummy_sink());
    *count = es.resultCount;
    return 0;
}

int ref_lazy_smj_count(const Tuple *left, uint64_t n_left, const Tuple *right, uint64_t n_right,
                       uint64_t distinct_keys, uint64_t batch_size, uint64_t sort_threads, uint64_t *count) {
    if (!batch_size || n_left % batch_size || n_right % batch_size) return -1;
    Windowing::Lazy::Executor::CPU_SMJ joiner(distinct_keys, batch_size, sort_threads);
    auto es = joiner.execute(const_cast<Tuple *>(left), const_cast<Tuple *>(right),
                             batch_offsets(n_left, batch_size), batch_offsets(n_right, batch_size), dummy_sink());
    *count = es.resultCount;
    return 0;
}

int ref_lazy_nlj_count(const Tuple *left, uint64_t n_left, const Tuple *right, uint64_t n_right,
                       uint64_t batch_size, uint64_t *count) {
    if (!batch_size || n_left % batch_size || n_right % batch_size) return -1;
    Windowing::Lazy::Executor::CPU_NLJ joiner(batch_size);
    auto es = joiner.execute(const_cast<Tuple *>(left), const_cast<Tuple *>(right),
                             batch_offsets(n_left, batch_size), batch_offsets(n_right, batch_size), dummy_sink());
    *count = es.resultCount;
    return 0;
}

// Eager CPU_HJ fed in the order Source::start produces (left batch i, then
// right batch i; src/sjb/source/Source.cpp:20-28) with the window close rule
// of Eager::CountBased::onIncoming{Left,Right}
// (include/sjb/windowing/eager/CountBased.cuh:36-72).  batch_counts gets
// 2*n_batches entries; returns the number of windows, -1 on bad arguments.
int64_t ref_eager_hj(const Tuple *left, const Tuple *right, uint64_t n_batches, uint64_t batch_size,
                     uint64_t window_size, uint64_t distinct_keys, uint64_t *batch_counts,
                     uint64_t *window_counts, uint64_t max_windows) {
    if (!batch_size || !window_size || !distinct_keys) return -1;
    // The reference sizes each side's table as maxTupleInWindow slots per key
    // (CPU_HJ.cpp:12-13); a side never exceeds window_size + batch_size - 1.
    auto joiner = std::make_unique<Windowing::Eager::Executor::CPU_HJ>(window_size + batch_size, distinct_keys,
                                                                       batch_size);
    uint64_t tot[2] = {0, 0};
    int64_t window = 0;
    uint64_t wsum = 0;
    for (uint64_t b = 0; b < n_batches; b++) {
        for (int side = 0; side < 2; side++) {
            if (tot[0] >= window_size || tot[1] >= window_size) {
                joiner->clearStates();
                tot[0] = tot[1] = 0;
                if (window_counts && (uint64_t)window < max_windows) window_counts[window] = wsum;
                window++;
                wsum = 0;
            }
            Tuple *batch = const_cast<Tuple *>((side == 0 ? left : right) + b * batch_size);
            uint64_t c = joiner->execute(batch, side == 0, tot[side], dummy_sink());
            if (batch_counts) batch_counts[2 * b + side] = c;
            wsum += c;
            tot[side] += batch_size;
        }
    }
    if (n_batches) {
        if (window_counts && (uint64_t)window < max_windows) window_counts[window] = wsum;
        window++;
    }
    return window;
}

}  // extern "C"
