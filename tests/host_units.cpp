// host_units.cpp - unit driver of the host windowing (gpu-stream-join-benchmark_gb300/host)
// with CPU stand-in executors, so the windowing logic runs without a GPU.
//
//   host_units ring    the lazy ring buffer runs out of free batch slots while a
//                      window is being joined: "Ring buffer is full" is thrown
//                      (the reference exits the process there,
//                      include/sjb/windowing/lazy/CountBased.cuh:55-63), and the
//                      windowing goes on once the join returns.
//   host_units eager   eight source threads feed the eager windowing: the close
//                      check, the batch's execution and the window counters run
//                      as one step, so the executor is never entered twice at
//                      once and every batch's matches land in the window it
//                      joined (sum of batch counts == sum of window totals).
// Each mode prints key=value lines for tests/test_host_harness.py.
#include <atomic>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "sjb_host.hpp"

namespace {

// A lazy executor whose first call blocks until released.
struct BlockingLazy : Windowing::Lazy::Executor::BaseLazyExecutor {
    std::mutex m;
    std::condition_variable cv;
    bool entered = false, released = false;
    uint64_t calls = 0;
    ExecutionStatistic execute(Tuple *, Tuple *, std::vector<uint64_t> l, std::vector<uint64_t> r, Sink &) override {
        std::unique_lock<std::mutex> g(m);
        entered = true;
        cv.notify_all();
        cv.wait(g, [&] { return released; });
        calls++;
        ExecutionStatistic s;
        s.resultCount = l.size() * 1000 + r.size();
        return s;
    }
};

int ring_mode() {
    const uint64_t B = 4;
    std::vector<Tuple> data(8 * B);
    for (uint64_t i = 0; i < data.size(); i++) data[i] = Tuple{(uint32_t)(i % 3), (uint32_t)i, i};
    Sink sink;
    auto ex = std::make_shared<BlockingLazy>();
    std::vector<std::shared_ptr<Windowing::Lazy::Executor::BaseLazyExecutor>> pool{ex};
    Windowing::Lazy::CountBased cb(sink, 2 * B, 5, 2 * B, B, pool, "blocking");
    std::thread a([&] {
        cb.onIncomingLeft(&data[0]);
        cb.onIncomingRight(&data[B]);
        cb.onIncomingLeft(&data[2 * B]);
        cb.onIncomingRight(&data[3 * B]);   // completes the window: the join blocks here
    });
    {
        std::unique_lock<std::mutex> g(ex->m);
        ex->cv.wait(g, [&] { return ex->entered; });
    }
    int thrown = 0;
    std::string what;
    try {
        cb.onIncomingLeft(&data[4 * B]);   // both left slots belong to the window being joined
    } catch (const std::runtime_error &e) {
        thrown = 1;
        what = e.what();
    }
    {
        std::lock_guard<std::mutex> g(ex->m);
        ex->released = true;
    }
    ex->cv.notify_all();
    a.join();
    // the slots are free again: a second window goes through
    cb.onIncomingLeft(&data[4 * B]);
    cb.onIncomingRight(&data[5 * B]);
    cb.onIncomingLeft(&data[6 * B]);
    cb.onIncomingRight(&data[7 * B]);
    std::printf("ring_full_thrown=%d\nmessage=%s\nwindows=%lu\nmatch_count=%lu\n", thrown, what.c_str(),
                (unsigned long)sink.getExecutedWindows(), (unsigned long)sink.getMatchCount());
    return 0;
}

// An exact eager hash join on the CPU that notices concurrent calls.
struct CpuEager : Windowing::Eager::Executor::BaseEagerExecutor {
    explicit CpuEager(uint64_t batch) : batch(batch) {}
    uint64_t batch;
    std::unordered_map<uint32_t, uint64_t> side[2];
    uint64_t open = 0;              // matches of the open window
    uint64_t closedTotal = 0, closedWindows = 0;
    std::atomic<int> inside{0};
    std::atomic<bool> overlap{false};
    uint64_t execute(Tuple *t, bool left, uint64_t, Sink &) override {
        if (inside.fetch_add(1) != 0) overlap = true;
        const int me = left ? 0 : 1;
        uint64_t m = 0;
        for (uint64_t i = 0; i < batch; i++) {
            auto it = side[1 - me].find(t[i].key);
            if (it != side[1 - me].end()) m += it->second;
        }
        for (uint64_t i = 0; i < batch; i++) side[me][t[i].key]++;
        open += m;
        std::this_thread::yield();   // widen the window for another thread to slip in
        inside.fetch_sub(1);
        return m;
    }
    void clearStates() override {
        if (inside.load() != 0) overlap = true;
        closedTotal += open;
        closedWindows++;
        open = 0;
        side[0].clear();
        side[1].clear();
    }
    void onEndOfStream() override {}
};

int eager_mode() {
    const uint64_t B = 64, W = 1024, nb = 600;
    std::vector<Tuple> left(nb * B), right(nb * B);
    uint64_t x = 88172645463325252ull;
    for (uint64_t i = 0; i < nb * B; i++) {
        x ^= x << 13, x ^= x >> 7, x ^= x << 17;
        left[i] = Tuple{(uint32_t)(x % 97), (uint32_t)i, i};
        x ^= x << 13, x ^= x >> 7, x ^= x << 17;
        right[i] = Tuple{(uint32_t)(x % 97), (uint32_t)i, i};
    }
    Sink sink;
    auto ex = std::make_shared<CpuEager>(B);
    auto win = std::make_shared<Windowing::Eager::CountBased>(sink, W, B, ex, "cpu_eager");
    Source src(nb * B, B);
    src.start(left.data(), right.data(), 8, win);
    std::printf("overlap=%d\nmatch_count=%lu\nwindow_total=%lu\nwindows_closed=%lu\nsink_windows=%lu\n",
                ex->overlap.load() ? 1 : 0, (unsigned long)sink.getMatchCount(),
                (unsigned long)(ex->closedTotal + ex->open), (unsigned long)ex->closedWindows,
                (unsigned long)sink.getExecutedWindows());
    return 0;
}

}  // namespace

int main(int argc, char **argv) {
    const std::string mode = argc > 1 ? argv[1] : "";
    if (mode == "ring") return ring_mode();
    if (mode == "eager") return eager_mode();
    std::fprintf(stderr, "usage: host_units ring|eager\n");
    return 2;
}
