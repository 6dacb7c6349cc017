// sjb_host.cpp - the reference's windowing, sink, source and factory over the
// GPU joiners of libsjbg.  See sjb_host.hpp for the reference file of each class.
#include "sjb_host.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstdio>
#include <cctype>
#include <condition_variable>
#include <fstream>
#include <sstream>
#include <thread>

#include <dlfcn.h>

namespace {

[[noreturn]] void throw_sjbg(sjbg_handle *h, int rc, const char *what) {
    std::ostringstream m;
    m << what << " failed (status " << rc << "): " << sjbg_last_error(h);
    throw std::runtime_error(m.str());
}

sjbg_handle *create_handle(const sjbg_config &cfg) {
    sjbg_handle *h = nullptr;
    const int rc = sjbg_create(&cfg, &h);
    if (rc != SJBG_OK) throw_sjbg(nullptr, rc, "sjbg_create");
    return h;
}

// Pair buffer of the GPU executors when the result mode writes pairs: as many
// pairs as the reference's sink buffer holds result tuples
// (include/sjb/sink/Sink.h:14-16, 1 RT_GiB = 32 * 1024 * 1014).
constexpr uint64_t kSinkPairs = 32ull * 1024 * 1014;

// A bounded pool of joiners: the reference's tbb::concurrent_queue of executors
// with a busy-wait pop (CountBased.cuh:128-132), here with a condition variable.
class JoinerPool {
public:
    explicit JoinerPool(std::vector<std::shared_ptr<Windowing::Lazy::Executor::BaseLazyExecutor>> js)
        : free(std::move(js)) {}
    std::shared_ptr<Windowing::Lazy::Executor::BaseLazyExecutor> pop() {
        std::unique_lock<std::mutex> g(mu);
        cv.wait(g, [&] { return !free.empty(); });
        auto j = free.back();
        free.pop_back();
        return j;
    }
    void push(std::shared_ptr<Windowing::Lazy::Executor::BaseLazyExecutor> j) {
        {
            std::lock_guard<std::mutex> g(mu);
            free.push_back(std::move(j));
        }
        cv.notify_one();
    }

private:
    std::mutex mu;
    std::condition_variable cv;
    std::vector<std::shared_ptr<Windowing::Lazy::Executor::BaseLazyExecutor>> free;
};

}  // namespace

// ---- Sink (src/sjb/sink/Sink.cpp:13-23) ----
void Sink::addToCounter(uint64_t m, bool closed) {
    const uint64_t now = counter.fetch_add(m) + m;
    const auto us = std::chrono::duration_cast<std::chrono::microseconds>(
                        std::chrono::high_resolution_clock::now() - start)
                        .count();
    std::lock_guard<std::mutex> g(mu);
    progress.push_back(Progress{now, closed, (uint64_t)us});
}

namespace Windowing {
namespace Lazy {
namespace Executor {

GPUJoinLazyExecutor::GPUJoinLazyExecutor(const sjbg_config &cfg) : h(create_handle(cfg)) {
    if (cfg.result_mode != SJBG_RESULT_NO_OUTPUT) {
        pairs.reset(new sjbg_pair[kSinkPairs]);
        pairsCapacity = kSinkPairs;
    }
}

GPUJoinLazyExecutor::~GPUJoinLazyExecutor() { sjbg_destroy(h); }

ExecutionStatistic GPUJoinLazyExecutor::execute(Tuple *leftRingBuffer, Tuple *rightRingBuffer,
                                                std::vector<uint64_t> leftIndexesToJoin,
                                                std::vector<uint64_t> rightIndexesToJoin, Sink &sink) {
    sjbg_window_result r{};
    const int rc = sjbg_lazy_execute_ring(
        h, reinterpret_cast<const sjbg_tuple *>(leftRingBuffer), leftIndexesToJoin.data(), leftIndexesToJoin.size(),
        reinterpret_cast<const sjbg_tuple *>(rightRingBuffer), rightIndexesToJoin.data(), rightIndexesToJoin.size(),
        pairs.get(), pairsCapacity, &r);
    if (rc != SJBG_OK) throw_sjbg(h, rc, "sjbg_lazy_execute_ring");
    sink.addChecksums(r.xor_checksum, r.prod_checksum);
    ExecutionStatistic st;
    st.resultCount = r.count;
    // The GPU joins are not split into build/probe or sort/merge phases: the
    // device time of the whole window is reported as probe time (microseconds).
    st.probeTime = (uint64_t)(r.ms * 1000.0f);
    return st;
}

}  // namespace Executor
}  // namespace Lazy

namespace Eager {
namespace Executor {

GPUJoinEagerExecutor::GPUJoinEagerExecutor(const sjbg_config &cfg) : h(create_handle(cfg)), batch(cfg.batch_size) {}

GPUJoinEagerExecutor::~GPUJoinEagerExecutor() { sjbg_destroy(h); }

uint64_t GPUJoinEagerExecutor::execute(Tuple *tupleBuffer, bool isLeftSide, uint64_t, Sink &) {
    uint64_t m = 0;
    std::lock_guard<std::mutex> g(mu);
    const int rc = sjbg_eager_execute(h, reinterpret_cast<const sjbg_tuple *>(tupleBuffer), batch, isLeftSide ? 1 : 0,
                                      SJBG_MEM_HOST, &m);
    if (rc != SJBG_OK) throw_sjbg(h, rc, "sjbg_eager_execute");
    return m;
}

sjbg_window_result GPUJoinEagerExecutor::windowResult() {
    sjbg_window_result r{};
    std::lock_guard<std::mutex> g(mu);
    const int rc = sjbg_eager_window_result(h, nullptr, 0, &r);
    if (rc != SJBG_OK) throw_sjbg(h, rc, "sjbg_eager_window_result");
    return r;
}

void GPUJoinEagerExecutor::clearStates() {
    std::lock_guard<std::mutex> g(mu);
    const int rc = sjbg_eager_clear_states(h);
    if (rc != SJBG_OK) throw_sjbg(h, rc, "sjbg_eager_clear_states");
}

void GPUJoinEagerExecutor::onEndOfStream() {
    std::lock_guard<std::mutex> g(mu);
    const int rc = sjbg_eager_end_of_stream(h);
    if (rc != SJBG_OK) throw_sjbg(h, rc, "sjbg_eager_end_of_stream");
}

}  // namespace Executor
}  // namespace Eager

// ---- Lazy::CountBased (include/sjb/windowing/lazy/CountBased.cuh:22-166) ----
namespace Lazy {

struct CountBased::Impl {
    explicit Impl(std::vector<std::shared_ptr<Executor::BaseLazyExecutor>> js) : pool(std::move(js)) {}
    JoinerPool pool;
};

CountBased::CountBased(Sink &sink, uint64_t ringBufferSize, uint64_t ringBufferMaxTries, uint64_t windowSize,
                       uint64_t batchSize, std::vector<std::shared_ptr<Executor::BaseLazyExecutor>> joiners,
                       std::string name)
    : BaseWindowing(sink, std::move(name)), ringBufferSize(ringBufferSize), ringBufferMaxTries(ringBufferMaxTries),
      windowSize(windowSize), batchSize(batchSize), impl(new Impl(std::move(joiners))) {
    if (batchSize == 0 || windowSize < batchSize || ringBufferSize < windowSize)
        throw std::invalid_argument("CountBased: need 0 < batchSize <= windowSize <= ringBufferSize");
    for (uint64_t i = 0; i < ringBufferSize / batchSize; i++) {
        available[0].push_back(i * batchSize);
        available[1].push_back(i * batchSize);
    }
    // Pinned, as the reference's ring (include/sjb/windowing/lazy/CountBased.cuh:35-36), so the
    // joiners' host-to-device copies of a window's batches run at the link's rate.  Without a
    // CUDA device (executors that are not GPU joiners) the ring is plain host memory.
    void *p0 = nullptr, *p1 = nullptr;
    ringPinned = cudaMallocHost(&p0, sizeof(Tuple) * ringBufferSize) == cudaSuccess &&
                 cudaMallocHost(&p1, sizeof(Tuple) * ringBufferSize) == cudaSuccess;
    if (!ringPinned) {
        cudaGetLastError();
        if (p0) cudaFreeHost(p0);
        p0 = std::malloc(sizeof(Tuple) * ringBufferSize);
        p1 = std::malloc(sizeof(Tuple) * ringBufferSize);
        if (!p0 || !p1) {
            std::free(p0);
            std::free(p1);
            throw std::runtime_error("CountBased: the ring buffer could not be allocated");
        }
    }
    ring[0] = static_cast<Tuple *>(p0);
    ring[1] = static_cast<Tuple *>(p1);
}

CountBased::~CountBased() {
    for (Tuple *r : ring) {
        if (!r) continue;
        if (ringPinned) cudaFreeHost(r);
        else std::free(r);
    }
}

void CountBased::incoming(Tuple *batch, int side) {
    uint64_t slot = 0;
    for (uint64_t trial = 0;; trial++) {
        {
            std::lock_guard<std::mutex> g(mu);
            if (!available[side].empty()) {
                slot = available[side].front();
                available[side].pop_front();
                break;
            }
        }
        // The reference exits the process here ("Ring buffer is full").
        if (trial > ringBufferMaxTries) throw std::runtime_error("Ring buffer is full");
        std::this_thread::sleep_for(std::chrono::microseconds(1));
    }
    std::copy(batch, batch + batchSize, ring[side] + slot);
    {
        std::lock_guard<std::mutex> g(mu);
        executable[side].push_back(slot);
    }
    execute();
}

void CountBased::execute() {
    const uint64_t per = windowSize / batchSize;
    std::vector<uint64_t> li, ri;
    {
        std::lock_guard<std::mutex> g(mu);
        if (executable[0].size() * batchSize >= windowSize && executable[1].size() * batchSize >= windowSize) {
            for (uint64_t i = 0; i < per; i++) {
                li.push_back(executable[0].front());
                executable[0].pop_front();
                ri.push_back(executable[1].front());
                executable[1].pop_front();
            }
        }
    }
    if (li.empty()) return;
    auto joiner = impl->pool.pop();
    ExecutionStatistic st;
    try {
        st = joiner->execute(ring[0], ring[1], li, ri, sink);
    } catch (...) {
        impl->pool.push(joiner);
        throw;
    }
    sink.addToPossibleMatches(batchSize * li.size() * batchSize * ri.size());
    sink.addToCounter(st.resultCount, true);
    sink.addToStatistics(st);
    sink.addToExecutedWindows(1);
    {
        std::lock_guard<std::mutex> g(mu);
        for (uint64_t i = 0; i < per; i++) {
            available[0].push_back(li[i]);
            available[1].push_back(ri[i]);
        }
    }
    impl->pool.push(joiner);
}

// ---- Lazy::DeviceRing ----
DeviceRing::DeviceRing(Sink &sink, uint64_t windowSize, uint64_t batchSize, uint32_t depth, const sjbg_config &cfg,
                       std::string name)
    : BaseWindowing(sink, std::move(name)), h(create_handle(cfg)), windowSize(windowSize), batchSize(batchSize) {
    const int rc = sjbg_ring_open(h, windowSize, depth);
    if (rc != SJBG_OK) {
        std::string msg = sjbg_last_error(h);
        sjbg_destroy(h);
        throw std::runtime_error("sjbg_ring_open failed: " + msg);
    }
}

DeviceRing::~DeviceRing() { sjbg_destroy(h); }

void DeviceRing::drain() {
    sjbg_stream_window res[64];
    uint32_t n = 0;
    do {
        const int rc = sjbg_ring_poll(h, res, 64, &n);
        if (rc != SJBG_OK) throw_sjbg(h, rc, "sjbg_ring_poll");
        for (uint32_t i = 0; i < n; i++) {
            const sjbg_window_result &r = res[i].result;
            if (r.status != SJBG_OK) throw_sjbg(h, (int)r.status, "ring window join");
            sink.addChecksums(r.xor_checksum, r.prod_checksum);
            sink.addToPossibleMatches(res[i].n_left * res[i].n_right);
            sink.addToCounter(r.count, true);
            ExecutionStatistic st;
            st.resultCount = r.count;
            st.probeTime = (uint64_t)(r.ms * 1000.0f);   // device time of the window's join, microseconds
            sink.addToStatistics(st);
            sink.addToExecutedWindows(1);
        }
    } while (n == 64);
}

void DeviceRing::push(Tuple *batch, bool left) {
    std::lock_guard<std::mutex> g(mu);
    const int rc = sjbg_ring_push(h, reinterpret_cast<const sjbg_tuple *>(batch), batchSize, left ? 1 : 0,
                                  SJBG_MEM_HOST);
    // the reference exits the process here ("Ring buffer is full")
    if (rc == SJBG_E_CAPACITY) throw std::runtime_error("Ring buffer is full");
    if (rc != SJBG_OK) throw_sjbg(h, rc, "sjbg_ring_push");
    drain();
}

void DeviceRing::onEndOfStream() {
    std::lock_guard<std::mutex> g(mu);
    if (closed) return;
    closed = true;
    const int rc = sjbg_ring_close(h, nullptr);
    if (rc != SJBG_OK) throw_sjbg(h, rc, "sjbg_ring_close");
    drain();
}

}  // namespace Lazy

// ---- Eager::CountBased (include/sjb/windowing/eager/CountBased.cuh:36-72) ----
namespace Eager {

void CountBased::closeWindowIfFull(bool &closed) {
    if (total[0] >= windowSize || total[1] >= windowSize) {
        harvestChecksums();
        joiner->clearStates();
        total[0] = total[1] = 0;
        sink.addToExecutedWindows(1);
        closed = true;
    }
}

void CountBased::harvestChecksums() {
    if (auto *gpu = dynamic_cast<Executor::GPUJoinEagerExecutor *>(joiner.get())) {
        const sjbg_window_result r = gpu->windowResult();
        sink.addChecksums(r.xor_checksum, r.prod_checksum);
        sink.addWindowPairs(r.count);
    }
}

void CountBased::incoming(Tuple *batch, bool left) {
    std::lock_guard<std::mutex> g(mu);
    bool closed = false;
    closeWindowIfFull(closed);
    const int me = left ? 0 : 1;
    const uint64_t m = joiner->execute(batch, left, total[me], sink);
    total[me] += batchSize;
    sink.addToCounter(m, closed);
    sink.addToPossibleMatches(batchSize * total[1 - me]);
}

void CountBased::onEndOfStream() {
    {
        std::lock_guard<std::mutex> g(mu);
        harvestChecksums();
    }
    joiner->onEndOfStream();
}

}  // namespace Eager

// ---- WindowingFactory (src/sjb/windowing/WindowingFactory.cpp:52-298) ----
namespace {

// GPU executors share one device each: at most this many lazy joiners (each a
// handle with its own CUDA stream and window buffers) are created, whatever
// joinerThreads asks for.
constexpr uint64_t kMaxGpuJoiners = 8;

const char *result_suffix(uint8_t m) {
    switch (m) {
    case RESULT_WRITING_METHOD::NoOutput: return "nm";
    case RESULT_WRITING_METHOD::CountKernel: return "ck";
    case RESULT_WRITING_METHOD::EstimatedSelectivity: return "es";
    case RESULT_WRITING_METHOD::Bitmap: return "bm";
    case RESULT_WRITING_METHOD::Atomic: return "at";
    default: return nullptr;
    }
}

const char *alg_name(uint8_t a) {
    switch (a) {
    case ALGORITHM_TYPE::NLJ: return "nlj";
    case ALGORITHM_TYPE::HJ: return "hj";
    case ALGORITHM_TYPE::SMJ: return "smj";
    default: return nullptr;
    }
}

}  // namespace

std::string WindowingFactory::algorithmName(const AlgorithmConfig &a) {
    if (a.device != DEVICE_TYPE::GPU) throw std::runtime_error("Not Implemented");
    const char *alg = alg_name(a.underlyingAlgorithm);
    const char *res = result_suffix(a.resultWritingMethod);
    if (!alg || !res) throw std::runtime_error("Not Implemented");
    // Bitmap materialisation exists for the nested-loop join only, as in the reference.
    if (a.resultWritingMethod == RESULT_WRITING_METHOD::Bitmap && a.underlyingAlgorithm != ALGORITHM_TYPE::NLJ)
        throw std::runtime_error("Not Implemented");
    std::string name = a.progressiveness == PROGRESSIVENESS_TYPE::LAZY ? "lazy_gpu_" : "eager_gpu_";
    // eager joiners as one persistent kernel (the reference's usePK; its GPU_HJ_PK has no factory name)
    const bool pk = a.progressiveness == PROGRESSIVENESS_TYPE::EAGER && a.eagerJoinConfig.usePK;
    return name + alg + (pk ? "_pk_" : "_") + res;
}

sjbg_config WindowingFactory::toConfig(const AlgorithmConfig &a, const DataConfig &d, const QueryConfig &q,
                                       const EngineConfig &e) {
    sjbg_config c{};
    c.algorithm = a.underlyingAlgorithm;
    c.progressiveness = a.progressiveness;
    c.result_mode = a.resultWritingMethod;
    c.partitioner = SJBG_PART_AUTO;
    c.batch_size = d.batchSize;
    c.max_tuples_per_window = std::max<uint64_t>(e.maxTupleInWindow, q.windowSize);
    c.window_size = q.windowSize;
    c.num_distinct_keys = d.numDistinctKey;
    c.device = e.gpuDevice;
    // the reference's EagerJoinConfig::usePK (persistent kernels) for eager executors
    if (a.progressiveness == Windowing::EAGER && a.eagerJoinConfig.usePK) c.flags |= SJBG_F_PERSISTENT;
    return c;
}

std::shared_ptr<BaseWindowing> WindowingFactory::create(AlgorithmConfig algorithmConfig, DataConfig dataConfig,
                                                        QueryConfig queryConfig, EngineConfig engineConfig,
                                                        Sink &sink) {
    const std::string name = algorithmName(algorithmConfig);
    const sjbg_config cfg = toConfig(algorithmConfig, dataConfig, queryConfig, engineConfig);
    if (algorithmConfig.progressiveness == PROGRESSIVENESS_TYPE::LAZY && engineConfig.deviceRing) {
        // the ring's joins report counts and checksums, no pairs
        if (algorithmConfig.resultWritingMethod != RESULT_WRITING_METHOD::NoOutput)
            throw std::runtime_error("Not Implemented");
        const uint64_t slots = queryConfig.windowSize ? engineConfig.ringBufferSize / queryConfig.windowSize : 0;
        const uint32_t depth = (uint32_t)std::min<uint64_t>(64, std::max<uint64_t>(2, slots));
        return std::make_shared<Lazy::DeviceRing>(sink, queryConfig.windowSize, dataConfig.batchSize, depth, cfg,
                                                  name + "_ring");
    }
    if (algorithmConfig.progressiveness == PROGRESSIVENESS_TYPE::LAZY) {
        std::vector<std::shared_ptr<Lazy::Executor::BaseLazyExecutor>> joiners;
        const uint64_t n = std::max<uint64_t>(1, std::min(engineConfig.joinerThreads, kMaxGpuJoiners));
        for (uint64_t i = 0; i < n; i++) joiners.push_back(std::make_shared<Lazy::Executor::GPUJoinLazyExecutor>(cfg));
        return std::make_shared<Lazy::CountBased>(sink, engineConfig.ringBufferSize, engineConfig.ringBufferMaxTries,
                                                  queryConfig.windowSize, dataConfig.batchSize, joiners, name);
    }
    auto joiner = std::make_shared<Eager::Executor::GPUJoinEagerExecutor>(cfg);
    return std::make_shared<Eager::CountBased>(sink, queryConfig.windowSize, dataConfig.batchSize, joiner, name);
}

}  // namespace Windowing

// ---- Source (src/sjb/source/Source.cpp:13-32) ----
void Source::start(Tuple *leftTuples, Tuple *rightTuples, uint64_t sourceThreads,
                   const std::shared_ptr<Windowing::BaseWindowing> &windowing) {
    const uint64_t nb = bufferSize ? count / bufferSize : 0;
    std::atomic<uint64_t> next{0};
    std::mutex err_mu;
    std::exception_ptr err;
    auto work = [&] {
        try {
            for (;;) {
                const uint64_t i = next.fetch_add(1);
                if (i >= nb) break;
                windowing->onIncomingLeft(leftTuples + i * bufferSize);
                windowing->onIncomingRight(rightTuples + i * bufferSize);
            }
        } catch (...) {
            std::lock_guard<std::mutex> g(err_mu);
            if (!err) err = std::current_exception();
            next.store(nb);
        }
    };
    const uint64_t nt = std::max<uint64_t>(1, std::min(sourceThreads, nb));
    std::vector<std::thread> ts;
    for (uint64_t t = 1; t < nt; t++) ts.emplace_back(work);
    work();
    for (auto &t : ts) t.join();
    if (err) std::rethrow_exception(err);
    windowing->onEndOfStream();
}

// ---- PowerSampler ----
namespace {
// The few NVML entry points used, resolved from libnvidia-ml at run time.
struct Nvml {
    void *lib = nullptr;
    int (*init)() = nullptr;
    int (*shutdown)() = nullptr;
    int (*handle)(unsigned, void **) = nullptr;
    int (*handle_pci)(const char *, void **) = nullptr;
    int (*power)(void *, unsigned *) = nullptr;   // milliwatts
    bool load() {
        lib = dlopen("libnvidia-ml.so.1", RTLD_NOW | RTLD_LOCAL);
        if (!lib) return false;
        init = reinterpret_cast<int (*)()>(dlsym(lib, "nvmlInit_v2"));
        shutdown = reinterpret_cast<int (*)()>(dlsym(lib, "nvmlShutdown"));
        handle = reinterpret_cast<int (*)(unsigned, void **)>(dlsym(lib, "nvmlDeviceGetHandleByIndex_v2"));
        handle_pci = reinterpret_cast<int (*)(const char *, void **)>(dlsym(lib, "nvmlDeviceGetHandleByPciBusId_v2"));
        power = reinterpret_cast<int (*)(void *, unsigned *)>(dlsym(lib, "nvmlDeviceGetPowerUsage"));
        return init && shutdown && handle && power;
    }
};
}  // namespace

bool PowerSampler::start() {
    if (thread) return true;
    auto *nv = new Nvml();
    void *dev = nullptr;
    char bus[32] = {0};
    const bool have_bus = cudaDeviceGetPCIBusId(bus, (int)sizeof(bus), device) == cudaSuccess;
    if (!have_bus) cudaGetLastError();
    if (!nv->load() || nv->init() != 0 ||
        (have_bus && nv->handle_pci ? nv->handle_pci(bus, &dev) : nv->handle((unsigned)device, &dev)) != 0) {
        std::fprintf(stderr, "runExperiment: NVML unavailable, power is not measured\n");
        if (nv->lib) dlclose(nv->lib);
        delete nv;
        return false;
    }
    run = true;
    n = 0;
    thread = new std::thread([this, nv, dev] {
        FILE *fp = std::fopen(path.c_str(), "a");
        while (run) {
            unsigned mw = 0;
            if (fp && nv->power(dev, &mw) == 0) {
                const long long ms = std::chrono::duration_cast<std::chrono::milliseconds>(
                                         std::chrono::system_clock::now().time_since_epoch())
                                         .count();
                std::fprintf(fp, "%lld,%.3f\n", ms, mw / 1000.0);
                n++;
            }
            std::this_thread::sleep_for(std::chrono::milliseconds(period_ms));
        }
        if (fp) std::fclose(fp);
        nv->shutdown();
        dlclose(nv->lib);
        delete nv;
    });
    return true;
}

void PowerSampler::end() {
    if (!thread) return;
    run = false;
    auto *t = static_cast<std::thread *>(thread);
    t->join();
    delete t;
    thread = nullptr;
}

// ---- YamlLite ----
namespace {

std::string trim(const std::string &s) {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) a++;
    while (b > a && std::isspace((unsigned char)s[b - 1])) b--;
    return s.substr(a, b - a);
}

std::string strip_comment(const std::string &line) {
    char quote = 0;
    for (size_t i = 0; i < line.size(); i++) {
        const char c = line[i];
        if (quote) {
            if (c == quote) quote = 0;
        } else if (c == '"' || c == '\'') {
            quote = c;
        } else if (c == '#') {
            return line.substr(0, i);
        }
    }
    if (quote) throw std::invalid_argument("YAML: unterminated quote in: " + line);
    return line;
}

std::string unquote(const std::string &s) {
    const std::string t = trim(s);
    if (t.size() >= 2 && (t.front() == '"' || t.front() == '\'') && t.back() == t.front())
        return t.substr(1, t.size() - 2);
    return t;
}

}  // namespace

YamlLite YamlLite::parse(const std::string &text) {
    YamlLite y;
    std::istringstream in(text);
    std::string raw;
    int lineno = 0;
    while (std::getline(in, raw)) {
        lineno++;
        const std::string line = trim(strip_comment(raw));
        if (line.empty() || line == "---") continue;
        const size_t colon = line.find(':');
        if (colon == std::string::npos || colon == 0)
            throw std::invalid_argument("YAML line " + std::to_string(lineno) + ": expected `key: value`");
        const std::string key = trim(line.substr(0, colon));
        const std::string rest = trim(line.substr(colon + 1));
        std::vector<std::string> vals;
        if (!rest.empty() && rest.front() == '[') {
            if (rest.back() != ']')
                throw std::invalid_argument("YAML line " + std::to_string(lineno) + ": unterminated list");
            const std::string body = rest.substr(1, rest.size() - 2);
            std::string cur;
            char quote = 0;
            for (char c : body) {
                if (quote) {
                    if (c == quote) quote = 0;
                    cur += c;
                } else if (c == '"' || c == '\'') {
                    quote = c;
                    cur += c;
                } else if (c == ',') {
                    vals.push_back(unquote(cur));
                    cur.clear();
                } else {
                    cur += c;
                }
            }
            if (!trim(cur).empty() || !vals.empty()) vals.push_back(unquote(cur));
        } else {
            vals.push_back(unquote(rest));
        }
        for (auto &e : y.entries)
            if (e.first == key) throw std::invalid_argument("YAML: duplicate key " + key);
        y.entries.emplace_back(key, vals);
    }
    return y;
}

YamlLite YamlLite::load(const std::string &path) {
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    return parse(ss.str());
}

bool YamlLite::has(const std::string &key) const {
    for (auto &e : entries)
        if (e.first == key) return true;
    return false;
}

std::vector<std::string> YamlLite::list(const std::string &key) const {
    for (auto &e : entries)
        if (e.first == key) return e.second;
    throw std::invalid_argument("YAML: missing key " + key);
}

std::string YamlLite::scalar(const std::string &key) const {
    const auto v = list(key);
    if (v.size() != 1) throw std::invalid_argument("YAML: key " + key + " is not a scalar");
    return v[0];
}
