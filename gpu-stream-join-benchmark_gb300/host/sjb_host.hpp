// sjb_host.hpp - C++ host side of the drop-in: the reference's joiner
// interfaces, windowing, sink and factory, with the GPU joiners provided by
// libsjbg.so through its C ABI (include/sjbg.h).
//
// Names, argument meaning and error behaviour mirror the reference:
//   Tuple, ExecutionStatistic       include/sjb/utils/{Tuple,ExecutionStatistic}.hpp
//   enums                           include/sjb/windowing/BaseWindowing.cuh:9-41
//   BaseLazyExecutor::execute       include/sjb/windowing/lazy/executor/BaseLazyExecutor.hpp:26-30
//   BaseEagerExecutor               include/sjb/windowing/eager/executor/BaseEagerExecutor.hpp:16-20
//   Lazy::CountBased                include/sjb/windowing/lazy/CountBased.cuh:19-196
//   Eager::CountBased               include/sjb/windowing/eager/CountBased.cuh:17-86
//   Sink                            include/sjb/sink/Sink.h:23-126
//   WindowingFactory::create        src/sjb/windowing/WindowingFactory.cpp:52-298
//   Config structs                  include/experiment/Config.hpp:6-65
// Unsupported combinations throw std::runtime_error("Not Implemented"), as the
// reference's factory does.
#pragma once

#include <atomic>
#include <chrono>
#include <cstdint>
#include <deque>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "sjbg.h"

class Tuple {
public:
    uint32_t key;
    uint32_t val;
    uint64_t ts;
};
static_assert(sizeof(Tuple) == sizeof(sjbg_tuple), "Tuple must keep the 16-byte layout");

class ExecutionStatistic {
public:
    uint64_t resultCount{};
    uint64_t buildTime{};
    uint64_t probeTime{};
    uint64_t sortTime{};
    uint64_t mergeTime{};
};

namespace Windowing {
enum ALGORITHM_TYPE : uint8_t { EMPTY = 0, NLJ = 1, HJ = 2, SMJ = 3, SABER = 4, HELLS = 5 };
enum PROGRESSIVENESS_TYPE : uint8_t { EAGER = 0, LAZY = 1 };
enum RESULT_WRITING_METHOD : uint8_t { NoOutput = 0, CountKernel = 1, EstimatedSelectivity = 2, Bitmap = 3, Atomic = 4 };
enum DEVICE_TYPE : uint8_t { CPU = 0, GPU = 1 };
enum PARALLELIZATION_STRATEGY : uint8_t { INTER = 0, INTRA = 1, HYBRID = 2 };
}  // namespace Windowing

struct Progress {
    uint64_t currentMatches;
    bool isWindowClosed;
    uint64_t timestamp;
};

// Result side of the interface: counters and progress records.
class Sink {
public:
    void addToCounter(uint64_t m, bool closed);
    void addToPossibleMatches(uint64_t c) { possible += c; }
    void addToExecutedWindows(uint64_t c) { windows += c; }
    // Matches of closed eager windows, from each window's own totals (no
    // reference counterpart): equal to getMatchCount(), the sum of the batch
    // counts, when every batch is counted into the window it joined.
    void addWindowPairs(uint64_t c) { windowPairs += c; }
    uint64_t getWindowPairs() const { return windowPairs; }
    void addChecksums(uint64_t xr, uint64_t prod) {
        std::lock_guard<std::mutex> g(mu);
        xorChecksum ^= xr;
        prodChecksum += prod;
    }
    void addToStatistics(const ExecutionStatistic &st) {
        buildTime += st.buildTime;
        probeTime += st.probeTime;
        sortTime += st.sortTime;
        mergeTime += st.mergeTime;
    }
    void markProcessingStart() { start = std::chrono::high_resolution_clock::now(); }
    uint64_t getMatchCount() const { return counter; }
    uint64_t getPossibleMatches() const { return possible; }
    uint64_t getExecutedWindows() const { return windows; }
    // Average phase times per executed window, microseconds (Sink.h:53-76).
    uint64_t getAverageBuildTime() const { return windows ? buildTime / windows : 0; }
    uint64_t getAverageProbeTime() const { return windows ? probeTime / windows : 0; }
    uint64_t getAverageSortTime() const { return windows ? sortTime / windows : 0; }
    uint64_t getAverageMergeTime() const { return windows ? mergeTime / windows : 0; }
    std::vector<Progress> getProgress() const {
        std::lock_guard<std::mutex> g(mu);
        return progress;
    }
    uint64_t xorChecksum = 0, prodChecksum = 0;

private:
    std::atomic<uint64_t> counter{0}, possible{0}, windows{0}, windowPairs{0};
    std::atomic<uint64_t> buildTime{0}, probeTime{0}, sortTime{0}, mergeTime{0};
    std::chrono::time_point<std::chrono::high_resolution_clock> start = std::chrono::high_resolution_clock::now();
    mutable std::mutex mu;
    std::vector<Progress> progress;
};

// ---- configuration (include/experiment/Config.hpp) ----
struct CPUHJConfig { uint64_t nProheThreads = 1; };
struct CPUSMJConfig { uint64_t nSortThreads = 1; };
struct EagerJoinConfig { bool usePK = false; };
struct DataConfig {
    uint64_t dataSize;
    float zipfTheta;
    uint8_t tsMode;
    uint64_t batchSize;
    uint64_t numDistinctKey;
    uint64_t timestampUpperBound = 1000;
};
struct QueryConfig { uint64_t windowSize; };
struct AlgorithmConfig {
    uint8_t underlyingAlgorithm;
    uint8_t device;
    uint8_t progressiveness;
    uint8_t resultWritingMethod = 0;
    CPUHJConfig cpuhjConfig;
    CPUSMJConfig cpusmjConfig;
    EagerJoinConfig eagerJoinConfig;
};
struct EngineConfig {
    uint64_t ringBufferSize;
    uint64_t ringBufferMaxTries;
    uint64_t joinerThreads;
    uint64_t nSourceThreads;
    uint64_t maxTupleInWindow;
    int gpuDevice = 0;   // CUDA device of the GPU joiners (no reference counterpart)
    bool deviceRing = false;   // lazy windows over the device-resident ring (no reference counterpart)
};

namespace Windowing {
namespace Lazy {
namespace Executor {
class BaseLazyExecutor {
public:
    virtual ~BaseLazyExecutor() = default;
    virtual ExecutionStatistic execute(Tuple *leftRingBuffer, Tuple *rightRingBuffer,
                                       std::vector<uint64_t> leftIndexesToJoin,
                                       std::vector<uint64_t> rightIndexesToJoin, Sink &sink) = 0;
};

// The GPU joiners of libsjbg behind the lazy interface.
class GPUJoinLazyExecutor : public BaseLazyExecutor {
public:
    GPUJoinLazyExecutor(const sjbg_config &cfg);
    ~GPUJoinLazyExecutor() override;
    ExecutionStatistic execute(Tuple *leftRingBuffer, Tuple *rightRingBuffer, std::vector<uint64_t> leftIndexesToJoin,
                               std::vector<uint64_t> rightIndexesToJoin, Sink &sink) override;

private:
    sjbg_handle *h = nullptr;
    std::unique_ptr<sjbg_pair[]> pairs;  // uninitialised; NULL when no pairs are written
    uint64_t pairsCapacity = 0;
};
}  // namespace Executor
}  // namespace Lazy

namespace Eager {
namespace Executor {
class BaseEagerExecutor {
public:
    virtual ~BaseEagerExecutor() = default;
    virtual uint64_t execute(Tuple *tupleBuffer, bool isLeftSide, uint64_t windowTupleCount, Sink &sink) = 0;
    virtual void clearStates() = 0;
    virtual void onEndOfStream() = 0;
};

class GPUJoinEagerExecutor : public BaseEagerExecutor {
public:
    GPUJoinEagerExecutor(const sjbg_config &cfg);
    ~GPUJoinEagerExecutor() override;
    uint64_t execute(Tuple *tupleBuffer, bool isLeftSide, uint64_t windowTupleCount, Sink &sink) override;
    void clearStates() override;
    void onEndOfStream() override;
    // Totals (count and checksums) of the window not yet cleared.
    sjbg_window_result windowResult();

private:
    sjbg_handle *h = nullptr;
    uint64_t batch;
    std::mutex mu;  // one handle, called from every source thread
};
}  // namespace Executor
}  // namespace Eager

// ---- windowing ----
class BaseWindowing {
public:
    BaseWindowing(Sink &sink, std::string name) : sink(sink), algorithmName(std::move(name)) {}
    virtual ~BaseWindowing() = default;
    virtual void onIncomingLeft(Tuple *tupleBuffer) = 0;
    virtual void onIncomingRight(Tuple *tupleBuffer) = 0;
    virtual void onEndOfStream() = 0;
    const std::string &getAlgorithmName() const { return algorithmName; }

protected:
    Sink &sink;
    std::string algorithmName;
};

namespace Lazy {
// Count-based tumbling windows over a ring of batch slots
// (include/sjb/windowing/lazy/CountBased.cuh:45-166).
class CountBased : public BaseWindowing {
public:
    CountBased(Sink &sink, uint64_t ringBufferSize, uint64_t ringBufferMaxTries, uint64_t windowSize,
               uint64_t batchSize, std::vector<std::shared_ptr<Executor::BaseLazyExecutor>> joiners,
               std::string name);
    ~CountBased() override;
    void onIncomingLeft(Tuple *tupleBuffer) override { incoming(tupleBuffer, 0); }
    void onIncomingRight(Tuple *tupleBuffer) override { incoming(tupleBuffer, 1); }
    void onEndOfStream() override {}

private:
    void incoming(Tuple *batch, int side);
    void execute();
    struct Impl;
    uint64_t ringBufferSize, ringBufferMaxTries, windowSize, batchSize;
    std::unique_ptr<Impl> impl;
    Tuple *ring[2] = {nullptr, nullptr};   // pinned host memory (cudaMallocHost), as the reference's
    bool ringPinned = false;               // false: no CUDA device, plain host memory
    std::deque<uint64_t> available[2], executable[2];
    std::mutex mu;
};
// Count-based tumbling windows over a device-resident ring (sjbg_ring_*, the
// optional YAML key deviceRing: "Yes"): each batch is copied into HBM as it
// arrives, and each full window is joined there, asynchronously, while the
// next one fills.  Results reach the sink as the joins finish.  The windows
// are those of CountBased above (tuples [kW, (k+1)W) of each side in arrival
// order); its pinned host ring and per-window copies are what this replaces.
class DeviceRing : public BaseWindowing {
public:
    DeviceRing(Sink &sink, uint64_t windowSize, uint64_t batchSize, uint32_t depth, const sjbg_config &cfg,
               std::string name);
    ~DeviceRing() override;
    void onIncomingLeft(Tuple *tupleBuffer) override { push(tupleBuffer, true); }
    void onIncomingRight(Tuple *tupleBuffer) override { push(tupleBuffer, false); }
    void onEndOfStream() override;

private:
    void push(Tuple *batch, bool left);
    void drain();   // finished windows into the sink (caller holds mu)
    sjbg_handle *h = nullptr;
    uint64_t windowSize, batchSize;
    bool closed = false;
    std::mutex mu;
};
}  // namespace Lazy

namespace Eager {
// Eager count-based windows (include/sjb/windowing/eager/CountBased.cuh:36-72).
class CountBased : public BaseWindowing {
public:
    CountBased(Sink &sink, uint64_t windowSize, uint64_t batchSize,
               std::shared_ptr<Executor::BaseEagerExecutor> joiner, std::string name)
        : BaseWindowing(sink, std::move(name)), windowSize(windowSize), batchSize(batchSize),
          joiner(std::move(joiner)) {}
    void onIncomingLeft(Tuple *tupleBuffer) override { incoming(tupleBuffer, true); }
    void onIncomingRight(Tuple *tupleBuffer) override { incoming(tupleBuffer, false); }
    void onEndOfStream() override;

private:
    void incoming(Tuple *batch, bool left);
    void closeWindowIfFull(bool &closed);   // caller holds mu
    void harvestChecksums();                // caller holds mu
    uint64_t windowSize, batchSize;
    // Tuples of the current window per side.  The close check, the batch's
    // execution and the update of total[] happen under mu as one step, so
    // source threads that deliver batches concurrently cannot both close a
    // window or count a batch into a window that was just closed (the
    // reference reads and writes these counters without a lock,
    // include/sjb/windowing/eager/CountBased.cuh:47-49).
    uint64_t total[2] = {0, 0};
    std::shared_ptr<Executor::BaseEagerExecutor> joiner;
    std::mutex mu;
};
}  // namespace Eager

class WindowingFactory {
public:
    static std::shared_ptr<BaseWindowing> create(AlgorithmConfig algorithmConfig, DataConfig dataConfig,
                                                 QueryConfig queryConfig, EngineConfig engineConfig, Sink &sink);
    // The reference's algorithm name of a configuration ("lazy_gpu_hj_nm", ...);
    // throws "Not Implemented" for combinations the library does not provide.
    static std::string algorithmName(const AlgorithmConfig &a);
    // The library configuration of one executor.
    static sjbg_config toConfig(const AlgorithmConfig &a, const DataConfig &d, const QueryConfig &q,
                                const EngineConfig &e);
};
}  // namespace Windowing

// Feeds batch i of the left stream, then batch i of the right stream, for every
// batch (src/sjb/source/Source.cpp:20-28), from one thread.
class Source {
public:
    Source(uint64_t count, uint64_t bufferSize) : count(count), bufferSize(bufferSize) {}
    void start(Tuple *leftTuples, Tuple *rightTuples, uint64_t sourceThreads,
               const std::shared_ptr<Windowing::BaseWindowing> &windowing);

private:
    uint64_t count, bufferSize;
};

// GPU power sampling while an experiment runs (measurePowerUsage: "Yes"),
// the role of the reference's PowerMeasurementAgent
// (src/sjb/utils/PowerMeasurementAgent.cpp:50-175): a thread reads the board
// power of the CUDA device `device` (the one the joiners run on; NVML finds it
// by its PCI bus id, so CUDA_VISIBLE_DEVICES renumbering does not matter)
// through NVML every `period_ms` and appends "epoch_ms,watts" lines to a file.
// NVML is loaded at run time; when it is missing, start() says so on stderr
// and the experiment runs unmeasured.  Read-only: no GPU setting is changed.
class PowerSampler {
public:
    explicit PowerSampler(std::string path = "power_data.txt", unsigned period_ms = 10, int device = 0)
        : path(std::move(path)), period_ms(period_ms), device(device) {}
    ~PowerSampler() { end(); }
    bool start();
    void end();
    unsigned samples() const { return n; }

private:
    std::string path;
    unsigned period_ms;
    int device;
    std::atomic<bool> run{false};
    std::atomic<unsigned> n{0};
    void *thread = nullptr;   // std::thread, kept opaque
};

// Minimal reader of the flat YAML the reference's configs use: `key: value`
// and `key: [a, "b", c]` lines with `#` comments.
class YamlLite {
public:
    static YamlLite parse(const std::string &text);
    static YamlLite load(const std::string &path);
    bool has(const std::string &key) const;
    std::vector<std::string> list(const std::string &key) const;
    std::string scalar(const std::string &key) const;

private:
    std::vector<std::pair<std::string, std::vector<std::string>>> entries;
};
