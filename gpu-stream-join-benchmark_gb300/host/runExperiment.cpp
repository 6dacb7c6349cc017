// runExperiment - the reference's experiment driver over the GPU joiners:
//   ./runExperiment <path_to_yaml_config> <outputFileName> [--list]
// Reads the same YAML keys (executable/runExperiment.cpp:40-160), expands the
// same cross product of configurations, and runs them as Runner does
// (src/experiment/Runner.cpp): generate both streams into pinned host memory,
// feed them batch by batch through the windowing, and append the same CSV
// lines ("Throughput": the sustainable-rate search; "cumulativePercentage":
// the progress records, written to progressiveness.csv).
//
// Optional keys with no reference counterpart: dataSize (tuples per stream,
// default 2560 MiB of tuples), sourceThreads (default 32), tsUpperBound
// (default 1000), gpuDevice (CUDA device of the joiners and of the power
// sampler, default 0), usePK ("Yes" / "No", default "No": the reference's
// EagerJoinConfig::usePK, include/experiment/Config.hpp:15 - eager joiners
// run as one persistent kernel fed by a queue), deviceRing ("Yes" / "No",
// default "No": lazy windows over the device-resident ingest ring instead of
// the pinned host ring; NoOutput only).  --list prints the expanded configurations and their
// algorithm names without touching a GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <limits>
#include <sstream>
#include <thread>

#include "sjb_host.hpp"

#define KiB (1024 / sizeof(Tuple))
#define MiB (KiB * 1024)

namespace {

enum TS_MODE : uint8_t { STEADY = 0, BURST = 1 };

struct ExperimentConfig {
    DataConfig dataConfig;
    AlgorithmConfig algorithmConfig;
    QueryConfig queryConfig;
    EngineConfig engineConfig;
    uint64_t precision;
    uint64_t repeat;
    bool measurePower = false;
    uint64_t sourceThreads = 32;
};

#define LOG_INFO(...)                       \
    do {                                    \
        std::printf("[INFO] " __VA_ARGS__); \
        std::printf("\n");                  \
        std::fflush(stdout);                \
    } while (0)

void cuda_ok(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

// Both streams of one configuration in pinned host memory.  Keys come from the
// library's device generator (uniform over numDistinctKey when zipfTheta is 0,
// else Zipf(zipfTheta) ranks through a seeded permutation), seeds 123 and 456
// as in the reference (Runner.cpp:20-33); val = key and the STEADY timestamps
// floor(i / floor(count / tsUpperBound)) follow DataGenerator.cpp:14-72.
void generate(Tuple *out, uint64_t count, float theta, uint64_t distinct, uint64_t seed, uint64_t tsUpper) {
    sjbg_config gc{};
    gc.algorithm = SJBG_ALG_HJ;
    gc.progressiveness = SJBG_LAZY;
    gc.max_tuples_per_window = 1;
    sjbg_handle *h = nullptr;
    if (sjbg_create(&gc, &h) != SJBG_OK) throw std::runtime_error(std::string("sjbg_create: ") + sjbg_last_error(nullptr));
    const uint64_t chunk = std::min<uint64_t>(count, 1ull << 26);
    sjbg_tuple *d = nullptr;
    uint64_t *dtab = nullptr;
    try {
        cuda_ok(cudaMalloc(&d, std::max<uint64_t>(chunk, 1) * sizeof(sjbg_tuple)), "cudaMalloc");
        if (theta > 0.0f) {
            std::vector<uint64_t> tab(distinct);
            if (sjbg_zipf_table(tab.data(), distinct, theta) != SJBG_OK) throw std::runtime_error("sjbg_zipf_table");
            cuda_ok(cudaMalloc(&dtab, distinct * sizeof(uint64_t)), "cudaMalloc");
            cuda_ok(cudaMemcpy(dtab, tab.data(), distinct * sizeof(uint64_t), cudaMemcpyHostToDevice), "cudaMemcpy");
        }
        for (uint64_t first = 0; first < count; first += chunk) {
            const uint64_t n = std::min(chunk, count - first);
            const int rc = sjbg_generate(h, d, first, n, seed, distinct, dtab, 3);
            if (rc != SJBG_OK) throw std::runtime_error(std::string("sjbg_generate: ") + sjbg_last_error(h));
            cuda_ok(cudaMemcpy(out + first, d, n * sizeof(sjbg_tuple), cudaMemcpyDeviceToHost), "cudaMemcpy");
        }
    } catch (...) {
        cudaFree(d);
        cudaFree(dtab);
        sjbg_destroy(h);
        throw;
    }
    cudaFree(d);
    cudaFree(dtab);
    sjbg_destroy(h);
    if (count <= tsUpper) throw std::invalid_argument("dataSize must exceed the timestamp upper bound");
    const uint64_t perMs = (uint64_t)std::floor((double)count / (double)tsUpper);
    const unsigned nt = std::max(1u, std::thread::hardware_concurrency());
    std::vector<std::thread> ts;
    for (unsigned t = 0; t < nt; t++)
        ts.emplace_back([=] {
            for (uint64_t i = count * t / nt; i < count * (t + 1) / nt; i++) {
                out[i].val = out[i].key;
                out[i].ts = (uint64_t)std::floor(1.0 * i / perMs);
            }
        });
    for (auto &t : ts) t.join();
}

std::pair<std::string, uint64_t> runExperimentWithConfig(const ExperimentConfig &config, bool trackProgress) {
    const uint64_t n = config.dataConfig.dataSize;
    Tuple *left = nullptr, *right = nullptr;
    cuda_ok(cudaMallocHost(&left, sizeof(Tuple) * n), "cudaMallocHost");
    cuda_ok(cudaMallocHost(&right, sizeof(Tuple) * n), "cudaMallocHost");
    std::ostringstream result;
    uint64_t msElapsed = 0;
    try {
        generate(left, n, config.dataConfig.zipfTheta, config.dataConfig.numDistinctKey, 123,
                 config.dataConfig.timestampUpperBound);
        generate(right, n, config.dataConfig.zipfTheta, config.dataConfig.numDistinctKey, 456,
                 config.dataConfig.timestampUpperBound);
        Source source(n, config.dataConfig.batchSize);
        Sink sink;
        auto windowing = Windowing::WindowingFactory::create(config.algorithmConfig, config.dataConfig,
                                                             config.queryConfig, config.engineConfig, sink);
        PowerSampler power("power_data.txt", 10, config.engineConfig.gpuDevice);   // as the reference writes it
        if (config.measurePower) power.start();
        auto t0 = std::chrono::high_resolution_clock::now();
        sink.markProcessingStart();
        source.start(left, right, config.sourceThreads, windowing);
        auto t1 = std::chrono::high_resolution_clock::now();
        power.end();
        if (config.measurePower) LOG_INFO("Power samples: %u (power_data.txt)", power.samples());
        msElapsed = std::chrono::duration_cast<std::chrono::milliseconds>(t1 - t0).count();
        const uint64_t matchCount = sink.getMatchCount();
        const double selectivity = 100.0 * matchCount / std::max<uint64_t>(1, sink.getPossibleMatches());
        LOG_INFO("Joiner: %s, Match Count: %lu, Selectivity: %.6f%%, ElapsedTime: %lu ms",
                 windowing->getAlgorithmName().c_str(), (unsigned long)matchCount, selectivity,
                 (unsigned long)msElapsed);
        LOG_INFO("Windows: %lu, Prod checksum: %lu, Window pairs: %lu", (unsigned long)sink.getExecutedWindows(),
                 (unsigned long)sink.prodChecksum, (unsigned long)sink.getWindowPairs());
        LOG_INFO("Avg Build: %lu, Avg Probe: %lu", (unsigned long)sink.getAverageBuildTime(),
                 (unsigned long)sink.getAverageProbeTime());
        LOG_INFO("Avg Sort: %lu, Avg Merge: %lu", (unsigned long)sink.getAverageSortTime(),
                 (unsigned long)sink.getAverageMergeTime());
        if (trackProgress) {
            for (const auto &p : sink.getProgress())
                result << windowing->getAlgorithmName() << "," << config.dataConfig.batchSize << "," << selectivity
                       << "," << p.isWindowClosed << "," << p.currentMatches << "," << p.timestamp << "\n";
        } else {
            result << windowing->getAlgorithmName() << "," << std::to_string(config.algorithmConfig.resultWritingMethod)
                   << "," << config.dataConfig.dataSize << "," << config.dataConfig.batchSize << ","
                   << config.dataConfig.zipfTheta << "," << config.dataConfig.numDistinctKey << ","
                   << config.queryConfig.windowSize << "," << config.algorithmConfig.cpuhjConfig.nProheThreads << ","
                   << config.engineConfig.joinerThreads << "," << selectivity << "," << msElapsed << "\n";
        }
    } catch (...) {
        cudaFreeHost(left);
        cudaFreeHost(right);
        throw;
    }
    cudaFreeHost(left);
    cudaFreeHost(right);
    return {result.str(), msElapsed};
}

double computeMedian(std::vector<uint64_t> v) {
    std::sort(v.begin(), v.end());
    if (v.size() % 2 == 0) return (v[v.size() / 2 - 1] + v[v.size() / 2]) / 2;
    return v[v.size() / 2];
}

// Sustainable-rate search of Runner::runExperimentsAndWriteResultToFile
// (src/experiment/Runner.cpp:101-188): grow or bisect dataSize until one
// configuration takes about one second.
void runThroughput(std::vector<ExperimentConfig> configs, const std::string &outputFileName) {
    std::ofstream out(outputFileName, std::ios_base::app);
    if (out.tellp() == 0)
        out << "algorithm_name,write_result,ingestion_rate,batch_size,zipf_theta,distinct_key,window_size,"
               "probe_threads,joiner_threads,selectivity,time\n";
    LOG_INFO("Running a total of %lu configurations", (unsigned long)configs.size());
    for (size_t i = 0; i < configs.size(); i++) {
        LOG_INFO("Running configuration %lu of %lu..", (unsigned long)i + 1, (unsigned long)configs.size());
        auto cur = configs[i];
        std::pair<std::string, uint64_t> result;
        uint64_t delta = std::numeric_limits<int64_t>::max();
        uint64_t latestUnsustained = 0, nextRate = cur.dataConfig.dataSize, currentRate = cur.dataConfig.dataSize;
        uint64_t latestSustained = cur.dataConfig.dataSize;
        while (delta > cur.precision) {
            std::vector<uint64_t> times;
            for (uint64_t rep = 0; rep < cur.repeat; rep++) {
                result = runExperimentWithConfig(cur, false);
                times.push_back(result.second);
            }
            const double median = computeMedian(times);
            if (median < 1000) {
                latestSustained = currentRate;
                nextRate = latestUnsustained == 0 ? nextRate * 2 : (latestUnsustained + currentRate) / 2;
            } else {
                latestUnsustained = currentRate;
                nextRate = (latestSustained + currentRate) / 2;
            }
            delta = currentRate > nextRate ? currentRate - nextRate : nextRate - currentRate;
            LOG_INFO("Latest ms elapsed: %lu dataSize: %lu delta:%lu", (unsigned long)result.second,
                     (unsigned long)cur.dataConfig.dataSize, (unsigned long)delta);
            currentRate = nextRate;
            cur.dataConfig.dataSize = currentRate;
            if (std::abs(median - 1000) <= 50) break;
        }
        out << result.first;
    }
}

// Runner::runProgressivenessExperimentAndWriteResultToFile (Runner.cpp:209-235).
void runProgress(const std::vector<ExperimentConfig> &configs, const std::string &outputFileName) {
    for (size_t i = 0; i < configs.size(); i++) {
        LOG_INFO("Running configuration %lu of %lu..", (unsigned long)i + 1, (unsigned long)configs.size());
        auto result = runExperimentWithConfig(configs[i], true);
        std::ofstream out(outputFileName, std::ios_base::app);
        if (out.tellp() == 0) out << "algorithm_name,batch_size,selectivity,isWindowClosed,match_count,timestamp\n";
        out << result.first;
    }
}

template <class E>
std::vector<E> parse_enum(const YamlLite &y, const char *key, const std::vector<std::pair<const char *, E>> &names,
                          const char *what) {
    std::vector<E> out;
    for (const auto &s : y.list(key)) {
        bool found = false;
        for (const auto &n : names)
            if (s == n.first) {
                out.push_back(n.second);
                found = true;
            }
        if (!found) throw std::invalid_argument(std::string("Unknown ") + what + ": " + s);
    }
    return out;
}

std::vector<uint64_t> parse_u64(const YamlLite &y, const char *key) {
    std::vector<uint64_t> out;
    for (const auto &s : y.list(key)) {
        size_t pos = 0;
        const unsigned long long v = std::stoull(s, &pos);
        if (pos != s.size()) throw std::invalid_argument(std::string("not an integer in ") + key + ": " + s);
        out.push_back(v);
    }
    return out;
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 3) {
        std::cout << "Please run using ./runExperiment <path_to_yaml_config> <outputFileName>." << std::endl;
        return 1;
    }
    const bool listOnly = argc > 3 && std::strcmp(argv[3], "--list") == 0;
    try {
        // DEFAULT PARAMETERS (executable/runExperiment.cpp:23-38)
        ExperimentConfig ec;
        ec.dataConfig = {2560 * MiB, 0.0f, STEADY, 128 * KiB, 1000, 1000};
        ec.algorithmConfig = {Windowing::HJ, Windowing::CPU, Windowing::EAGER, Windowing::NoOutput, {}, {}, {}};
        ec.algorithmConfig.cpuhjConfig.nProheThreads = 1;
        ec.algorithmConfig.cpusmjConfig.nSortThreads = 1;
        ec.engineConfig = {1024 * MiB, 128, 1, 32, 32 * MiB};
        ec.queryConfig = {1 * MiB};
        ec.precision = 32 * KiB;

        const YamlLite y = YamlLite::load(argv[1]);
        using namespace Windowing;
        const auto parStrats = parse_enum<PARALLELIZATION_STRATEGY>(
            y, "parStrats", {{"INTRA", INTRA}, {"INTER", INTER}, {"HYBRID", HYBRID}}, "parallelization strategy");
        const auto algTypes =
            parse_enum<ALGORITHM_TYPE>(y, "algTypes", {{"NLJ", NLJ}, {"HJ", HJ}, {"SMJ", SMJ}}, "algorithm type");
        const auto devTypes = parse_enum<DEVICE_TYPE>(y, "deviceTypes", {{"CPU", CPU}, {"GPU", GPU}}, "device type");
        const auto progModes = parse_enum<PROGRESSIVENESS_TYPE>(y, "progressivenessModes",
                                                                {{"LAZY", LAZY}, {"EAGER", EAGER}}, "progressiveness mode");
        const auto resModes = parse_enum<RESULT_WRITING_METHOD>(
            y, "resultMaterializationMethod",
            {{"NoOutput", NoOutput}, {"CountKernel", CountKernel}, {"EstimatedSelectivity", EstimatedSelectivity},
             {"Bitmap", Bitmap}, {"Atomic", Atomic}},
            "result materialization method");
        const auto distinct = parse_u64(y, "distinctKeys");
        std::vector<float> thetas;
        for (const auto &s : y.list("zipfThetas")) thetas.push_back(std::stof(s));
        auto windowSizes = parse_u64(y, "windowSizesMB");
        for (auto &w : windowSizes) w *= MiB;
        auto batchSizes = parse_u64(y, "batchSizeKB");
        for (auto &b : batchSizes) b *= KiB;
        const std::string power = y.scalar("measurePowerUsage");
        if (power == "Yes") ec.measurePower = true;
        else if (power == "No") ec.measurePower = false;
        else throw std::invalid_argument("Unknown parameter for measure power: " + power);
        ec.repeat = std::stoull(y.scalar("repeat"));
        if (y.has("dataSize")) ec.dataConfig.dataSize = std::stoull(y.scalar("dataSize"));
        if (y.has("sourceThreads")) ec.sourceThreads = std::stoull(y.scalar("sourceThreads"));
        if (y.has("tsUpperBound")) ec.dataConfig.timestampUpperBound = std::stoull(y.scalar("tsUpperBound"));
        if (y.has("gpuDevice")) ec.engineConfig.gpuDevice = std::stoi(y.scalar("gpuDevice"));
        if (y.has("deviceRing")) {
            const std::string dr = y.scalar("deviceRing");
            if (dr != "Yes" && dr != "No") throw std::invalid_argument("Unknown parameter for deviceRing: " + dr);
            ec.engineConfig.deviceRing = dr == "Yes";
        }
        if (y.has("usePK")) {
            const std::string pk = y.scalar("usePK");
            if (pk != "Yes" && pk != "No") throw std::invalid_argument("Unknown parameter for usePK: " + pk);
            ec.algorithmConfig.eagerJoinConfig.usePK = pk == "Yes";
        }
        const std::string metric = y.scalar("measuredMetric");
        if (metric != "Throughput" && metric != "cumulativePercentage")
            throw std::invalid_argument("Unknown measured metrics: " + metric);

        const uint64_t hw = std::max(1u, std::thread::hardware_concurrency());
        std::vector<ExperimentConfig> configs;
        for (auto a : algTypes)
            for (auto d : devTypes)
                for (auto p : progModes)
                    for (auto k : distinct)
                        for (auto r : resModes)
                            for (auto w : windowSizes)
                                for (auto b : batchSizes)
                                    for (auto z : thetas)
                                        for (auto s : parStrats) {
                                            ec.dataConfig.batchSize = b;
                                            ec.dataConfig.zipfTheta = z;
                                            ec.algorithmConfig.progressiveness = p;
                                            ec.algorithmConfig.device = d;
                                            ec.algorithmConfig.underlyingAlgorithm = a;
                                            ec.algorithmConfig.resultWritingMethod = r;
                                            ec.dataConfig.numDistinctKey = k;
                                            ec.queryConfig.windowSize = w;
                                            ec.engineConfig.maxTupleInWindow = w;
                                            if (s == INTRA) {
                                                ec.engineConfig.joinerThreads = 1;
                                                ec.algorithmConfig.cpuhjConfig.nProheThreads = hw;
                                                ec.algorithmConfig.cpusmjConfig.nSortThreads = hw;
                                            } else if (s == INTER) {
                                                ec.engineConfig.joinerThreads = hw;
                                                ec.algorithmConfig.cpuhjConfig.nProheThreads = 1;
                                                ec.algorithmConfig.cpusmjConfig.nSortThreads = 1;
                                            } else {
                                                ec.engineConfig.joinerThreads = 4;
                                                ec.algorithmConfig.cpuhjConfig.nProheThreads = hw / 4;
                                                ec.algorithmConfig.cpusmjConfig.nSortThreads = hw / 4;
                                            }
                                            configs.push_back(ec);
                                        }
        if (listOnly) {
            std::cout << "algorithm_name,window_size,batch_size,zipf_theta,distinct_key,joiner_threads,data_size\n";
            for (const auto &c : configs) {
                std::string name;
                try {
                    name = WindowingFactory::algorithmName(c.algorithmConfig);
                } catch (const std::exception &e) {
                    name = e.what();
                }
                std::cout << name << "," << c.queryConfig.windowSize << "," << c.dataConfig.batchSize << ","
                          << c.dataConfig.zipfTheta << "," << c.dataConfig.numDistinctKey << ","
                          << c.engineConfig.joinerThreads << "," << c.dataConfig.dataSize << "\n";
            }
            return 0;
        }
        if (metric == "Throughput") runThroughput(configs, argv[2]);
        else runProgress(configs, "progressiveness.csv");
    } catch (const std::exception &e) {
        std::cerr << "runExperiment: " << e.what() << std::endl;
        return 2;
    }
    return 0;
}
