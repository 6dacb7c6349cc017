// noalloc.cu - an allocation-free entry point for callers that cannot allocate
// device memory.
//
// Some callers of this library cannot call cudaMalloc: code running inside a
// host framework that owns all device memory through its own pool (and
// forbids other allocations), or code that must not allocate once it is in a
// latency-critical steady state.  They still own their inputs and outputs.
// sjbg_lazy_hj_noalloc serves them: the lazy hash join of one window (count
// and prod checksum, radix partitioning) with every intermediate buffer carved
// out of one file-scope device array, so the call allocates nothing and
// copies nothing from the host.
//
// The array costs kNoAllocScratchBytes of device memory on every GPU that
// loads this library, until the process exits.  Its device address is looked
// up once per device (cudaGetSymbolAddress, with that device current) on the
// first call made on that device; that first call should therefore come
// before any stream capture.  All calls share the array and each call
// re-initialises what must start at zero, so calls that overlap on the GPU
// (on different streams, or from different threads) race with each other and
// must be serialised by the caller.
#include <mutex>
#include <string>

#include "runtime.h"

namespace sjbg {

// Largest window side this entry point accepts, and the scratch it needs.
constexpr uint64_t kNoAllocMaxTuples = 1ull << 20;
constexpr size_t kNoAllocScratchBytes = (17ull << 20);   // 16 MiB of partitions + plan and counters

size_t hj_raw_scratch_bytes(uint64_t max_tuples);
int hj_count_window_raw(const sjbg_tuple *dL, uint64_t nL, const sjbg_tuple *dR, uint64_t nR, uint8_t *sc,
                        size_t sc_bytes, sjbg_window_result *dOut, cudaStream_t st);

static __device__ __align__(256) uint8_t g_noalloc_scratch[kNoAllocScratchBytes];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_mu;
uint8_t *g_scratch_addr[kMaxDevices] = {};
}  // namespace

}  // namespace sjbg

using namespace sjbg;

extern "C" int sjbg_lazy_hj_noalloc(const sjbg_tuple *left, uint64_t n_left, const sjbg_tuple *right,
                                    uint64_t n_right, sjbg_window_result *out, void *cuda_stream) {
    if ((n_left && !left) || (n_right && !right) || !out)
        return fail(nullptr, SJBG_E_INVALID, "sjbg_lazy_hj_noalloc: null input or output");
    if (n_left > kNoAllocMaxTuples || n_right > kNoAllocMaxTuples)
        return fail(nullptr, SJBG_E_CAPACITY,
                    "sjbg_lazy_hj_noalloc: a window side exceeds 2^20 tuples (the fixed scratch holds no more)");
    if (hj_raw_scratch_bytes(kNoAllocMaxTuples) > kNoAllocScratchBytes)
        return fail(nullptr, SJBG_E_CAPACITY, "sjbg_lazy_hj_noalloc: scratch too small");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return fail(nullptr, SJBG_E_CUDA, "sjbg_lazy_hj_noalloc: no current CUDA device");
    }
    uint8_t *scratch = nullptr;
    {
        std::lock_guard<std::mutex> g(g_mu);
        if (!g_scratch_addr[dev]) {
            // the symbol's name is only a host-side stand-in: ask the runtime for
            // the array's address on the current device
            void *p = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) {
                cudaGetLastError();
                return fail(nullptr, SJBG_E_CUDA, std::string("sjbg_lazy_hj_noalloc: scratch address: ") +
                                                      cudaGetErrorString(e));
            }
            g_scratch_addr[dev] = static_cast<uint8_t *>(p);
        }
        scratch = g_scratch_addr[dev];
    }
    return hj_count_window_raw(left, n_left, right, n_right, scratch, kNoAllocScratchBytes, out,
                               static_cast<cudaStream_t>(cuda_stream));
}
