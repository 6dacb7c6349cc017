// api.cu - the extern "C" boundary (include/sjbg.h) and the handle runtime.
#include <algorithm>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "eager.cuh"
#include "runtime.h"
#include "stream.cuh"

namespace {
std::mutex g_err_mu;
std::string g_create_err;
}  // namespace

sjbg_handle::~sjbg_handle() {
    if (device >= 0) cudaSetDevice(device);
    eager.reset();
    streaming.reset();
    ring.reset();
    for (auto &g : graphs) {
        if (g->exec) cudaGraphExecDestroy(g->exec);
        for (auto &b : g->pinned)
            if (b.p) cudaFreeHost(b.p);
    }
    for (auto &b : ws)
        if (b.p) cudaFree(b.p);
    for (auto &b : pinned)
        if (b.p) cudaFreeHost(b.p);
    for (auto &p : pending) {
        event_pool.push_back(p.a);
        event_pool.push_back(p.b);
    }
    for (auto e : event_pool) cudaEventDestroy(e);
    if (own_stream) cudaStreamDestroy(own_stream);
    if (copy_stream) cudaStreamDestroy(copy_stream);
}

namespace sjbg {

int fail(sjbg_handle *h, int code, const std::string &msg) {
    if (h) h->err = msg;
    else {
        std::lock_guard<std::mutex> g(g_err_mu);
        g_create_err = msg;
    }
    return code;
}

int cuda_fail(sjbg_handle *h, cudaError_t e, const char *what) {
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    return fail(h, e == cudaErrorMemoryAllocation ? SJBG_E_NOMEM : SJBG_E_CUDA, m);
}

cudaError_t raise_smem_limit(const void *kernel, size_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<int, const void *>, size_t> granted;   // (device, kernel) -> limit set
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> g(mu);
    size_t &cur = granted[{dev, kernel}];
    if (bytes <= cur) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) cur = bytes;
    return e;
}

void *ws_get(sjbg_handle *h, WsSlot s, size_t bytes) {
    DevBuf &b = h->ws[s];
    bytes = std::max<size_t>(16, (bytes + 15) & ~(size_t)15);   // whole 16-byte words (stage_copy, zero_fill)
    if (b.bytes >= bytes) return b.p;
    if (b.p) {
        cudaStreamSynchronize(h->stream);   // a kernel may still use the old buffer
        cudaFree(b.p);
        b.p = nullptr;
        b.bytes = 0;
    }
    size_t want = std::max(bytes, b.bytes + b.bytes / 4);
    if (cudaMalloc(&b.p, want) != cudaSuccess) {
        cudaGetLastError();
        if (cudaMalloc(&b.p, bytes) != cudaSuccess) {
            cudaGetLastError();
            b.p = nullptr;
            return nullptr;
        }
        want = bytes;
    }
    b.bytes = want;
    return b.p;
}

void *pinned_get(sjbg_handle *h, int i, size_t bytes) {
    DevBuf &b = h->pinned[i];
    bytes = std::max<size_t>(16, (bytes + 15) & ~(size_t)15);
    if (b.bytes >= bytes) return b.p;
    if (b.p) {
        cudaStreamSynchronize(h->stream);
        cudaFreeHost(b.p);
        b.p = nullptr;
        b.bytes = 0;
    }
    size_t want = std::max(bytes, (size_t)4096);
    if (cudaMallocHost(&b.p, want) != cudaSuccess) {
        cudaGetLastError();
        b.p = nullptr;
        return nullptr;
    }
    b.bytes = want;
    return b.p;
}

// Small staging transfers (plans, accumulators) between pinned host memory
// and device memory are done by a kernel over mapped pinned memory, not by a
// copy engine: a copy engine works its queue in order, so a plan upload
// queued behind a large input copy on another stream would wait for it.
// Both buffers come from ws_get / pinned_get, whose sizes are whole 16-byte
// words, so a 16-byte-aligned pair is copied in whole words: one round of
// loads over the host link, no byte tail.
__global__ void stage_copy_kernel(uint8_t *__restrict__ dst, const uint8_t *__restrict__ src, size_t bytes,
                                  bool vec) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t n16 = vec ? (bytes + 15) / 16 : 0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n16; i += stride)
        reinterpret_cast<uint4 *>(dst)[i] = reinterpret_cast<const uint4 *>(src)[i];
    if (vec) return;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < bytes; i += stride) dst[i] = src[i];
}

__global__ void zero_fill_kernel(uint4 *__restrict__ dst, size_t n16) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n16; i += stride) dst[i] = make_uint4(0, 0, 0, 0);
}

int zero_fill(sjbg_handle *h, void *dst, size_t bytes) {
    const size_t n16 = (bytes + 15) / 16;
    if (n16 == 0) return SJBG_OK;
    const uint32_t blocks =
        (uint32_t)std::min<size_t>((n16 + 255) / 256, (size_t)8 * (size_t)std::max(h->num_sms, 1));
    SJBG_CK(h, launch(h, "zero_fill", zero_fill_kernel, dim3(blocks), dim3(256), 0, static_cast<uint4 *>(dst), n16));
    return SJBG_OK;
}

// CTA 0 copies the staged bytes (16-byte words when both sides allow); every
// CTA zeroes its share of zdst.
__global__ void stage_copy_zero_kernel(uint8_t *__restrict__ dst, const uint8_t *__restrict__ src, size_t bytes,
                                       bool vec, uint4 *__restrict__ zdst, size_t n16) {
    if (blockIdx.x == 0) {
        if (vec) {
            for (size_t i = threadIdx.x; i < (bytes + 15) / 16; i += blockDim.x)
                reinterpret_cast<uint4 *>(dst)[i] = reinterpret_cast<const uint4 *>(src)[i];
        } else {
            for (size_t i = threadIdx.x; i < bytes; i += blockDim.x) dst[i] = src[i];
        }
    }
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n16; i += stride) zdst[i] = make_uint4(0, 0, 0, 0);
}

int stage_copy_zero(sjbg_handle *h, void *dst, const void *src, size_t bytes, void *zdst, size_t zbytes) {
    const size_t n16 = (zbytes + 15) / 16;
    if (bytes == 0) return zero_fill(h, zdst, zbytes);
    if (n16 == 0) return stage_copy(h, dst, src, bytes);
    const bool vec = (((uintptr_t)dst | (uintptr_t)src) & 15u) == 0;
    const uint32_t blocks =
        (uint32_t)std::min<size_t>((n16 + 255) / 256, (size_t)8 * (size_t)std::max(h->num_sms, 1));
    SJBG_CK(h, launch(h, "stage_copy_zero", stage_copy_zero_kernel, dim3(std::max<uint32_t>(blocks, 1)), dim3(256), 0,
                      static_cast<uint8_t *>(dst), static_cast<const uint8_t *>(src), bytes, vec,
                      static_cast<uint4 *>(zdst), n16));
    return SJBG_OK;
}

int stage_copy(sjbg_handle *h, void *dst, const void *src, size_t bytes) {
    if (bytes == 0) return SJBG_OK;
    const bool vec = (((uintptr_t)dst | (uintptr_t)src) & 15u) == 0;
    const uint32_t blocks = (uint32_t)std::min<size_t>(64, (bytes + 4095) / 4096);
    SJBG_CK(h, launch(h, "stage_copy", stage_copy_kernel, dim3(blocks), dim3(256), 0, static_cast<uint8_t *>(dst),
                      static_cast<const uint8_t *>(src), bytes, vec));
    return SJBG_OK;
}

int kernel_id(sjbg_handle *h, const char *name) {
    for (size_t i = 0; i < h->knames.size(); i++)
        if (h->knames[i] == name) return (int)i;
    h->knames.emplace_back(name);
    h->klaunches.push_back(0);
    h->kms.push_back(0.0);
    return (int)h->knames.size() - 1;
}

cudaEvent_t event_get(sjbg_handle *h) {
    if (!h->event_pool.empty()) {
        cudaEvent_t e = h->event_pool.back();
        h->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}

void profile_collect(sjbg_handle *h) {
    for (auto &p : h->pending) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
            h->klaunches[p.kid]++;
            h->kms[p.kid] += ms;
        }
        h->event_pool.push_back(p.a);
        h->event_pool.push_back(p.b);
    }
    h->pending.clear();
}

// ---- lazy batches ---------------------------------------------------------------
static bool wants_pairs(const sjbg_handle *h) { return h->cfg.result_mode != SJBG_RESULT_NO_OUTPUT; }

// Run windows whose spans index device arrays dL / dR; dPairs (device) may be null.
int run_lazy_device(sjbg_handle *h, const sjbg_tuple *dL, const sjbg_tuple *dR, const WinHost *wins, uint32_t n,
                           sjbg_pair *dPairs, WinAcc *hAcc, uint32_t *part_used) {
    const bool pairs = dPairs != nullptr;
    const bool enumerate = pairs || (h->cfg.flags & SJBG_F_XOR);
    // acc[n].info is the call's device status word (kErr* bits)
    WinAcc *acc = static_cast<WinAcc *>(ws_get(h, WS_WIN_ACC, sizeof(WinAcc) * (n + 1)));
    if (!acc) return fail(h, SJBG_E_NOMEM, "window accumulators");
    SJBG_CK(h, cudaMemsetAsync(acc, 0, sizeof(WinAcc) * (n + 1), h->stream));
    int rc = SJBG_OK;
    *part_used = SJBG_PART_NONE;
    switch (h->cfg.algorithm) {
        case SJBG_ALG_HJ: rc = hj_lazy_batch(h, dL, dR, wins, n, dPairs, acc, enumerate, part_used); break;
        case SJBG_ALG_NLJ: rc = nlj_lazy_batch(h, dL, dR, wins, n, dPairs, acc, enumerate); break;
        case SJBG_ALG_SMJ: rc = smj_lazy_batch(h, dL, dR, wins, n, dPairs, acc, enumerate); break;
        default: rc = fail(h, SJBG_E_UNSUPPORTED, "unknown algorithm");
    }
    if (rc) return rc;
    return stage_copy(h, hAcc, acc, sizeof(WinAcc) * (n + 1));
}

int device_status_error(sjbg_handle *h, unsigned long long bits) {
    if (!bits) return SJBG_OK;
    if (bits & kErrTimeout) return fail(h, SJBG_E_TIMEOUT, "a bounded device-side wait gave up");
    if (bits & kErrTableFull) return fail(h, SJBG_E_CAPACITY, "a device hash table could not take a key");
    if (bits & kErrQueue) return fail(h, SJBG_E_CAPACITY, "a device work queue overflowed");
    return fail(h, SJBG_E_INVALID, "a kernel rejected a window descriptor");
}

static void fill_result(const sjbg_handle *h, const WinAcc &a, const WinHost &w, bool enumerate, bool pairs,
                        uint32_t part_used, float ms, sjbg_window_result *out) {
    std::memset(out, 0, sizeof(*out));
    out->count = a.count;
    out->prod_checksum = a.prod;
    out->partitioner_used = part_used;
    if (part_used == SJBG_PART_LEARNED && (a.info & (kInfoFallback | kInfoRadixByCost))) {
        out->partitioner_used = SJBG_PART_RADIX;
        out->flags |= (a.info & kInfoFallback) ? SJBG_WR_FALLBACK : SJBG_WR_RADIX_BY_COST;
    }
    out->ms = ms;
    if (enumerate) {
        out->xor_checksum = a.xr;
        out->flags |= SJBG_WR_XOR;
    }
    if (pairs) {
        out->n_pairs = std::min<uint64_t>(a.npairs, w.pairs_cap);
        if (a.npairs > w.pairs_cap) out->flags |= SJBG_WR_PAIRS_TRUNCATED;
    }
    (void)h;
}

// Batched lazy call on device inputs through a cached CUDA graph: the first
// call with a given signature runs normally (sizing every workspace), then is
// captured with private pinned staging buffers; later identical calls replay it.
static int lazy_graph(sjbg_handle *h, const sjbg_tuple *dL, const sjbg_tuple *dR, const WinHost *wins, uint32_t n,
                      sjbg_pair *dPairs, bool enumerate, sjbg_window_result *out) {
    std::vector<uint64_t> key = {h->cfg.algorithm, h->cfg.partitioner, h->tune.partitioner, h->cfg.flags, h->cfg.result_mode,
                                 (uint64_t)(uintptr_t)dL, (uint64_t)(uintptr_t)dR, (uint64_t)(uintptr_t)dPairs, n,
                                 h->tune.bucket_target, (uint64_t)h->tune.persistent_join,
                                 (uint64_t)(uintptr_t)h->stream};
    for (uint32_t w = 0; w < n; w++) {
        const WinHost &x = wins[w];
        key.insert(key.end(), {x.left_off, x.n_left, x.right_off, x.n_right, x.pairs_off, x.pairs_cap});
    }
    sjbg_handle::GraphEntry *entry = nullptr;
    for (auto &g : h->graphs)
        if (g->key == key) entry = g.get();
    cudaEvent_t e0 = event_get(h), e1 = event_get(h);
    WinAcc *hAcc = nullptr;
    uint32_t part_used = SJBG_PART_NONE;
    if (entry) {
        SJBG_CK(h, cudaEventRecord(e0, h->stream));
        SJBG_CK(h, cudaGraphLaunch(entry->exec, h->stream));
        SJBG_CK(h, cudaEventRecord(e1, h->stream));
        h->launches += entry->kernels;   // the replay runs every captured kernel again
        hAcc = static_cast<WinAcc *>(entry->pinned[3].p);
        part_used = entry->part_used;
    } else {
        hAcc = static_cast<WinAcc *>(pinned_get(h, 3, sizeof(WinAcc) * (n + 1)));
        if (!hAcc) return fail(h, SJBG_E_NOMEM, "result staging");
        SJBG_CK(h, cudaEventRecord(e0, h->stream));
        int rc = run_lazy_device(h, dL, dR, wins, n, dPairs, hAcc, &part_used);   // warm-up: sizes every buffer
        if (rc) return rc;
        SJBG_CK(h, cudaEventRecord(e1, h->stream));
        SJBG_CK(h, cudaStreamSynchronize(h->stream));
        profile_collect(h);
        auto e = std::make_unique<sjbg_handle::GraphEntry>();
        e->key = key;
        e->part_used = part_used;
        for (int i = 0; i < 6; i++) {   // private copies of the staging buffers the capture will reference
            if (!h->pinned[i].bytes) continue;
            if (cudaMallocHost(&e->pinned[i].p, h->pinned[i].bytes) != cudaSuccess) {
                cudaGetLastError();
                for (auto &b : e->pinned)
                    if (b.p) cudaFreeHost(b.p);
                return fail(h, SJBG_E_NOMEM, "graph staging");
            }
            e->pinned[i].bytes = h->pinned[i].bytes;
        }
        for (int i = 0; i < 6; i++) std::swap(h->pinned[i], e->pinned[i]);
        h->capturing = true;
        const uint64_t launches_before = h->launches;
        cudaGraph_t graph = nullptr;
        cudaError_t ce = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeRelaxed);
        uint32_t pu2 = 0;
        int rc2 = ce == cudaSuccess ? run_lazy_device(h, dL, dR, wins, n, dPairs,
                                                      static_cast<WinAcc *>(h->pinned[3].p), &pu2)
                                    : SJBG_E_CUDA;
        cudaError_t ce2 = cudaStreamEndCapture(h->stream, &graph);
        h->capturing = false;
        e->kernels = h->launches - launches_before;
        h->launches = launches_before;   // capture runs nothing
        for (int i = 0; i < 6; i++) std::swap(h->pinned[i], e->pinned[i]);
        if (rc2 == SJBG_OK && ce == cudaSuccess && ce2 == cudaSuccess && graph) {
            if (cudaGraphInstantiate(&e->exec, graph, 0) != cudaSuccess) e->exec = nullptr;
        }
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        if (e->exec) {
            if (h->graphs.size() >= 8) {
                auto &old = h->graphs.front();
                cudaGraphExecDestroy(old->exec);
                for (auto &b : old->pinned)
                    if (b.p) cudaFreeHost(b.p);
                h->graphs.erase(h->graphs.begin());
            }
            h->graphs.push_back(std::move(e));
        } else {
            for (auto &b : e->pinned)
                if (b.p) cudaFreeHost(b.p);
        }
    }
    SJBG_CK(h, cudaStreamSynchronize(h->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    h->event_pool.push_back(e0);
    h->event_pool.push_back(e1);
    if (int se = device_status_error(h, hAcc[n].info)) return se;
    for (uint32_t w = 0; w < n; w++) fill_result(h, hAcc[w], wins[w], enumerate, dPairs != nullptr, part_used, ms, &out[w]);
    return SJBG_OK;
}

// Host inputs, several windows: the windows are cut into groups of about an
// eighth of the input bytes; every group's input copy is enqueued at once on
// the copy stream, and each group's join starts as soon as its copy has
// landed, so the joins of early groups overlap the copies of later ones.
// The groups run one after another on the handle's stream (the staging
// buffers are reused), so the call lasts about the copy time plus the last
// group's join.
static int lazy_host_pipelined(sjbg_handle *h, const sjbg_tuple *L, const sjbg_tuple *R, const WinHost *wins,
                               uint32_t n, sjbg_pair *pairs, bool want, bool enumerate, uint64_t needL,
                               uint64_t needR, uint64_t needP, sjbg_window_result *out) {
    if (!h->copy_stream) SJBG_CK(h, cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
    sjbg_tuple *sL = static_cast<sjbg_tuple *>(ws_get(h, WS_IN_LEFT, sizeof(sjbg_tuple) * needL));
    sjbg_tuple *sR = static_cast<sjbg_tuple *>(ws_get(h, WS_IN_RIGHT, sizeof(sjbg_tuple) * needR));
    sjbg_pair *dP = want ? static_cast<sjbg_pair *>(ws_get(h, WS_PAIRS, sizeof(sjbg_pair) * needP)) : nullptr;
    if ((needL && !sL) || (needR && !sR) || (want && !dP)) return fail(h, SJBG_E_NOMEM, "input staging");
    uint64_t total = 0;
    for (uint32_t w = 0; w < n; w++) total += wins[w].n_left + wins[w].n_right;
    std::vector<uint32_t> gfirst;   // first window of each group
    uint64_t run = 0;
    for (uint32_t w = 0; w < n; w++) {
        if (w == 0 || run >= total / 8) {
            gfirst.push_back(w);
            run = 0;
        }
        run += wins[w].n_left + wins[w].n_right;
    }
    const uint32_t G = (uint32_t)gfirst.size();
    gfirst.push_back(n);
    std::vector<cudaEvent_t> landed(G);
    for (auto &e : landed) e = event_get(h);
    cudaEvent_t e0 = event_get(h), e1 = event_get(h);
    auto release = [&]() {
        for (auto e : landed) h->event_pool.push_back(e);
        h->event_pool.push_back(e0);
        h->event_pool.push_back(e1);
    };
    SJBG_CK(h, cudaEventRecord(e0, h->stream));
    SJBG_CK(h, cudaStreamWaitEvent(h->copy_stream, e0, 0));
    for (uint32_t g = 0; g < G; g++) {
        uint64_t lo[2] = {~0ull, ~0ull}, hi[2] = {0, 0};
        for (uint32_t w = gfirst[g]; w < gfirst[g + 1]; w++) {
            if (wins[w].n_left) {
                lo[0] = std::min(lo[0], wins[w].left_off);
                hi[0] = std::max(hi[0], wins[w].left_off + wins[w].n_left);
            }
            if (wins[w].n_right) {
                lo[1] = std::min(lo[1], wins[w].right_off);
                hi[1] = std::max(hi[1], wins[w].right_off + wins[w].n_right);
            }
        }
        if (hi[0] > lo[0] && lo[0] != ~0ull)
            SJBG_CK(h, cudaMemcpyAsync(sL + lo[0], L + lo[0], sizeof(sjbg_tuple) * (hi[0] - lo[0]),
                                       cudaMemcpyHostToDevice, h->copy_stream));
        if (hi[1] > lo[1] && lo[1] != ~0ull)
            SJBG_CK(h, cudaMemcpyAsync(sR + lo[1], R + lo[1], sizeof(sjbg_tuple) * (hi[1] - lo[1]),
                                       cudaMemcpyHostToDevice, h->copy_stream));
        SJBG_CK(h, cudaEventRecord(landed[g], h->copy_stream));
    }
    std::vector<WinAcc> acc(n);
    uint32_t part_used = SJBG_PART_NONE;
    for (uint32_t g = 0; g < G; g++) {
        const uint32_t w0 = gfirst[g], m = gfirst[g + 1] - w0;
        WinAcc *hAcc = static_cast<WinAcc *>(pinned_get(h, 3, sizeof(WinAcc) * (m + 1)));
        if (!hAcc) {
            release();
            return fail(h, SJBG_E_NOMEM, "result staging");
        }
        SJBG_CK(h, cudaStreamWaitEvent(h->stream, landed[g], 0));
        uint32_t pu = SJBG_PART_NONE;
        int rc = run_lazy_device(h, sL, sR, wins + w0, m, dP, hAcc, &pu);
        if (rc) {
            cudaStreamSynchronize(h->copy_stream);
            release();
            return rc;
        }
        if (g == 0) part_used = pu;
        // the staging buffers (pinned plan uploads, accumulators) are reused by the next group
        SJBG_CK(h, cudaStreamSynchronize(h->stream));
        if (int se = device_status_error(h, hAcc[m].info)) {
            cudaStreamSynchronize(h->copy_stream);
            release();
            return se;
        }
        std::copy(hAcc, hAcc + m, acc.begin() + w0);
    }
    if (want) {
        for (uint32_t w = 0; w < n; w++) {
            const uint64_t np = std::min<uint64_t>(acc[w].npairs, wins[w].pairs_cap);
            if (np)
                SJBG_CK(h, cudaMemcpyAsync(pairs + wins[w].pairs_off, dP + wins[w].pairs_off, sizeof(sjbg_pair) * np,
                                           cudaMemcpyDeviceToHost, h->stream));
        }
    }
    SJBG_CK(h, cudaEventRecord(e1, h->stream));
    SJBG_CK(h, cudaStreamSynchronize(h->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    release();
    profile_collect(h);
    for (uint32_t w = 0; w < n; w++) fill_result(h, acc[w], wins[w], enumerate, want, part_used, ms, &out[w]);
    return SJBG_OK;
}

int lazy_common(sjbg_handle *h, const sjbg_tuple *L, const sjbg_tuple *R, uint32_t mem, const WinHost *wins,
                uint32_t n, sjbg_pair *pairs, sjbg_window_result *out) {
    if (!h) return SJBG_E_INVALID;
    if (h->cfg.progressiveness != SJBG_LAZY) return fail(h, SJBG_E_STATE, "lazy call on an eager handle");
    if (mem != SJBG_MEM_HOST && mem != SJBG_MEM_DEVICE) return fail(h, SJBG_E_INVALID, "bad memory kind");
    if (n && !wins) return fail(h, SJBG_E_INVALID, "null window list");
    if (!out) return fail(h, SJBG_E_INVALID, "null result");
    SJBG_CK(h, cudaSetDevice(h->device));
    uint64_t needL = 0, needR = 0, needP = 0;
    for (uint32_t w = 0; w < n; w++) {
        if (wins[w].n_left > h->cfg.max_tuples_per_window || wins[w].n_right > h->cfg.max_tuples_per_window)
            return fail(h, SJBG_E_CAPACITY, "window larger than max_tuples_per_window");
        needL = std::max(needL, wins[w].left_off + wins[w].n_left);
        needR = std::max(needR, wins[w].right_off + wins[w].n_right);
        needP = std::max(needP, wins[w].pairs_off + wins[w].pairs_cap);
    }
    if ((needL && !L) || (needR && !R)) return fail(h, SJBG_E_INVALID, "null input span");
    const bool want = wants_pairs(h) && pairs != nullptr && needP > 0;
    const bool enumerate = want || (h->cfg.flags & SJBG_F_XOR);

    if (h->cfg.flags & SJBG_F_AUTOTUNE) {
        if (mem == SJBG_MEM_DEVICE) {
            int rc = autotune_lazy(h, L, R, wins, n, enumerate);
            if (rc) return rc;
        }
    }
    if ((h->cfg.flags & SJBG_F_GRAPH) && mem == SJBG_MEM_DEVICE && h->cfg.result_mode != SJBG_RESULT_COUNT_KERNEL)
        return lazy_graph(h, L, R, wins, n, want ? pairs : nullptr, enumerate, out);
    if (mem == SJBG_MEM_HOST && n > 1 && !(want && h->cfg.result_mode == SJBG_RESULT_COUNT_KERNEL))
        return lazy_host_pipelined(h, L, R, wins, n, pairs, want, enumerate, needL, needR, needP, out);
    cudaEvent_t e0 = event_get(h), e1 = event_get(h);
    SJBG_CK(h, cudaEventRecord(e0, h->stream));
    const sjbg_tuple *dL = L, *dR = R;
    sjbg_pair *dP = want ? pairs : nullptr;
    if (mem == SJBG_MEM_HOST) {
        sjbg_tuple *sL = static_cast<sjbg_tuple *>(ws_get(h, WS_IN_LEFT, sizeof(sjbg_tuple) * needL));
        sjbg_tuple *sR = static_cast<sjbg_tuple *>(ws_get(h, WS_IN_RIGHT, sizeof(sjbg_tuple) * needR));
        if (!sL || !sR) return fail(h, SJBG_E_NOMEM, "input staging");
        if (needL) SJBG_CK(h, cudaMemcpyAsync(sL, L, sizeof(sjbg_tuple) * needL, cudaMemcpyHostToDevice, h->stream));
        if (needR) SJBG_CK(h, cudaMemcpyAsync(sR, R, sizeof(sjbg_tuple) * needR, cudaMemcpyHostToDevice, h->stream));
        dL = sL;
        dR = sR;
        if (want) {
            dP = static_cast<sjbg_pair *>(ws_get(h, WS_PAIRS, sizeof(sjbg_pair) * needP));
            if (!dP) return fail(h, SJBG_E_NOMEM, "pair staging");
        }
    }
    // CountKernel mode: an exact count first; refuse instead of truncating
    if (want && h->cfg.result_mode == SJBG_RESULT_COUNT_KERNEL) {
        WinAcc *hp = static_cast<WinAcc *>(pinned_get(h, 4, sizeof(WinAcc) * (n + 1)));
        if (!hp) return fail(h, SJBG_E_NOMEM, "count staging");
        uint32_t pu;
        int rc = run_lazy_device(h, dL, dR, wins, n, nullptr, hp, &pu);
        if (rc) return rc;
        SJBG_CK(h, cudaStreamSynchronize(h->stream));
        if (int se = device_status_error(h, hp[n].info)) return se;
        for (uint32_t w = 0; w < n; w++)
            if (hp[w].count > wins[w].pairs_cap)
                return fail(h, SJBG_E_CAPACITY, "pair buffer smaller than the window's match count");
    }
    WinAcc *hAcc = static_cast<WinAcc *>(pinned_get(h, 3, sizeof(WinAcc) * (n + 1)));
    if (!hAcc) return fail(h, SJBG_E_NOMEM, "result staging");
    uint32_t part_used = SJBG_PART_NONE;
    int rc = run_lazy_device(h, dL, dR, wins, n, dP, hAcc, &part_used);
    if (rc) return rc;
    if (mem == SJBG_MEM_HOST && want) {
        // copy back each window's written pairs
        SJBG_CK(h, cudaStreamSynchronize(h->stream));
        if (int se = device_status_error(h, hAcc[n].info)) return se;
        for (uint32_t w = 0; w < n; w++) {
            const uint64_t np = std::min<uint64_t>(hAcc[w].npairs, wins[w].pairs_cap);
            if (np)
                SJBG_CK(h, cudaMemcpyAsync(pairs + wins[w].pairs_off, dP + wins[w].pairs_off, sizeof(sjbg_pair) * np,
                                           cudaMemcpyDeviceToHost, h->stream));
        }
    }
    SJBG_CK(h, cudaEventRecord(e1, h->stream));
    SJBG_CK(h, cudaStreamSynchronize(h->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    h->event_pool.push_back(e0);
    h->event_pool.push_back(e1);
    profile_collect(h);
    if (int se = device_status_error(h, hAcc[n].info)) return se;
    for (uint32_t w = 0; w < n; w++) fill_result(h, hAcc[w], wins[w], enumerate, want, part_used, ms, &out[w]);
    return SJBG_OK;
}

}  // namespace sjbg

using namespace sjbg;

extern "C" {

int sjbg_version(void) { return SJBG_ABI_VERSION; }

int sjbg_create(const sjbg_config *cfg, sjbg_handle **out) {
    if (!cfg || !out) return fail(nullptr, SJBG_E_INVALID, "null argument");
    *out = nullptr;
    if (cfg->algorithm != SJBG_ALG_HJ && cfg->algorithm != SJBG_ALG_NLJ && cfg->algorithm != SJBG_ALG_SMJ)
        return fail(nullptr, SJBG_E_UNSUPPORTED, "algorithm must be NLJ, HJ or SMJ");
    if (cfg->progressiveness != SJBG_LAZY && cfg->progressiveness != SJBG_EAGER)
        return fail(nullptr, SJBG_E_INVALID, "progressiveness must be LAZY or EAGER");
    if (cfg->result_mode > SJBG_RESULT_ATOMIC) return fail(nullptr, SJBG_E_INVALID, "bad result mode");
    if (cfg->partitioner > SJBG_PART_LEARNED) return fail(nullptr, SJBG_E_INVALID, "bad partitioner");
    if (cfg->radix_bits > 14) return fail(nullptr, SJBG_E_INVALID, "radix_bits must be <= 14");
    if (cfg->max_tuples_per_window == 0) return fail(nullptr, SJBG_E_INVALID, "max_tuples_per_window must be > 0");
    if (cfg->progressiveness == SJBG_EAGER && (cfg->batch_size == 0 || cfg->window_size == 0))
        return fail(nullptr, SJBG_E_INVALID, "eager handles need batch_size and window_size");
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(nullptr, SJBG_E_CUDA, "no CUDA device available");
    }
    if (cfg->device < 0 || cfg->device >= ndev) return fail(nullptr, SJBG_E_INVALID, "bad device ordinal");
    std::unique_ptr<sjbg_handle> h(new sjbg_handle());
    h->cfg = *cfg;
    // SJBG_PART_AUTO stays: each hash-join call picks (hj.cu: choose_partitioner)
    // tuning knobs pinned from the environment (the autotuner then leaves them)
    if (const char *e = std::getenv("SJBG_BUCKET_TARGET")) {
        const long v = std::strtol(e, nullptr, 10);
        if (v >= 256 && v <= (1 << 16)) h->tune.bucket_target = (uint32_t)v;
    }
    if (const char *e = std::getenv("SJBG_PERSISTENT_JOIN")) h->tune.persistent_join = std::atoi(e) != 0;
    h->device = cfg->device;
    if ((e = cudaSetDevice(h->device)) != cudaSuccess) return fail(nullptr, SJBG_E_CUDA, cudaGetErrorString(e));
    cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device);
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device);
    h->max_smem_optin = (size_t)optin;
    if ((e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking)) != cudaSuccess)
        return fail(nullptr, SJBG_E_CUDA, cudaGetErrorString(e));
    h->stream = h->own_stream;
    if (cfg->progressiveness == SJBG_EAGER) {
        int rc = eager_init_and_clear(h.get());
        if (rc) {
            std::lock_guard<std::mutex> g(g_err_mu);
            g_create_err = h->err;
            return rc;
        }
    }
    *out = h.release();
    return SJBG_OK;
}

int sjbg_destroy(sjbg_handle *h) {
    if (!h) return SJBG_E_INVALID;
    eager_shutdown(h);
    if (h->stream) cudaStreamSynchronize(h->stream);
    delete h;
    return SJBG_OK;
}

const char *sjbg_last_error(const sjbg_handle *h) {
    if (h) return h->err.c_str();
    std::lock_guard<std::mutex> g(g_err_mu);
    return g_create_err.c_str();
}

int sjbg_set_stream(sjbg_handle *h, void *cuda_stream) {
    if (!h) return SJBG_E_INVALID;
    h->stream = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : h->own_stream;
    return SJBG_OK;
}

int sjbg_lazy_execute(sjbg_handle *h, const sjbg_tuple *left, uint64_t n_left, const sjbg_tuple *right,
                      uint64_t n_right, uint32_t mem, sjbg_pair *pairs, uint64_t pairs_capacity,
                      sjbg_window_result *out) {
    WinHost w{0, n_left, 0, n_right, 0, pairs ? pairs_capacity : 0};
    return lazy_common(h, left, right, mem, &w, 1, pairs, out);
}

int sjbg_lazy_execute_ring(sjbg_handle *h, const sjbg_tuple *left_ring, const uint64_t *left_batch_offsets,
                           uint64_t n_left_batches, const sjbg_tuple *right_ring, const uint64_t *right_batch_offsets,
                           uint64_t n_right_batches, sjbg_pair *pairs, uint64_t pairs_capacity,
                           sjbg_window_result *out) {
    if (!h) return SJBG_E_INVALID;
    const uint64_t B = h->cfg.batch_size;
    if (B == 0) return fail(h, SJBG_E_INVALID, "batch_size must be set for ring windows");
    if ((n_left_batches && (!left_ring || !left_batch_offsets)) ||
        (n_right_batches && (!right_ring || !right_batch_offsets)))
        return fail(h, SJBG_E_INVALID, "null ring or offsets");
    // gather the window's batches into contiguous pinned spans (the reference's
    // copyTuplesToLocalStore assumes contiguity, GPU_HJ.cu:237-242)
    const uint64_t nL = n_left_batches * B, nR = n_right_batches * B;
    sjbg_tuple *g = static_cast<sjbg_tuple *>(pinned_get(h, 2, sizeof(sjbg_tuple) * (nL + nR)));
    if (!g) return fail(h, SJBG_E_NOMEM, "ring gather buffer");
    for (uint64_t i = 0; i < n_left_batches; i++)
        std::memcpy(g + i * B, left_ring + left_batch_offsets[i], sizeof(sjbg_tuple) * B);
    for (uint64_t i = 0; i < n_right_batches; i++)
        std::memcpy(g + nL + i * B, right_ring + right_batch_offsets[i], sizeof(sjbg_tuple) * B);
    WinHost w{0, nL, 0, nR, 0, pairs ? pairs_capacity : 0};
    return lazy_common(h, g, g + nL, SJBG_MEM_HOST, &w, 1, pairs, out);
}

int sjbg_lazy_execute_batch(sjbg_handle *h, const sjbg_tuple *left, const sjbg_tuple *right, uint32_t mem,
                            const sjbg_window_desc *windows, uint32_t n_windows, sjbg_pair *pairs,
                            sjbg_window_result *out) {
    if (!h) return SJBG_E_INVALID;
    std::vector<WinHost> w(n_windows);
    for (uint32_t i = 0; i < n_windows; i++) {
        const sjbg_window_desc &d = windows[i];
        w[i] = WinHost{d.left_offset, d.n_left, d.right_offset, d.n_right, d.pairs_offset,
                       pairs ? d.pairs_capacity : 0};
    }
    return lazy_common(h, left, right, mem, w.data(), n_windows, pairs, out);
}

int sjbg_generate(sjbg_handle *h, sjbg_tuple *dev_out, uint64_t first, uint64_t n, uint64_t seed, uint64_t domain,
                  const uint64_t *zipf_table, uint64_t perm_seed) {
    if (!h || (!dev_out && n)) return SJBG_E_INVALID;
    if (domain == 0 || domain > (1ull << 32)) return fail(h, SJBG_E_INVALID, "domain must be in [1, 2^32]");
    SJBG_CK(h, cudaSetDevice(h->device));
    int rc = generate_device(h, dev_out, first, n, seed, domain, zipf_table, perm_seed);
    if (rc) return rc;
    SJBG_CK(h, cudaStreamSynchronize(h->stream));
    return SJBG_OK;
}

int sjbg_zipf_table(uint64_t *table, uint64_t n, double z) {
    if (!table || n == 0 || !(z >= 0.0)) return SJBG_E_INVALID;
    sjbg_zipf_table_fill(table, n, z);
    return SJBG_OK;
}

int sjbg_kernel_stats(sjbg_handle *h, uint32_t index, char *name, size_t name_len, uint64_t *launches,
                      double *total_ms) {
    if (!h) return SJBG_E_INVALID;
    if (index >= h->knames.size()) return SJBG_E_INVALID;
    if (name && name_len) {
        std::strncpy(name, h->knames[index].c_str(), name_len - 1);
        name[name_len - 1] = 0;
    }
    if (launches) *launches = h->klaunches[index];
    if (total_ms) *total_ms = h->kms[index];
    return SJBG_OK;
}

int sjbg_kernel_stats_reset(sjbg_handle *h) {
    if (!h) return SJBG_E_INVALID;
    std::fill(h->klaunches.begin(), h->klaunches.end(), 0);
    std::fill(h->kms.begin(), h->kms.end(), 0.0);
    return SJBG_OK;
}

uint64_t sjbg_launch_count(const sjbg_handle *h) { return h ? h->launches : 0; }

}  // extern "C"
