// ring.cu - device-resident ingest ring for count-based lazy windows (sm_103a host runtime).
//
// The reference's Lazy::CountBased (include/sjb/windowing/lazy/CountBased.cuh:45-101)
// memmoves every incoming batch into a pinned host ring (`:65`); once both
// sides hold a window's worth of batches it hands their ring offsets to a
// joiner, which copies the window to the device and joins it
// (e.g. src/sjb/windowing/lazy/executor/GPU/GPU_HJ.cu, copyTuplesToLocalStore),
// one window per call.  Here the ring lives in HBM:
//
//   * per side, `depth` window slots of W tuples each; window k (tuples
//     [kW, (k+1)W) of each side in arrival order, the reference's tumbling
//     count window) occupies slot k mod depth;
//   * a pushed batch is copied straight into its slot on the ring's copy
//     stream (pinned host batches asynchronously, with no host memmove),
//     split where it crosses a window boundary;
//   * when both sides have filled window k, its join is enqueued on the
//     handle's stream behind an event wait on the two copies only, so the
//     copies of window k + 1 run while window k is joined;
//   * results come back through sjbg_ring_poll, in window order; a slot is
//     reused once its window's join has finished.  A side that runs `depth`
//     windows ahead of the other has nowhere to put its next batch: the push
//     fails with SJBG_E_CAPACITY (the reference exits: "Ring buffer is full").
#include <algorithm>
#include <cstring>
#include <deque>
#include <vector>

#include "runtime.h"

namespace sjbg {

struct RingSlot {
    uint64_t id = 0;                     // window in the slot
    int state = 0;                       // 0 free / filling, 1 join enqueued
    bool filled[2] = {false, false};
    cudaEvent_t copied[2] = {nullptr, nullptr};   // the side's last copy into the window
    cudaEvent_t done = nullptr;
    DevBuf pinned[6];                    // private staging of this window's join
    uint32_t part_used = 0;
    int last_side = 0;                   // the side whose copy completed the window last
};

struct RingState {
    uint64_t W = 0;
    uint32_t depth = 0;
    sjbg_tuple *buf[2] = {nullptr, nullptr};
    cudaStream_t copy = nullptr;
    uint64_t pushed[2] = {0, 0};   // tuples per side so far
    uint64_t launched = 0;         // windows whose joins are enqueued: ids < launched
    uint64_t harvested = 0;        // windows reported: ids < harvested
    std::vector<RingSlot> slots;
    std::deque<sjbg_stream_window> ready;
    std::vector<double> lat_ms;
    uint64_t joined = 0, fallbacks = 0;
    ~RingState() {
        if (copy) cudaStreamSynchronize(copy);
        for (auto &s : slots) {
            if (s.done) cudaEventSynchronize(s.done);
            for (cudaEvent_t e : {s.copied[0], s.copied[1], s.done})
                if (e) cudaEventDestroy(e);
            for (auto &b : s.pinned)
                if (b.p) cudaFreeHost(b.p);
        }
        for (sjbg_tuple *b : buf)
            if (b) cudaFree(b);
        if (copy) cudaStreamDestroy(copy);
    }
};

void RingDeleter::operator()(RingState *p) const { delete p; }

static RingState *rs(sjbg_handle *h) { return h->ring.get(); }

// Report the finished windows, in window order (wait: block on each).
static int ring_harvest(sjbg_handle *h, RingState &st, bool wait) {
    while (st.harvested < st.launched) {
        RingSlot &s = st.slots[st.harvested % st.depth];
        if (wait) {
            SJBG_CK(h, cudaEventSynchronize(s.done));
        } else if (cudaEventQuery(s.done) != cudaSuccess) {
            cudaGetLastError();
            break;
        }
        const WinAcc *a = static_cast<const WinAcc *>(s.pinned[3].p);
        sjbg_stream_window r;
        std::memset(&r, 0, sizeof(r));
        r.window_id = s.id;
        r.n_left = r.n_right = st.W;
        r.result.count = a[0].count;
        r.result.prod_checksum = a[0].prod;
        if (h->cfg.flags & SJBG_F_XOR) {
            r.result.xor_checksum = a[0].xr;
            r.result.flags |= SJBG_WR_XOR;
        }
        r.result.partitioner_used = s.part_used;
        if (s.part_used == SJBG_PART_LEARNED && (a[0].info & (kInfoFallback | kInfoRadixByCost))) {
            r.result.partitioner_used = SJBG_PART_RADIX;
            if (a[0].info & kInfoFallback) {
                r.result.flags |= SJBG_WR_FALLBACK;
                st.fallbacks++;
            } else {
                r.result.flags |= SJBG_WR_RADIX_BY_COST;
            }
        }
        const unsigned long long bits = a[1].info;   // the join's device status word
        if (bits) r.result.status = bits & kErrTimeout ? SJBG_E_TIMEOUT : SJBG_E_CAPACITY;
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, s.copied[s.last_side], s.done) == cudaSuccess) {
            r.result.ms = ms;
            st.lat_ms.push_back(ms);
        } else {
            cudaGetLastError();
        }
        st.ready.push_back(r);
        st.joined += 2 * st.W;
        s.state = 0;
        s.filled[0] = s.filled[1] = false;
        st.harvested++;
    }
    return SJBG_OK;
}

// Enqueue the join of the window in slot s (both sides copied).
static int ring_launch(sjbg_handle *h, RingState &st, RingSlot &s) {
    SJBG_CK(h, cudaStreamWaitEvent(h->stream, s.copied[0], 0));
    SJBG_CK(h, cudaStreamWaitEvent(h->stream, s.copied[1], 0));
    const uint64_t off = (s.id % st.depth) * st.W;
    for (int i = 0; i < 6; i++) std::swap(h->pinned[i], s.pinned[i]);
    WinHost wh{0, st.W, 0, st.W, 0, 0};
    WinAcc *hacc = static_cast<WinAcc *>(pinned_get(h, 3, 2 * sizeof(WinAcc)));   // window + status word
    int rc = hacc ? run_lazy_device(h, st.buf[0] + off, st.buf[1] + off, &wh, 1, nullptr, hacc, &s.part_used)
                  : fail(h, SJBG_E_NOMEM, "window staging");
    for (int i = 0; i < 6; i++) std::swap(h->pinned[i], s.pinned[i]);
    if (rc) return rc;
    SJBG_CK(h, cudaEventRecord(s.done, h->stream));
    s.state = 1;
    st.launched++;
    return SJBG_OK;
}

}  // namespace sjbg

using namespace sjbg;

extern "C" {

int sjbg_ring_open(sjbg_handle *h, uint64_t window_tuples, uint32_t depth) {
    if (!h) return SJBG_E_INVALID;
    if (h->cfg.progressiveness != SJBG_LAZY) return fail(h, SJBG_E_STATE, "the ingest ring needs a lazy handle");
    if (window_tuples == 0 || depth < 2) return fail(h, SJBG_E_INVALID, "ring: window_tuples > 0 and depth >= 2");
    if (window_tuples > h->cfg.max_tuples_per_window)
        return fail(h, SJBG_E_CAPACITY, "ring: window larger than max_tuples_per_window");
    SJBG_CK(h, cudaSetDevice(h->device));
    h->ring.reset();
    auto st = std::make_unique<RingState>();
    st->W = window_tuples;
    st->depth = depth;
    const size_t bytes = sizeof(sjbg_tuple) * window_tuples * depth;
    for (int s = 0; s < 2; s++) {
        void *p = nullptr;
        if (cudaMalloc(&p, bytes) != cudaSuccess) {
            cudaGetLastError();
            return fail(h, SJBG_E_NOMEM, "ring buffers");
        }
        st->buf[s] = static_cast<sjbg_tuple *>(p);
    }
    SJBG_CK(h, cudaStreamCreateWithFlags(&st->copy, cudaStreamNonBlocking));
    st->slots.resize(depth);
    for (auto &s : st->slots) {
        SJBG_CK(h, cudaEventCreate(&s.copied[0]));
        SJBG_CK(h, cudaEventCreate(&s.copied[1]));
        SJBG_CK(h, cudaEventCreate(&s.done));
    }
    h->ring.reset(st.release());
    return SJBG_OK;
}

int sjbg_ring_push(sjbg_handle *h, const sjbg_tuple *batch, uint64_t n, int is_left, uint32_t mem) {
    if (!h) return SJBG_E_INVALID;
    RingState *st = rs(h);
    if (!st) return fail(h, SJBG_E_STATE, "ring not open");
    if (n == 0) return SJBG_OK;
    if (!batch || (mem != SJBG_MEM_HOST && mem != SJBG_MEM_DEVICE)) return fail(h, SJBG_E_INVALID, "bad batch");
    SJBG_CK(h, cudaSetDevice(h->device));
    const int side = is_left ? 0 : 1;
    // the window the batch's last tuple lands in must have a slot: the slot's
    // previous window must be joined already (else this side is too far ahead)
    const uint64_t last_win = (st->pushed[side] + n - 1) / st->W;
    if (last_win >= st->harvested + st->depth) {
        if (int rc = ring_harvest(h, *st, false)) return rc;
        while (last_win >= st->harvested + st->depth && st->harvested < st->launched)
            if (int rc = ring_harvest(h, *st, true)) return rc;
        if (last_win >= st->harvested + st->depth)
            return fail(h, SJBG_E_CAPACITY, "Ring buffer is full: one side is a whole ring of windows ahead");
    }
    const cudaMemcpyKind kind = mem == SJBG_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    uint64_t done = 0;
    while (done < n) {
        const uint64_t k = st->pushed[side] / st->W, off = st->pushed[side] % st->W;
        const uint64_t take = std::min(n - done, st->W - off);
        RingSlot &s = st->slots[k % st->depth];
        if (off == 0) s.id = k;
        SJBG_CK(h, cudaMemcpyAsync(st->buf[side] + (k % st->depth) * st->W + off, batch + done,
                                   sizeof(sjbg_tuple) * take, kind, st->copy));
        st->pushed[side] += take;
        done += take;
        if (off + take == st->W) {   // this side of window k is complete
            SJBG_CK(h, cudaEventRecord(s.copied[side], st->copy));
            s.filled[side] = true;
            s.last_side = side;
            if (s.filled[0] && s.filled[1])
                if (int rc = ring_launch(h, *st, s)) return rc;
        }
    }
    return ring_harvest(h, *st, false);
}

int sjbg_ring_poll(sjbg_handle *h, sjbg_stream_window *out, uint32_t max_out, uint32_t *n_out) {
    if (!h || !n_out || (max_out && !out)) return SJBG_E_INVALID;
    RingState *st = rs(h);
    if (!st) return fail(h, SJBG_E_STATE, "ring not open");
    if (int rc = ring_harvest(h, *st, false)) return rc;
    uint32_t k = 0;
    while (k < max_out && !st->ready.empty()) {
        out[k++] = st->ready.front();
        st->ready.pop_front();
    }
    *n_out = k;
    return SJBG_OK;
}

int sjbg_ring_close(sjbg_handle *h, sjbg_stream_stats *stats) {
    if (!h) return SJBG_E_INVALID;
    RingState *st = rs(h);
    if (!st) return fail(h, SJBG_E_STATE, "ring not open");
    if (int rc = ring_harvest(h, *st, true)) return rc;
    SJBG_CK(h, cudaStreamSynchronize(st->copy));
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->windows_closed = st->launched;
        stats->tuples_joined = st->joined;
        stats->fallbacks = st->fallbacks;
        std::vector<double> v = st->lat_ms;
        std::sort(v.begin(), v.end());
        if (!v.empty()) {
            stats->p50_ms = v[v.size() / 2];
            stats->p99_ms = v[std::min(v.size() - 1, (size_t)(0.99 * v.size()))];
            for (double x : v) stats->busy_ms += x;
        }
    }
    return SJBG_OK;
}

}  // extern "C"
