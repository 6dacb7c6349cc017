// stream.cu - event-time streaming loop (sm_103a host runtime).
//
// No compiled reference counterpart: the reference's event-time windowing
// (src/sjb/windowing/lazy/TimeBased.cu:18-183) is not built and depends on
// undefined macros; its idea - a window closes when the watermark passes its
// end (TimeBased.cu:56-57,110-119) - is kept:
//   * tuple t belongs to window floor(t.ts / window_ns); both sides' tuples of
//     a window are appended, in arrival order, to device buffers that come
//     from a stream-ordered memory pool whose memory stays resident;
//   * the watermark is min over the two sides of the largest pushed event
//     time; every window that ends at or before it is closed and its join
//     (the handle's lazy algorithm, e.g. the learned-partitioned hash join,
//     refitted on each window's own sample) is enqueued asynchronously with
//     private pinned staging, so ingest continues while it runs;
//   * admission: before a window's buffers grow past the HBM budget, the
//     loop waits for joins in flight to finish and release theirs; if that
//     is not enough the window is rejected (result status SJBG_E_BUDGET);
//   * latency of a window = device time from its close (an event on an idle
//     side stream) to the end of its join, so queueing behind earlier windows
//     is included.
#include <algorithm>
#include <cstring>

#include "stream.cuh"

namespace sjbg {

StreamState::~StreamState() {
    for (StreamWin *w : wins) {
        for (int s = 0; s < 2; s++)
            if (w->buf[s]) cudaFree(w->buf[s]);
        spare.push_back(w);
    }
    for (StreamWin *w : spare) {
        if (w->ev_close) cudaEventDestroy(w->ev_close);
        if (w->ev_done) cudaEventDestroy(w->ev_done);
        for (auto &b : w->pinned)
            if (b.p) cudaFreeHost(b.p);
        delete w;
    }
    if (d_bounds) cudaFree(d_bounds);
    if (h_bounds) cudaFreeHost(h_bounds);
}

constexpr uint32_t kMaxBounds = 1024;   // window boundaries one push may cross

// lower bound of each boundary b_k = (first_window + 1 + k) * W in the ts of a device batch
__global__ void stream_bounds_kernel(const sjbg_tuple *__restrict__ batch, uint64_t n, uint64_t first_window,
                                     uint64_t W, uint32_t nb, uint64_t *__restrict__ out) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nb) return;
    const uint64_t bound = (first_window + 1 + k) * W;
    uint64_t lo = 0, hi = n;
    while (lo < hi) {
        const uint64_t mid = (lo + hi) >> 1;
        if (batch[mid].ts < bound) lo = mid + 1; else hi = mid;
    }
    out[k] = lo;
}

static StreamState *ss(sjbg_handle *h) { return h->streaming.get(); }

static StreamWin *new_win(StreamState &st, uint64_t id) {
    StreamWin *w;
    if (!st.spare.empty()) {
        w = st.spare.back();
        st.spare.pop_back();
    } else {
        w = new StreamWin();
        cudaEventCreate(&w->ev_close);
        cudaEventCreate(&w->ev_done);
    }
    w->id = id;
    w->buf[0] = w->buf[1] = nullptr;
    w->n[0] = w->n[1] = w->cap[0] = w->cap[1] = 0;
    w->state = 0;
    w->part_used = 0;
    return w;
}

static void release_buffers(sjbg_handle *h, StreamState &st, StreamWin *w) {
    for (int s = 0; s < 2; s++) {
        if (w->buf[s]) cudaFreeAsync(w->buf[s], h->stream);
        st.used -= sizeof(sjbg_tuple) * w->cap[s];
        w->buf[s] = nullptr;
        w->cap[s] = 0;
    }
}

// Move finished windows (in id order) to the ready queue; wait for them if asked.
static void harvest(sjbg_handle *h, StreamState &st, bool wait) {
    while (!st.wins.empty()) {
        StreamWin *w = st.wins.front();
        if (w->state == 0 || w->state == 2) break;   // still open
        sjbg_window_result r;
        std::memset(&r, 0, sizeof(r));
        if (w->state == 1) {
            if (wait) cudaEventSynchronize(w->ev_done);
            else if (cudaEventQuery(w->ev_done) != cudaSuccess) {
                cudaGetLastError();
                break;
            }
            float lat = 0.f, busy = 0.f;
            cudaEventElapsedTime(&lat, w->ev_close, w->ev_done);
            const WinAcc &a = *static_cast<const WinAcc *>(w->pinned[3].p);
            const unsigned long long bits = static_cast<const WinAcc *>(w->pinned[3].p)[1].info;
            if (bits) r.status = bits & kErrTimeout ? SJBG_E_TIMEOUT : SJBG_E_CAPACITY;
            r.count = a.count;
            r.prod_checksum = a.prod;
            r.partitioner_used = w->part_used;
            if (w->part_used == SJBG_PART_LEARNED && (a.info & (kInfoFallback | kInfoRadixByCost))) {
                r.partitioner_used = SJBG_PART_RADIX;
                if (a.info & kInfoFallback) {
                    r.flags |= SJBG_WR_FALLBACK;
                    st.fallbacks++;
                } else {
                    r.flags |= SJBG_WR_RADIX_BY_COST;
                }
            }
            r.ms = lat;
            (void)busy;
            st.lat_ms.push_back(lat);
            st.joined += w->n[0] + w->n[1];
        } else {
            r.status = SJBG_E_BUDGET;
            st.rejected++;
        }
        sjbg_stream_window sw;
        sw.result = r;
        sw.window_id = w->id;
        sw.n_left = w->n[0];
        sw.n_right = w->n[1];
        st.ready.push_back(sw);
        release_buffers(h, st, w);
        st.wins.pop_front();
        st.spare.push_back(w);
    }
}

static int launch_join(sjbg_handle *h, StreamState &st, StreamWin *w, cudaStream_t side) {
    st.closed++;
    st.any_closed = true;
    st.last_closed_id = w->id;
    if (w->state == 2) {   // rejected: nothing to join, its result reports the refusal
        w->state = 3;
        return SJBG_OK;
    }
    // close marker on an idle stream: the window's latency includes queueing
    SJBG_CK(h, cudaEventRecord(w->ev_close, side));
    SJBG_CK(h, cudaStreamWaitEvent(h->stream, w->ev_close, 0));
    for (int i = 0; i < 6; i++) std::swap(h->pinned[i], w->pinned[i]);
    WinHost wh{0, w->n[0], 0, w->n[1], 0, 0};
    WinAcc *hacc = static_cast<WinAcc *>(pinned_get(h, 3, 2 * sizeof(WinAcc)));   // window + status
    int rc = hacc ? run_lazy_device(h, w->buf[0] ? w->buf[0] : nullptr, w->buf[1] ? w->buf[1] : nullptr, &wh, 1,
                                    nullptr, hacc, &w->part_used)
                  : fail(h, SJBG_E_NOMEM, "window staging");
    for (int i = 0; i < 6; i++) std::swap(h->pinned[i], w->pinned[i]);
    if (rc) return rc;
    SJBG_CK(h, cudaEventRecord(w->ev_done, h->stream));
    w->state = 1;
    return SJBG_OK;
}

static int close_ready(sjbg_handle *h, StreamState &st, cudaStream_t side, bool all) {
    const uint64_t wm = std::min(st.seen[0] ? st.wm[0] : 0, st.seen[1] ? st.wm[1] : 0);
    for (StreamWin *w : st.wins) {
        if (w->state != 0 && w->state != 2) continue;
        const uint64_t end = (w->id + 1) * st.window_ns;
        if (!all && !(st.seen[0] && st.seen[1] && end <= wm)) break;
        int rc = launch_join(h, st, w, side);
        if (rc) return rc;
    }
    return SJBG_OK;
}

// Find or admit window id (ids only grow; data for a closed window is late).
static StreamWin *get_win(StreamState &st, uint64_t id, bool *late) {
    *late = st.any_closed && id <= st.last_closed_id;
    if (*late) return nullptr;
    for (StreamWin *w : st.wins)
        if (w->id == id) return w;
    StreamWin *w = new_win(st, id);
    auto it = st.wins.begin();
    while (it != st.wins.end() && (*it)->id < id) ++it;
    st.wins.insert(it, w);
    return w;
}

// Make room for `need` more tuples on one side of window w, inside the budget.
static int reserve(sjbg_handle *h, StreamState &st, StreamWin *w, int side, uint64_t need) {
    if (w->n[side] + need <= w->cap[side]) return SJBG_OK;
    const uint64_t ncap = std::max<uint64_t>({2 * w->cap[side], w->n[side] + need, 1ull << 20});
    const uint64_t add = sizeof(sjbg_tuple) * (ncap - w->cap[side]);
    if (st.budget && st.used + add > st.budget) {
        SJBG_CK(h, cudaStreamSynchronize(h->stream));   // backpressure: let joins in flight finish
        harvest(h, st, true);
        if (st.used + add > st.budget) return SJBG_E_BUDGET;
    }
    void *nb = nullptr;
    SJBG_CK(h, cudaMallocFromPoolAsync(&nb, sizeof(sjbg_tuple) * ncap, st.pool, h->stream));
    if (w->n[side])
        SJBG_CK(h, cudaMemcpyAsync(nb, w->buf[side], sizeof(sjbg_tuple) * w->n[side], cudaMemcpyDeviceToDevice,
                                   h->stream));
    if (w->buf[side]) SJBG_CK(h, cudaFreeAsync(w->buf[side], h->stream));
    st.used += add;
    w->buf[side] = static_cast<sjbg_tuple *>(nb);
    w->cap[side] = ncap;
    return SJBG_OK;
}

static cudaStream_t side_stream(sjbg_handle *h) {
    static thread_local cudaStream_t s = nullptr;
    static thread_local int dev = -1;
    if (!s || dev != h->device) {
        cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        dev = h->device;
    }
    return s;
}

}  // namespace sjbg

using namespace sjbg;

extern "C" {

int sjbg_stream_open(sjbg_handle *h, uint64_t window_ns) {
    if (!h) return SJBG_E_INVALID;
    if (h->cfg.progressiveness != SJBG_LAZY) return fail(h, SJBG_E_STATE, "streaming needs a lazy handle");
    if (window_ns == 0) return fail(h, SJBG_E_INVALID, "window length must be > 0");
    SJBG_CK(h, cudaSetDevice(h->device));
    if (h->streaming) {
        SJBG_CK(h, cudaStreamSynchronize(h->stream));
        h->streaming.reset();
    }
    auto st = std::make_unique<StreamState>();
    st->window_ns = window_ns;
    st->budget = h->cfg.hbm_budget_bytes;
    SJBG_CK(h, cudaDeviceGetDefaultMemPool(&st->pool, h->device));
    uint64_t keep = UINT64_MAX;   // freed window buffers stay in the pool (resident)
    SJBG_CK(h, cudaMemPoolSetAttribute(st->pool, cudaMemPoolAttrReleaseThreshold, &keep));
    SJBG_CK(h, cudaMalloc(&st->d_bounds, sizeof(uint64_t) * kMaxBounds));
    SJBG_CK(h, cudaMallocHost(&st->h_bounds, sizeof(uint64_t) * (kMaxBounds + 2)));
    h->streaming = std::move(st);
    return SJBG_OK;
}

int sjbg_stream_push(sjbg_handle *h, const sjbg_tuple *batch, uint64_t n, int is_left, uint32_t mem) {
    if (!h) return SJBG_E_INVALID;
    StreamState *st = ss(h);
    if (!st) return fail(h, SJBG_E_STATE, "stream not open");
    if (n == 0) return SJBG_OK;
    if (!batch || (mem != SJBG_MEM_HOST && mem != SJBG_MEM_DEVICE)) return fail(h, SJBG_E_INVALID, "bad batch");
    SJBG_CK(h, cudaSetDevice(h->device));
    const int side = is_left ? 0 : 1;
    const uint64_t W = st->window_ns;
    // split the batch at window boundaries (event times are non-decreasing)
    uint64_t first_ts, last_ts;
    std::vector<uint64_t> cut;   // start offsets of the segments, then n
    if (mem == SJBG_MEM_HOST) {
        first_ts = batch[0].ts;
        last_ts = batch[n - 1].ts;
        cut.push_back(0);
        for (uint64_t wid = first_ts / W + 1; wid <= last_ts / W; wid++) {
            uint64_t lo = cut.back(), hi = n;
            while (lo < hi) {
                const uint64_t mid = (lo + hi) >> 1;
                if (batch[mid].ts < wid * W) lo = mid + 1; else hi = mid;
            }
            cut.push_back(lo);
        }
    } else {
        SJBG_CK(h, cudaMemcpyAsync(st->h_bounds, &batch[0].ts, 8, cudaMemcpyDeviceToHost, h->stream));
        SJBG_CK(h, cudaMemcpyAsync(st->h_bounds + 1, &batch[n - 1].ts, 8, cudaMemcpyDeviceToHost, h->stream));
        SJBG_CK(h, cudaStreamSynchronize(h->stream));
        first_ts = st->h_bounds[0];
        last_ts = st->h_bounds[1];
        cut.push_back(0);
        const uint64_t nb = last_ts / W - first_ts / W;
        if (nb > kMaxBounds) return fail(h, SJBG_E_INVALID, "a device batch may cross at most 1024 windows");
        if (nb) {
            SJBG_CK(h, launch(h, "stream_bounds", stream_bounds_kernel, dim3((uint32_t)((nb + 255) / 256)), dim3(256),
                              0, batch, n, first_ts / W, W, (uint32_t)nb, st->d_bounds));
            SJBG_CK(h, cudaMemcpyAsync(st->h_bounds, st->d_bounds, 8 * nb, cudaMemcpyDeviceToHost, h->stream));
            SJBG_CK(h, cudaStreamSynchronize(h->stream));
            for (uint64_t k = 0; k < nb; k++) cut.push_back(st->h_bounds[k]);
        }
    }
    if (st->seen[side] && first_ts < st->wm[side]) return fail(h, SJBG_E_INVALID, "event time went backwards");
    if (last_ts < first_ts) return fail(h, SJBG_E_INVALID, "event times in a batch must not decrease");
    cut.push_back(n);
    for (size_t k = 0; k + 1 < cut.size(); k++) {
        const uint64_t a = cut[k], b = cut[k + 1];
        if (a == b) continue;
        const uint64_t wid = first_ts / W + k;
        bool late = false;
        StreamWin *w = get_win(*st, wid, &late);
        if (late || !w || w->state == 2) continue;   // late data of a closed window is dropped
        int rc = reserve(h, *st, w, side, b - a);
        if (rc == SJBG_E_BUDGET) {   // reject the whole window
            w->state = 2;
            release_buffers(h, *st, w);
            continue;
        }
        if (rc) return rc;
        SJBG_CK(h, cudaMemcpyAsync(w->buf[side] + w->n[side], batch + a, sizeof(sjbg_tuple) * (b - a),
                                   mem == SJBG_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                                   h->stream));
        w->n[side] += b - a;
    }
    st->wm[side] = last_ts;
    st->seen[side] = true;
    int rc = close_ready(h, *st, side_stream(h), false);
    if (rc) return rc;
    harvest(h, *st, false);
    return SJBG_OK;
}

int sjbg_stream_poll(sjbg_handle *h, sjbg_stream_window *out, uint32_t max_out, uint32_t *n_out) {
    if (!h || !n_out || (max_out && !out)) return SJBG_E_INVALID;
    StreamState *st = ss(h);
    if (!st) return fail(h, SJBG_E_STATE, "stream not open");
    harvest(h, *st, false);
    uint32_t k = 0;
    while (k < max_out && !st->ready.empty()) {
        out[k++] = st->ready.front();
        st->ready.pop_front();
    }
    *n_out = k;
    return SJBG_OK;
}

int sjbg_stream_close(sjbg_handle *h, sjbg_stream_stats *stats) {
    if (!h) return SJBG_E_INVALID;
    StreamState *st = ss(h);
    if (!st) return fail(h, SJBG_E_STATE, "stream not open");
    int rc = close_ready(h, *st, side_stream(h), true);
    if (rc) return rc;
    SJBG_CK(h, cudaStreamSynchronize(h->stream));
    harvest(h, *st, true);
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->windows_closed = st->closed;
        stats->tuples_joined = st->joined;
        stats->windows_rejected = st->rejected;
        stats->fallbacks = st->fallbacks;
        std::vector<double> v = st->lat_ms;
        std::sort(v.begin(), v.end());
        if (!v.empty()) {
            stats->p50_ms = v[v.size() / 2];
            stats->p99_ms = v[std::min(v.size() - 1, (size_t)(0.99 * (double)v.size()))];
        }
        double busy = 0;
        for (double x : st->lat_ms) busy += x;
        stats->busy_ms = busy;
    }
    return SJBG_OK;
}

}  // extern "C"
