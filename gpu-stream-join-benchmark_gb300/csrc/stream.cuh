// stream.cuh - event-time streaming loop: state.
#pragma once

#include <deque>
#include <vector>

#include "runtime.h"

namespace sjbg {

// One event-time tumbling window: its tuples of both sides (device memory,
// arrival order), and, once closed, the join in flight.
struct StreamWin {
    uint64_t id = 0;
    sjbg_tuple *buf[2] = {nullptr, nullptr};
    uint64_t n[2] = {0, 0}, cap[2] = {0, 0};
    int state = 0;               // 0 open, 1 join enqueued, 2 rejected (still open), 3 rejected and closed
    cudaEvent_t ev_close = nullptr, ev_done = nullptr;
    DevBuf pinned[6];            // private staging of this window's join
    uint32_t part_used = 0;
};

struct StreamState {
    uint64_t window_ns = 0;
    uint64_t wm[2] = {0, 0};     // largest event time pushed per side
    bool seen[2] = {false, false};
    uint64_t budget = 0;         // bytes; 0 = unlimited
    uint64_t used = 0;           // bytes held by window buffers
    std::deque<StreamWin *> wins;      // open and in-flight windows, by id
    std::vector<StreamWin *> spare;    // recycled window records
    std::deque<sjbg_stream_window> ready;
    std::vector<double> lat_ms;
    uint64_t closed = 0, rejected = 0, joined = 0, fallbacks = 0, last_closed_id = 0;
    bool any_closed = false;
    double busy_ms = 0.0;
    uint64_t *d_bounds = nullptr;      // device boundary search scratch
    uint64_t *h_bounds = nullptr;      // pinned
    cudaMemPool_t pool = nullptr;
    ~StreamState();
};

}  // namespace sjbg
