// Minimal TBB-API shim (test infrastructure of the oracle only).
//
// oneTBB is not installed in this image and there is no network, so the
// reference's CPU joiners are compiled against this header set instead.  It
// provides only the names those sources use - task_arena, parallel_for,
// parallel_for_each, parallel_sort, parallel_invoke, blocked_range,
// concurrent_vector - implemented with std::thread.  The concurrency of the
// enclosing task_arena is honoured, as the reference relies on it to set
// nProbeThreads / nSortThreads (src/sjb/windowing/lazy/executor/CPU/CPU_HJ.cpp:54,
// CPU_SMJ.cpp:88).
#pragma once
#include <algorithm>
#include <cstddef>
#include <deque>
#include <functional>
#include <iterator>
#include <mutex>
#include <thread>
#include <utility>
#include <vector>

namespace tbb {
namespace shim {
inline int &arena_concurrency() {
    static thread_local int c = 0;
    return c;
}
inline int current_concurrency() {
    int c = arena_concurrency();
    if (c > 0) return c;
    unsigned h = std::thread::hardware_concurrency();
    return h ? (int)h : 1;
}
// Run body(begin_index, end_index) over [0, n) split into `threads` contiguous chunks.
template <class Body>
void run_chunks(std::size_t n, int threads, Body body) {
    if (threads < 1) threads = 1;
    if ((std::size_t)threads > n) threads = n ? (int)n : 1;
    if (threads == 1) { body((std::size_t)0, n); return; }
    int inherited = arena_concurrency();
    std::vector<std::thread> pool;
    pool.reserve(threads);
    for (int t = 0; t < threads; t++) {
        std::size_t b = n * t / threads, e = n * (t + 1) / threads;
        pool.emplace_back([=, &body]() { arena_concurrency() = 1; (void)inherited; body(b, e); });
    }
    for (auto &th : pool) th.join();
}
}  // namespace shim

class task_arena {
public:
    enum class priority { low, normal, high };
    explicit task_arena(int max_concurrency = -1, unsigned reserved_for_masters = 1,
                        priority p = priority::normal)
        : conc_(max_concurrency) { (void)reserved_for_masters; (void)p; }
    template <class F>
    auto execute(F &&f) -> decltype(f()) {
        int saved = shim::arena_concurrency();
        shim::arena_concurrency() = conc_ > 0 ? conc_ : shim::current_concurrency();
        struct restore { int v; ~restore() { shim::arena_concurrency() = v; } } r{saved};
        return f();
    }
    int max_concurrency() const { return conc_ > 0 ? conc_ : shim::current_concurrency(); }
private:
    int conc_;
};

template <class Value>
class blocked_range {
public:
    blocked_range(Value b, Value e, std::size_t grain = 1) : b_(b), e_(e) { (void)grain; }
    Value begin() const { return b_; }
    Value end() const { return e_; }
    std::size_t size() const { return (std::size_t)(e_ - b_); }
    bool empty() const { return !(b_ < e_); }
private:
    Value b_, e_;
};

template <class Value, class Body>
void parallel_for(const blocked_range<Value> &range, const Body &body) {
    std::size_t n = range.size();
    Value base = range.begin();
    shim::run_chunks(n, shim::current_concurrency(), [&](std::size_t b, std::size_t e) {
        body(blocked_range<Value>(base + (Value)b, base + (Value)e));
    });
}

template <class It, class F>
void parallel_for_each(It first, It last, const F &f) {
    std::vector<It> items;
    for (It it = first; it != last; ++it) items.push_back(it);
    shim::run_chunks(items.size(), shim::current_concurrency(), [&](std::size_t b, std::size_t e) {
        for (std::size_t i = b; i < e; i++) f(*items[i]);
    });
}

template <class RandomIt, class Compare>
void parallel_sort(RandomIt first, RandomIt last, const Compare &comp) {
    std::size_t n = (std::size_t)(last - first);
    int threads = shim::current_concurrency();
    if (threads <= 1 || n < 4096) { std::sort(first, last, comp); return; }
    std::vector<std::size_t> bounds(threads + 1);
    for (int t = 0; t <= threads; t++) bounds[t] = n * t / threads;
    shim::run_chunks((std::size_t)threads, threads, [&](std::size_t b, std::size_t e) {
        for (std::size_t t = b; t < e; t++) std::sort(first + bounds[t], first + bounds[t + 1], comp);
    });
    for (int width = 1; width < threads; width *= 2) {
        std::size_t merges = (threads + 2 * width - 1) / (2 * width);
        shim::run_chunks(merges, threads, [&](std::size_t b, std::size_t e) {
            for (std::size_t m = b; m < e; m++) {
                int p0 = (int)m * 2 * width, p1 = std::min(p0 + width, threads), p2 = std::min(p0 + 2 * width, threads);
                std::inplace_merge(first + bounds[p0], first + bounds[p1], first + bounds[p2], comp);
            }
        });
    }
}

template <class RandomIt>
void parallel_sort(RandomIt first, RandomIt last) {
    parallel_sort(first, last, std::less<typename std::iterator_traits<RandomIt>::value_type>());
}

template <class... F>
void parallel_invoke(const F &...fs) {
    std::vector<std::thread> pool;
    (pool.emplace_back([&fs]() { fs(); }), ...);
    for (auto &t : pool) t.join();
}

template <class T>
class concurrent_vector {
public:
    using iterator = typename std::deque<T>::iterator;
    using const_iterator = typename std::deque<T>::const_iterator;
    concurrent_vector() = default;
    concurrent_vector(const concurrent_vector &o) : d_(o.d_) {}
    concurrent_vector &operator=(const concurrent_vector &o) { d_ = o.d_; return *this; }
    iterator push_back(const T &v) { std::lock_guard<std::mutex> g(m_); d_.push_back(v); return std::prev(d_.end()); }
    template <class... A>
    iterator emplace_back(A &&...a) { std::lock_guard<std::mutex> g(m_); d_.emplace_back(std::forward<A>(a)...); return std::prev(d_.end()); }
    iterator begin() { return d_.begin(); }
    iterator end() { return d_.end(); }
    const_iterator begin() const { return d_.begin(); }
    const_iterator end() const { return d_.end(); }
    std::size_t size() const { return d_.size(); }
    T &operator[](std::size_t i) { return d_[i]; }
    void clear() { d_.clear(); }
private:
    std::deque<T> d_;
    std::mutex m_;
};
}  // namespace tbb
