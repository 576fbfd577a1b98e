// Host helpers of the graph preparation: a chunked parallel loop on the host's threads and the
// locality order (recursive BFS bisection) of batched runs on large graphs.  Plain C++ (no CUDA),
// so the order can be tested on its own.
#pragma once
#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <memory>
#include <mutex>
#include <system_error>
#include <thread>
#include <utility>
#include <vector>

namespace fbc_host {

// fn(lo, hi) over [0, count) in contiguous chunks on the host's threads (one chunk when small).
template <class F>
void host_parallel(int64_t count, F&& fn) {
    const int nthr = (int)std::min<unsigned>(std::max(1u, std::thread::hardware_concurrency()), 32u);
    if (nthr <= 1 || count < 65536) {
        fn((int64_t)0, count);
        return;
    }
    const int64_t chunk = (count + nthr - 1) / nthr;
    std::vector<std::thread> th;
    for (int i = 0; i < nthr; ++i) {
        const int64_t lo = (int64_t)i * chunk, hi = std::min<int64_t>(count, lo + chunk);
        if (lo >= hi) break;
        try {
            th.emplace_back([&fn, lo, hi] { fn(lo, hi); });
        } catch (const std::system_error&) {  // no thread to be had: this chunk here
            fn(lo, hi);
        }
    }
    for (auto& x : th) x.join();
}

// Recursive BFS bisection: a part (a range of `ord`) is laid out in the order of a BFS from its
// first vertex that stays inside the part (vertices it cannot reach follow in their current
// order), then halved; parts of at most `leaf` vertices are sorted by id.  Neighbours end up
// close together at every scale, so a wavefront's vertices share sectors and DRAM pages.
inline std::vector<int32_t> bisection_order(int32_t n, const std::vector<int64_t>& rp, const std::vector<int32_t>& col,
                                     int leaf) {
    std::vector<int32_t> ord((size_t)n), tmp((size_t)n);
    std::unique_ptr<std::atomic<int32_t>[]> part(new std::atomic<int32_t>[(size_t)std::max(n, 1)]);
    std::vector<char> vis((size_t)n, 0);
    for (int32_t i = 0; i < n; ++i) {
        ord[i] = i;
        part[i].store(0, std::memory_order_relaxed);
    }
    std::atomic<int32_t> pid{1};
    // One range [lo, hi) of the current order: lay it out in BFS order (from each not yet reached
    // vertex in turn, edges followed only inside the range), or sort a leaf.  Ranges processed at
    // the same time are disjoint, so they touch disjoint vertices; a neighbour outside the range
    // carries another range's id (ids are never reused), read and written atomically.
    auto split = [&](int64_t lo, int64_t hi) -> bool {
        const int64_t len = hi - lo;
        if (len <= leaf) {
            std::sort(ord.begin() + lo, ord.begin() + hi);
            return false;
        }
        const int32_t me = pid.fetch_add(1, std::memory_order_relaxed);
        for (int64_t i = lo; i < hi; ++i) part[ord[i]].store(me, std::memory_order_relaxed);
        int64_t qt = lo;
        for (int64_t i = lo; i < hi; ++i) {
            const int32_t s0 = ord[i];
            if (vis[s0]) continue;
            int64_t qh = qt;
            tmp[qt++] = s0;
            vis[s0] = 1;
            while (qh < qt) {
                const int32_t v = tmp[qh++];
                for (int64_t e = rp[v]; e < rp[v + 1]; ++e) {
                    const int32_t x = col[e];
                    if (part[x].load(std::memory_order_relaxed) == me && !vis[x]) {
                        vis[x] = 1;
                        tmp[qt++] = x;
                    }
                }
            }
        }
        for (int64_t i = lo; i < hi; ++i) {
            ord[i] = tmp[i];
            vis[tmp[i]] = 0;
        }
        return true;
    };
    // a range and everything below it, in this thread
    auto serial = [&](int64_t lo0, int64_t hi0) {
        std::vector<std::pair<int64_t, int64_t>> stk{{lo0, hi0}};
        while (!stk.empty()) {
            const auto [lo, hi] = stk.back();
            stk.pop_back();
            if (!split(lo, hi)) continue;
            const int64_t mid = lo + (hi - lo) / 2;
            stk.emplace_back(mid, hi);
            stk.emplace_back(lo, mid);
        }
    };
    // the top of the tree on a pool of host threads (the result does not depend on their number
    // or timing: each range's layout depends only on its own order and the graph)
    const int nthr = (int)std::min<unsigned>(std::max(1u, std::thread::hardware_concurrency()), 32u);
    constexpr int64_t kSerial = 65536;
    if (nthr <= 1 || n <= kSerial) {
        serial(0, n);
    } else {
        std::mutex mu;
        std::condition_variable cv;
        std::vector<std::pair<int64_t, int64_t>> q{{0, (int64_t)n}};
        int64_t pending = 1;  // ranges queued or in progress
        auto work = [&]() {
            for (;;) {
                std::pair<int64_t, int64_t> r;
                {
                    std::unique_lock<std::mutex> lk(mu);
                    cv.wait(lk, [&] { return !q.empty() || pending == 0; });
                    if (q.empty()) return;  // pending == 0: everything is done
                    r = q.back();
                    q.pop_back();
                }
                bool done_here = true;
                if (r.second - r.first <= kSerial) {
                    serial(r.first, r.second);
                } else if (split(r.first, r.second)) {
                    const int64_t mid = r.first + (r.second - r.first) / 2;
                    std::lock_guard<std::mutex> lk(mu);
                    q.emplace_back(mid, r.second);
                    q.emplace_back(r.first, mid);
                    pending += 2;
                    done_here = false;
                }
                std::lock_guard<std::mutex> lk(mu);
                --pending;
                if (!done_here) cv.notify_all();
                else if (pending == 0) cv.notify_all();
            }
        };
        std::vector<std::thread> th;
        try {
            for (int i = 0; i < nthr; ++i) th.emplace_back(work);
        } catch (const std::system_error&) {  // fewer threads than asked: the ones running finish
        }
        if (th.empty()) work();
        for (auto& x : th) x.join();
    }
    std::vector<int32_t> nw((size_t)n);
    for (int32_t i = 0; i < n; ++i) nw[ord[i]] = i;
    return nw;
}

}  // namespace fbc_host
