// gi_parallel.h - a parallel loop over the host's cores for the host steps of the library.
#pragma once

#include <algorithm>
#include <atomic>
#include <cstddef>
#include <thread>
#include <vector>

namespace gz {

// Runs fn(i) for every i in [0, n) on up to 16 host threads (the caller's included), in slices
// taken from a shared counter; with fewer than `per_thread` items a thread it runs on the caller
// alone. fn must not throw, and calls for different i must not write the same data.
template <class F>
void parallel_for(size_t n, size_t per_thread, F&& fn) {
    static const size_t hw = std::max<size_t>(1, std::min<size_t>(16, std::thread::hardware_concurrency()));
    const size_t nt = std::min(hw, n / std::max<size_t>(1, per_thread));
    if (nt <= 1) {
        for (size_t i = 0; i < n; i++) fn(i);
        return;
    }
    std::atomic<size_t> next{0};
    const size_t slice = std::max<size_t>(1, n / (nt * 16));
    auto work = [&] {
        for (;;) {
            const size_t a = next.fetch_add(slice);
            if (a >= n) return;
            const size_t b = std::min(n, a + slice);
            for (size_t i = a; i < b; i++) fn(i);
        }
    };
    std::vector<std::thread> th;
    th.reserve(nt - 1);
    for (size_t t = 1; t < nt; t++) th.emplace_back(work);
    work();
    for (std::thread& t : th) t.join();
}

}  // namespace gz
