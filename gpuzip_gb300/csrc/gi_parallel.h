// gi_parallel.h - a parallel loop over the host's cores for the host steps of the library.
#pragma once

#include <algorithm>
#include <atomic>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <thread>
#include <vector>

namespace gz {

// Host threads a parallel loop may use: GI_HOST_THREADS when set (1 keeps every loop on the calling
// thread), else the host's cores, at most 16.
inline size_t host_threads() {
    static const size_t n = [] {
        const char* e = std::getenv("GI_HOST_THREADS");
        const long v = e ? std::atol(e) : 0;
        if (v > 0) return (size_t)std::min<long>(v, 64);
        return std::max<size_t>(1, std::min<size_t>(16, std::thread::hardware_concurrency()));
    }();
    return n;
}

// Runs fn(i) for every i in [0, n) on up to host_threads() threads (the caller's included), in
// slices taken from a shared counter: one thread for each `per_thread` units of `work` (the items
// by default; a loop whose items are uneven gives its total work), so a small loop runs on the
// caller alone (starting threads costs more than it saves there). fn must not throw, and calls for
// different i must not write the same data.
template <class F>
void parallel_for(size_t n, size_t per_thread, F&& fn, size_t work = SIZE_MAX) {
    const size_t hw = host_threads();
    const size_t units = work == SIZE_MAX ? n : work;
    const size_t nt = std::min({hw, units / std::max<size_t>(1, per_thread), n});
    if (nt <= 1) {
        for (size_t i = 0; i < n; i++) fn(i);
        return;
    }
    std::atomic<size_t> next{0};
    const size_t slice = std::max<size_t>(1, n / (nt * 16));
    auto run = [&] {
        for (;;) {
            const size_t a = next.fetch_add(slice);
            if (a >= n) return;
            const size_t b = std::min(n, a + slice);
            for (size_t i = a; i < b; i++) fn(i);
        }
    };
    std::vector<std::thread> th;
    th.reserve(nt - 1);
    for (size_t t = 1; t < nt; t++) {
        try {
            th.emplace_back(run);
        } catch (...) {  // no thread to be had: the caller takes the slices the others would have
            break;
        }
    }
    run();
    for (std::thread& t : th) t.join();
}

}  // namespace gz
