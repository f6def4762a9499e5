// Driver for the host steps' parallel loop (gpuzip_gb300/csrc/gi_parallel.h), used by
// tests/test_parallel.py: reads "n per_thread work" lines (work -1: the loop's default) and prints,
// per line, 1 when every index in [0, n) ran exactly once (else 0), the number of distinct threads
// that ran them, and host_threads().
#include <atomic>
#include <cstdio>
#include <memory>
#include <set>
#include <thread>
#include <vector>

#include "gi_parallel.h"

int main() {
    long long n, per, work;
    while (scanf("%lld %lld %lld", &n, &per, &work) == 3) {
        std::unique_ptr<std::atomic<int>[]> seen(new std::atomic<int>[n > 0 ? n : 1]());
        std::vector<std::thread::id> who((size_t)(n > 0 ? n : 1));
        gz::parallel_for(
            (size_t)n, (size_t)per,
            [&](size_t i) {
                seen[i]++;
                who[i] = std::this_thread::get_id();
            },
            work < 0 ? SIZE_MAX : (size_t)work);
        int ok = 1;
        std::set<std::thread::id> ids;
        for (long long i = 0; i < n; i++) {
            ok &= seen[i].load() == 1;
            ids.insert(who[(size_t)i]);
        }
        printf("%d %zu %zu\n", ok, ids.size(), gz::host_threads());
        fflush(stdout);
    }
    return 0;
}
