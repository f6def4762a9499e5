// Driver for the request server's arena allocator (gpuzip_gb300/csrc/gi_arena.h), used by
// tests/test_arena.py: reads "c <capacity> <align>", "a <id> <bytes>", "f <id>" lines and prints,
// per line, the offset given (or -1), then the state: used bytes, peak, free ranges, largest free.
#include <cstdio>
#include <cstring>
#include <map>

#include "gi_arena.h"

int main() {
    gz::Arena a;
    std::map<long, std::pair<unsigned long long, unsigned long long>> live;  // id -> (offset, bytes)
    char op[8];
    while (scanf("%7s", op) == 1) {
        long long off = -1;
        if (!strcmp(op, "c")) {
            unsigned long long cap, align;
            if (scanf("%llu %llu", &cap, &align) != 2) return 2;
            a.reset(cap, align);
        } else if (!strcmp(op, "a")) {
            long id;
            unsigned long long n;
            if (scanf("%ld %llu", &id, &n) != 2) return 2;
            unsigned long long o = a.alloc(n);
            if (o != gz::Arena::NONE) {
                live[id] = {o, n};
                off = (long long)o;
            }
        } else if (!strcmp(op, "f")) {
            long id;
            if (scanf("%ld", &id) != 1) return 2;
            auto it = live.find(id);
            if (it == live.end()) return 3;
            a.release(it->second.first, it->second.second);
            live.erase(it);
        } else {
            return 2;
        }
        printf("%lld %llu %llu %zu %llu\n", off, (unsigned long long)a.used(), (unsigned long long)a.peak(),
               a.free_ranges(), (unsigned long long)a.largest_free());
    }
    return 0;
}
