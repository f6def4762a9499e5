// Host check of the finder's code-length-code test (gpuzip_gb300/csrc/gi_find_cl.h), used by
// tests/test_finder_cl.py: the table form against the field-by-field definition, on every
// HCLEN with seeded random fields, on every 12-bit table index, and on hand-made complete codes.
// Prints "<cases> <complete>" and exits 1 on the first disagreement.
#include <cstdio>
#include <cstdlib>
#include <cstdint>

#include "gi_find_cl.h"

static uint64_t sm = 0x9E3779B97F4A7C15ull;
static uint64_t next64() {  // SplitMix64
    uint64_t z = (sm += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

int main(int argc, char** argv) {
    long n = argc > 1 ? atol(argv[1]) : 2000000;
    uint16_t tab[gz::CL4_ENTRIES];
    for (uint32_t i = 0; i < (uint32_t)gz::CL4_ENTRIES; i++) tab[i] = gz::cl4_entry(i);
    long cases = 0, complete = 0;
    auto one = [&](uint64_t v1, uint64_t v2) {
        bool a = gz::cl_complete_tab(v1, v2, tab), b = gz::cl_complete_loop(v1, v2);
        cases++;
        complete += b;
        if (a != b) {
            printf("mismatch %016llx %016llx\n", (unsigned long long)v1, (unsigned long long)v2);
            return false;
        }
        return true;
    };
    for (long i = 0; i < n; i++) {
        uint64_t v1 = next64(), v2 = next64();
        if (!one(v1, v2)) return 1;
    }
    // complete codes by construction: lengths from a random full binary tree cut, every HCLEN
    for (long i = 0; i < n / 4; i++) {
        int hclen = (int)(next64() % 16) + 4;
        uint32_t len[19] = {0};
        // start from two codes of length 1 and split random leaves while there is room
        int nl = 2;
        len[0] = 1;
        len[1] = 1;
        for (int s = 0; s < 40 && nl < hclen; s++) {
            int k = (int)(next64() % nl);
            if (len[k] >= 7) continue;
            len[k]++;
            len[nl++] = len[k];
        }
        // scatter the lengths over the first hclen fields
        uint32_t field[19] = {0};
        for (int k = 0; k < nl; k++) {
            int pos;
            do pos = (int)(next64() % hclen); while (field[pos]);
            field[pos] = len[k];
        }
        uint64_t f = 0;
        for (int k = 0; k < 19; k++) f |= (uint64_t)(k < hclen ? field[k] : (uint32_t)(next64() & 7)) << (3 * k);
        uint64_t head = next64() & ((1ull << 13) - 1);
        uint64_t v1 = head | (uint64_t)(hclen - 4) << 13 | (f << 17);
        uint64_t v2 = (f >> 47) | (next64() << 10);
        if (!one(v1, v2)) return 1;
    }
    for (uint32_t x = 0; x < (uint32_t)gz::CL4_ENTRIES; x++) {  // every table index in every position
        for (int pos = 0; pos < 5; pos++) {
            uint64_t f = (uint64_t)x << (12 * pos);
            uint64_t v1 = (uint64_t)15 << 13 | (f << 17), v2 = f >> 47;
            if (!one(v1, v2)) return 1;
        }
    }
    printf("%ld %ld\n", cases, complete);
    return 0;
}
