// gi_find_cl.h - the code-length-code test of the block-start finder, shared by the finder kernel
// and a host check of it (compiled by nvcc and by a plain C++ compiler).
//
// A dynamic block's header (RFC 1951 3.2.7) starts BFINAL, BTYPE (2 bits), HLIT (5), HDIST (5),
// HCLEN (4), then HCLEN + 4 code lengths of 3 bits for the code-length alphabet. zlib accepts the
// header only if that code is complete: the Kraft sum of 2^-l over the nonzero lengths l is 1,
// i.e. the lengths' contributions 128 >> l add up to 128 (gpuinflate/inflate.cuh:300-311 applies
// the same test to the 128 bits at a candidate). Here the fields past HCLEN + 4 are masked off and
// the 19 fields are summed four at a time through a 4096-entry table of the contributions of four
// fields (five lookups instead of nineteen steps).
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define GI_HD __host__ __device__ __forceinline__
#else
#define GI_HD inline
#endif

namespace gz {

constexpr int CL4_ENTRIES = 4096;

// the table entry for four 3-bit lengths packed in x (first length in the low bits)
GI_HD uint16_t cl4_entry(uint32_t x) {
    uint32_t s = 0;
    for (int j = 0; j < 4; j++) {
        uint32_t l = (x >> (3 * j)) & 7;
        s += l ? 128u >> l : 0u;
    }
    return (uint16_t)s;
}

// v1, v2: the 128 bits at a candidate (bit 0 of v1 = BFINAL), whose first 17 bits passed the
// BTYPE/HLIT/HDIST tests; true if the code-length code is complete
GI_HD bool cl_complete_tab(uint64_t v1, uint64_t v2, const uint16_t* tab) {
    const int hclen = (int)((v1 >> 13) & 15) + 4;  // 4 .. 19 fields
    const uint64_t f = ((v1 >> 17) | (v2 << 47)) & ((1ull << (3 * hclen)) - 1);
    const uint32_t sum = (uint32_t)tab[f & 4095] + tab[(f >> 12) & 4095] + tab[(f >> 24) & 4095] +
                         tab[(f >> 36) & 4095] + tab[(f >> 48) & 4095];
    return sum == 128;
}

// the same test field by field (the definition the table form is checked against)
GI_HD bool cl_complete_loop(uint64_t v1, uint64_t v2) {
    const int hclen = (int)((v1 >> 13) & 15) + 4;
    const uint64_t f = (v1 >> 17) | (v2 << 47);
    uint32_t sum = 0;
    for (int i = 0; i < hclen; i++) {
        uint32_t l = (uint32_t)(f >> (3 * i)) & 7;
        sum += l ? 128u >> l : 0u;
    }
    return sum == 128;
}

}  // namespace gz
