// ref_driver.cpp - TEST INFRASTRUCTURE ONLY: a C entry point over the reference's own host
// decoder, so tests can pin the oracle (gi_oracle.c) against the reference itself.
//
// Compiled by oracle/Makefile against gpuinflate/inflate.cuh where it lies in the reference
// tree (nothing of it is copied here); the library goes to oracle/_ref/, which git ignores.
// ref_inflate() drives gi::Decoder the way the reference's harness does (gpuinflate/
// gi_test.cpp:47-91): one run from bit 0 with stream_start set, a new run after every
// overflow, then a pass that turns back-references into bytes and rejects one that reaches
// before the stream's start.
#include "inflate.cuh"

#include <cstdint>
#include <cstring>
#include <vector>

extern "C" {

// 0 ok, 1 invalid data, 2 truncated, 7 output larger than out_cap
int ref_inflate(const uint8_t* in, uint64_t size, uint8_t* out, uint64_t out_cap, uint64_t* out_len, uint64_t* in_used) {
    std::vector<uint8_t> buf((size + 3) / 4 * 4 + 64, 0);
    if (size) memcpy(buf.data(), in, size);
    std::vector<uint16_t> sym(out_cap + 2 * gi::MAX_SYMBOL_OUT + 1);
    static uint16_t luts[gi::LUT_U16];
    gi::Decoder* dec = new gi::Decoder;
    dec->attach(luts);
    gi::Start s{0, 0, gi::AT_BLOCK, -1};
    uint64_t op = 0;
    int rc = 0;
    for (;;) {
        uint64_t room = sym.size() - op;
        gi::Result r = dec->run(buf.data(), size, s, nullptr, 0, sym.data() + op,
                                (uint32_t)(room > 0xffffffffull ? 0xffffffffull : room), op == 0);
        op += r.out_len;
        if (r.status == gi::ERR_OVERFLOW) {
            if (sym.size() - op < 64 * 1024) { rc = 7; break; }
            s = r.resume;
            continue;
        }
        if (r.status != gi::OK) { rc = r.status == gi::ERR_INPUT ? 2 : 1; break; }
        *in_used = (r.end_bit + 7) / 8;
        break;
    }
    delete dec;
    if (rc) return rc;
    if (op > out_cap) return 7;
    for (uint64_t i = 0; i < op; i++) {
        uint16_t v = sym[i];
        if (v <= gi::REF) out[i] = (uint8_t)v;
        else if (v - gi::REF > i) return 1;
        else out[i] = out[i - (v - gi::REF)];
    }
    *out_len = op;
    return 0;
}

// One gi::Decoder::run over in[0..size) (zero padded) from the state (bit, header, mode, final)
// to stop_bit, into a buffer of `cap` symbols, stream_start `first`. res gets: status, end_bit,
// out_len, resume.bit, resume.header, resume.mode, resume.final, blocks, symbols.
int ref_run(const uint8_t* in, uint64_t size, uint64_t bit, uint64_t header, int mode, int final, int first,
            uint64_t stop, uint64_t cap, uint64_t* res) {
    static thread_local std::vector<uint8_t> buf;
    static thread_local std::vector<uint16_t> sym;
    static uint16_t luts[gi::LUT_U16];
    static thread_local gi::Decoder* dec = nullptr;
    if (!dec) {
        dec = new gi::Decoder;
        dec->attach(luts);
    }
    buf.assign((size + 3) / 4 * 4 + 64, 0);
    if (size) memcpy(buf.data(), in, size);
    if (sym.size() < cap) sym.resize(cap);
    gi::Start s{bit, header, (uint8_t)mode, (int8_t)final};
    gi::Result r = dec->run(buf.data(), size, s, nullptr, 0, sym.data(), (uint32_t)cap, first != 0, stop);
    res[0] = (uint64_t)r.status;
    res[1] = r.end_bit;
    res[2] = r.out_len;
    res[3] = r.resume.bit;
    res[4] = r.resume.header;
    res[5] = r.resume.mode;
    res[6] = (uint64_t)(int64_t)r.resume.final;
    res[7] = r.blocks;
    res[8] = r.symbols;
    return 0;
}

int ref_prefilter128(uint64_t v1, uint64_t v2) { return gi::header_prefilter128(v1, v2) ? 1 : 0; }

int ref_plausible_dynamic_header(const uint8_t* in, uint64_t size, uint64_t bit) {
    std::vector<uint8_t> buf((size + 3) / 4 * 4 + 64, 0);
    memcpy(buf.data(), in, size);
    return gi::plausible_dynamic_header(buf.data(), size, bit) ? 1 : 0;
}

}  // extern "C"
