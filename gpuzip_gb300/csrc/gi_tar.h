// gi_tar.h - the tar header rules the rescued output's tar walk applies (gi_rescue.cu): a number
// field and the header checksum, as gpuzip's reader reads them (src/rescue.rs:374-395). Host and
// device code (the header finder runs them on the GPU); tests/tar_check.cpp compiles them on the
// host against the oracle's restatement.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define GI_TAR_HD __host__ __device__
#else
#define GI_TAR_HD
#endif

namespace {

// a tar number field (src/rescue.rs:374-384): GNU base-256 when its first byte has the top bit;
// else the bytes up to a NUL or space, none meaning 0, trimmed of white space (as Rust's
// str::trim on Latin-1 characters: 0x09-0x0D, 0x20, 0x85, 0xA0) and read as octal with an optional
// '+'; false when that does not parse or passes 64 bits
GI_TAR_HD inline bool tar_octal(const uint8_t* f, int n, uint64_t& v) {
    v = 0;
    if (n > 0 && (f[0] & 0x80)) {
        for (int i = 1; i < n; i++) v = v << 8 | f[i];
        return true;
    }
    int e = 0;
    while (e < n && f[e] != 0 && f[e] != ' ') e++;
    if (e == 0) return true;
    auto ws = [](uint8_t c) { return (c >= 0x09 && c <= 0x0d) || c == 0x20 || c == 0x85 || c == 0xa0; };
    int a = 0;
    while (a < e && ws(f[a])) a++;
    while (e > a && ws(f[e - 1])) e--;
    if (a < e && f[a] == '+') a++;
    if (a == e) return false;
    for (int i = a; i < e; i++) {
        if (f[i] < '0' || f[i] > '7') return false;
        if (v >> 61) return false;
        v = v << 3 | (uint64_t)(f[i] - '0');
    }
    return true;
}

// the header checksum as an unsigned or a signed byte sum (src/rescue.rs:386-395)
GI_TAR_HD inline bool tar_header_valid(const uint8_t* h) {
    uint64_t want;
    if (!tar_octal(h + 148, 8, want)) return false;
    uint64_t u = 0;
    int64_t sg = 0;
    for (int i = 0; i < 512; i++) {
        uint8_t b = (i >= 148 && i < 156) ? (uint8_t)' ' : h[i];
        u += b;
        sg += (int8_t)b;
    }
    return want == u || (int64_t)want == sg;
}

}  // namespace
