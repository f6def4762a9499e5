// gi_tarindex.cu - the entries of a tar archive that lies decoded in GPU memory.
//
// gpuzip extracts a .tar.gz by reading the decoded stream through a tar reader on the host, entry
// after entry (src/gz.rs:622-785, the `tar` crate: a 512-byte header with its checksum, the
// entry's data padded to 512 bytes, GNU long names and pax records naming the next entry, an
// all-zero block ending the archive). Here the archive stays where the decoder wrote it: one
// kernel tests every 512-byte block at once for a header (its checksum, in the unsigned or signed
// sum) and gathers the 512 bytes of each one that passes; the host then walks the chain of headers
// from the archive's start over those copies, reading long names and pax records, each a few
// hundred bytes, straight from the device. A caller gets every entry's name, type, size and data
// offset in the decoded buffer, so GPU-resident consumers can take the files in place.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#define GI_BUILD
#include "gpuinflate.h"
#include "gi_common.cuh"
#include "gi_internal.h"
#include "gi_tar.h"

struct gi_tar {
    std::vector<gi_tar_entry> entries;
    std::vector<std::string> names;  // entries[k].name points into names[k]
    uint64_t end = 0;                // bytes the archive took, through its end-of-archive block
};

namespace {

constexpr unsigned TB_WARPS = 8;

// One warp per 512-byte block: the block is a header when its checksum field holds the sum of its
// bytes (the field read as spaces), unsigned or signed; its offset and its bytes are appended.
__global__ void k_tar_headers(const uint8_t* __restrict__ tar, uint64_t nblocks, uint64_t* __restrict__ at,
                              uint8_t* __restrict__ win, unsigned* __restrict__ count, unsigned cap) {
    const int lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t)gridDim.x * TB_WARPS;
    for (uint64_t b = (uint64_t)blockIdx.x * TB_WARPS + (threadIdx.x >> 5); b < nblocks; b += warps) {
        const uint8_t* h = tar + b * 512;
        const uint4 q = *(const uint4*)(h + lane * 16);  // 16 bytes a lane
        const uint8_t* x = (const uint8_t*)&q;
        uint32_t u = 0;
        int32_t sg = 0;
        for (int i = 0; i < 16; i++) {
            const int pos = lane * 16 + i;
            const uint8_t c = (pos >= 148 && pos < 156) ? (uint8_t)' ' : x[i];
            u += c;
            sg += (int8_t)c;
        }
        for (int d = 16; d; d >>= 1) {
            u += __shfl_xor_sync(0xffffffffu, u, d);
            sg += __shfl_xor_sync(0xffffffffu, sg, d);
        }
        uint64_t want = 0;
        const bool parsed = tar_octal(h + 148, 8, want);
        const bool header = parsed && (want == u || (int64_t)want == (int64_t)sg);
        unsigned k = 0;
        if (lane == 0 && header) k = atomicAdd(count, 1u);
        k = __shfl_sync(0xffffffffu, k, 0);
        if (header && k < cap) {
            if (lane == 0) at[k] = b * 512;
            *(uint4*)(win + (uint64_t)k * 512 + lane * 16) = q;
        }
    }
}

// a NUL-ended field of at most n bytes
std::string field(const uint8_t* f, size_t n) {
    const uint8_t* z = (const uint8_t*)memchr(f, 0, n);
    return std::string((const char*)f, z ? (size_t)(z - f) : n);
}

}  // namespace

extern "C" {

GI_API int gi_tar_index_device(gi_ctx* g, const void* d_tar, uint64_t size, gi_tar** out) {
    if (!g) return GI_ERR_ARG;
    if (out) *out = nullptr;
    if (!out || (!d_tar && size)) return gi_ctx_refuse(g, GI_ERR_ARG, "no buffer or no result pointer");
    if (((uintptr_t)d_tar & 15) != 0) return gi_ctx_refuse(g, GI_ERR_ARG, "the archive is not 16-byte aligned");
    const uint8_t* tar = (const uint8_t*)d_tar;
    const uint64_t nblocks = size / 512;
    cudaStream_t st = (cudaStream_t)gi_ctx_stream(g);
    std::vector<uint64_t> at;
    std::vector<uint8_t> win;
    gi_ctx_clear_error(g);
    int rc = [&]() -> int {
        if (cudaSetDevice(gi_ctx_device(g)) != cudaSuccess) return GI_ERR_GPU;
        const unsigned cap = (unsigned)std::min<uint64_t>(nblocks + 1, 1u << 24);
        uint64_t* d_at = nullptr;
        uint8_t* d_win = nullptr;
        unsigned* d_n = nullptr;
        cudaError_t e = cudaMallocAsync(&d_n, sizeof(unsigned), st);
        unsigned n = 0;
        for (int pass = 0; pass < 2 && e == cudaSuccess; pass++) {
            // a first pass counts the headers; the second gathers them into buffers of that size
            const unsigned room = pass ? std::min(n, cap) : 0;
            if (pass && room) {
                e = cudaMallocAsync(&d_at, room * sizeof(uint64_t), st);
                if (e == cudaSuccess) e = cudaMallocAsync(&d_win, (uint64_t)room * 512, st);
            }
            if (e == cudaSuccess) e = cudaMemsetAsync(d_n, 0, sizeof(unsigned), st);
            if (e == cudaSuccess && nblocks) {
                const uint64_t grid = std::min<uint64_t>((nblocks + TB_WARPS - 1) / TB_WARPS, (uint64_t)gz::sm_count() * 16);
                k_tar_headers<<<(unsigned)grid, TB_WARPS * 32, 0, st>>>(tar, nblocks, d_at, d_win, d_n, room);
                e = cudaGetLastError();
            }
            if (e == cudaSuccess) e = cudaMemcpyAsync(&n, d_n, sizeof n, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (pass && e == cudaSuccess && room) {
                at.resize(room);
                win.resize((uint64_t)room * 512);
                e = cudaMemcpyAsync(at.data(), d_at, room * sizeof(uint64_t), cudaMemcpyDeviceToHost, st);
                if (e == cudaSuccess) e = cudaMemcpyAsync(win.data(), d_win, (uint64_t)room * 512, cudaMemcpyDeviceToHost, st);
                if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            }
        }
        cudaFreeAsync(d_at, st);
        cudaFreeAsync(d_win, st);
        cudaFreeAsync(d_n, st);
        cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            cudaGetLastError();
            gi_ctx_set_error(g, std::string("tar index: ") + cudaGetErrorString(e));
            return GI_ERR_GPU;
        }
        return GI_OK;
    }();
    if (rc != GI_OK) return rc;
    // the headers in archive order (the kernel appends them in no order)
    std::vector<uint32_t> ord(at.size());
    for (uint32_t i = 0; i < ord.size(); i++) ord[i] = i;
    std::sort(ord.begin(), ord.end(), [&](uint32_t a, uint32_t b) { return at[a] < at[b]; });
    std::vector<uint64_t> sorted(at.size());
    for (size_t i = 0; i < ord.size(); i++) sorted[i] = at[ord[i]];
    auto header_at = [&](uint64_t p) -> const uint8_t* {
        auto it = std::lower_bound(sorted.begin(), sorted.end(), p);
        return it != sorted.end() && *it == p ? win.data() + (uint64_t)ord[it - sorted.begin()] * 512 : nullptr;
    };
    auto device_bytes = [&](uint64_t p, uint64_t n, std::vector<uint8_t>& buf) -> bool {
        buf.resize(n);
        return n == 0 || (cudaMemcpy(buf.data(), tar + p, n, cudaMemcpyDeviceToHost) == cudaSuccess);
    };

    gi_tar* t = new gi_tar;
    std::string long_name, pax_path;
    bool have_long = false, have_pax_path = false, have_pax_size = false;
    uint64_t pax_size = 0;
    uint64_t p = 0;
    std::vector<uint8_t> buf;
    auto damaged = [&](const std::string& why) {
        delete t;
        return gi_ctx_refuse(g, GI_ERR_DATA, ("tar archive is damaged: " + why).c_str());
    };
    for (;;) {
        if (p + 512 > size) return damaged("it ends inside a header at byte " + std::to_string(p));
        const uint8_t* h = header_at(p);
        if (!h) {
            if (!device_bytes(p, 512, buf)) return damaged("the header at byte " + std::to_string(p) + " cannot be read");
            if (std::all_of(buf.begin(), buf.end(), [](uint8_t c) { return c == 0; })) {
                t->end = p + 512;
                break;
            }
            return damaged("no valid header at byte " + std::to_string(p));
        }
        uint64_t len = 0;
        if (!tar_octal(h + 124, 12, len)) return damaged("the size field at byte " + std::to_string(p + 124));
        if (have_pax_size) len = pax_size;
        const uint8_t type = h[156];
        const uint64_t data = p + 512, next = data + (len + 511) / 512 * 512;
        if (data + len > size) return damaged("entry at byte " + std::to_string(p) + " runs past the end");
        if (type == 'L' || type == 'K' || type == 'x') {  // names and records for the next entry
            if (len > (64u << 20)) return damaged("metadata entry of " + std::to_string(len) + " bytes");
            if (!device_bytes(data, len, buf)) return damaged("metadata at byte " + std::to_string(data) + " cannot be read");
            if (type == 'L') {
                long_name = field(buf.data(), buf.size());
                have_long = true;
            } else if (type == 'x') {  // "<len> key=value\n" records
                size_t q = 0;
                while (q < buf.size()) {
                    const uint8_t* sp = (const uint8_t*)memchr(buf.data() + q, ' ', buf.size() - q);
                    if (!sp) break;
                    uint64_t rl = 0;
                    bool ok = sp > buf.data() + q;
                    for (const uint8_t* c = buf.data() + q; c < sp && ok; c++) {
                        ok = *c >= '0' && *c <= '9' && rl < (1ull << 40);
                        rl = rl * 10 + (uint64_t)(*c - '0');
                    }
                    if (!ok || rl == 0 || q + rl > buf.size() || (uint64_t)(sp - buf.data()) + 1 > q + rl - 1) break;
                    const std::string kv((const char*)sp + 1, (size_t)(q + rl - 1 - (uint64_t)(sp + 1 - buf.data())));
                    const size_t eq = kv.find('=');
                    if (eq != std::string::npos) {
                        const std::string k = kv.substr(0, eq), v = kv.substr(eq + 1);
                        if (k == "path") {
                            pax_path = v;
                            have_pax_path = true;
                        } else if (k == "size") {
                            pax_size = 0;
                            have_pax_size = !v.empty() && v.find_first_not_of("0123456789") == std::string::npos;
                            for (char c : v) pax_size = pax_size * 10 + (uint64_t)(c - '0');
                        }
                    }
                    q += rl;
                }
            }
            p = next;
            continue;
        }
        std::string name;
        if (have_pax_path) name = pax_path;
        else if (have_long) name = long_name;
        else {
            name = field(h, 100);
            const bool ustar = memcmp(h + 257, "ustar\0", 6) == 0;  // POSIX ustar: a prefix field
            const std::string prefix = ustar ? field(h + 345, 155) : std::string();
            if (!prefix.empty()) name = prefix + "/" + name;
        }
        have_long = have_pax_path = have_pax_size = false;
        t->names.push_back(name);
        t->entries.push_back(gi_tar_entry{nullptr, p, data, len, type, 0});
        p = next;
    }
    for (size_t k = 0; k < t->entries.size(); k++) t->entries[k].name = t->names[k].c_str();
    *out = t;
    return GI_OK;
}

GI_API uint32_t gi_tar_entries(const gi_tar* t, const gi_tar_entry** entries) {
    if (!t) return 0;
    if (entries) *entries = t->entries.data();
    return (uint32_t)t->entries.size();
}

GI_API uint64_t gi_tar_end(const gi_tar* t) { return t ? t->end : 0; }

GI_API void gi_tar_free(gi_tar* t) { delete t; }

}  // extern "C"
