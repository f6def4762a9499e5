// gi_find.cu - the block-start finder: for every chunk of the compressed input, the first bit
// position that passes every check zlib applies to a dynamic-Huffman block header.
//
// The two tests are the reference's (gpuinflate/inflate.cuh:300-332): a cheap one on the 128
// bits at a candidate (BTYPE 2, HLIT and HDIST at most 29, a complete code-length code) and the
// full header check (code lengths decode, 16 not first, no repeat past the end, an end-of-block
// code, Kraft rules for the literal/length and distance codes, and no read past the input).
// The layout of the work is this file's own: a warp owns a chunk and walks it 32 words at a
// time; each lane computes the BTYPE/HLIT/HDIST test for the 32 bit offsets of its word at once
// as bit-sliced masks (a dozen shifts and ANDs instead of 32 tests), runs the code-length-code
// test on the survivors, and the warp compacts the survivors in bit order through a ballot
// prefix. Full checks then run 32 candidates at a time, one per lane; passing lanes (a ballot)
// are kept in bit order, up to four per chunk (the reference keeps one, and misses the second
// of two blocks that start in one chunk, which then gets no decoder of its own).
// Chunks of 4 KiB hold about 30 such candidates in real data (the reference measured 1 in
// 1,100 bit positions surviving the cheap tests), so the list usually drains once per chunk.
#include <cuda_runtime.h>

#include "gi_common.cuh"
#include "gi_find_cl.h"

namespace gz {
namespace {

constexpr int FIND_WARPS = 8;
constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ uint32_t ldw(const uint32_t* w, uint64_t i, uint64_t end) {
    return i < end ? __ldg(w + i) : 0u;
}

struct LaneBits {
    const uint32_t* w;
    uint64_t end_word;
    uint64_t next;
    uint64_t buf;
    int cnt;

    __device__ void init(const uint32_t* w_, uint64_t end_w, uint64_t bit) {
        w = w_;
        end_word = end_w;
        next = bit >> 5;
        buf = 0;
        cnt = 0;
        refill();
        int s = (int)(bit & 31);
        buf >>= s;
        cnt -= s;
    }
    __device__ void refill() {
        while (cnt <= 32) {
            buf |= (uint64_t)ldw(w, next, end_word) << cnt;
            next++;
            cnt += 32;
        }
    }
    __device__ uint32_t peek(int n) {
        if (cnt < n) refill();
        return (uint32_t)(buf & ((1ull << n) - 1));
    }
    __device__ void drop(int n) {
        buf >>= n;
        cnt -= n;
    }
    __device__ uint32_t get(int n) {
        uint32_t v = peek(n);
        drop(n);
        return v;
    }
    __device__ uint64_t pos() const { return next * 32 - (uint64_t)cnt; }
};

__device__ const uint8_t c_cl_order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

// 0 complete, 1 incomplete, -1 over-subscribed, from counts per length (index 0 ignored)
__device__ __forceinline__ int kraft_counts(const uint16_t* cnt) {
    int left = 1;
    for (int len = 1; len < 16; len++) {
        left = (left << 1) - cnt[len];
        if (left < 0) return -1;
    }
    return left > 0 ? 1 : 0;
}

// the full check of a dynamic header at `bit` (inflate.cuh:315-332 states the same rules)
__device__ bool verify_header(const uint32_t* w, uint64_t end_word, uint64_t end_bit, uint64_t bit) {
    LaneBits b;
    b.init(w, end_word, bit);
    b.drop(3);
    int hlit = (int)b.get(5) + 257;
    int hdist = (int)b.get(5) + 1;
    int hclen = (int)b.get(4) + 4;
    if (hlit > 286 || hdist > 30) return false;
    uint8_t cl[19];
    for (int i = 0; i < 19; i++) cl[i] = 0;
    for (int i = 0; i < hclen; i++) cl[c_cl_order[i]] = (uint8_t)b.get(3);
    uint16_t ccount[16];
    for (int i = 0; i < 16; i++) ccount[i] = 0;
    for (int i = 0; i < 19; i++) ccount[cl[i]]++;
    ccount[0] = 0;
    if (kraft_counts(ccount) != 0) return false;  // the code-length code must be complete
    uint8_t sorted[19];
    {
        uint8_t offs[8];
        offs[1] = 0;
        for (int l = 1; l < 7; l++) offs[l + 1] = (uint8_t)(offs[l] + ccount[l]);
        for (int s = 0; s < 19; s++)
            if (cl[s]) sorted[offs[cl[s]]++] = (uint8_t)s;
    }
    uint16_t lit_cnt[16], dist_cnt[16];
    for (int i = 0; i < 16; i++) lit_cnt[i] = dist_cnt[i] = 0;
    int total = hlit + hdist;
    int prev = 0;
    bool eob = false;
    for (int i = 0; i < total;) {
        uint32_t bits = b.peek(7);
        int code = 0, first = 0, index = 0, sym = -1;
        for (int len = 1; len <= 7; len++) {
            code |= (int)((bits >> (len - 1)) & 1);
            int c = ccount[len];
            if (code - c < first) {
                b.drop(len);
                sym = sorted[index + (code - first)];
                break;
            }
            index += c;
            first = (first + c) << 1;
            code <<= 1;
        }
        if (sym < 0) return false;
        int rep = 1, val = sym;
        if (sym == 16) {
            if (i == 0) return false;
            val = prev;
            rep = 3 + (int)b.get(2);
        } else if (sym == 17) {
            val = 0;
            rep = 3 + (int)b.get(3);
        } else if (sym == 18) {
            val = 0;
            rep = 11 + (int)b.get(7);
        }
        if (i + rep > total) return false;
        // counts per length for the two codes; position 256 is the end-of-block code
        int nlit = i < hlit ? min(rep, hlit - i) : 0;
        lit_cnt[val] += (uint16_t)nlit;
        dist_cnt[val] += (uint16_t)(rep - nlit);
        if (i <= 256 && 256 < i + rep && 256 < hlit) eob = val != 0;
        prev = val;
        i += rep;
    }
    if (!eob) return false;
    int nz = hlit - lit_cnt[0], ones = lit_cnt[1];
    int r = kraft_counts(lit_cnt);
    if (r < 0 || (r > 0 && !(nz == 1 && ones == 1))) return false;
    nz = hdist - dist_cnt[0];
    ones = dist_cnt[1];
    r = kraft_counts(dist_cnt);
    if (r < 0 || (r > 0 && !(nz == 0 || (nz == 1 && ones == 1)))) return false;
    return b.pos() <= end_bit;
}

// Candidates that pass the cheap tests queue up in bit order in the warp's shared-memory list and
// are verified 32 at a time (one per lane), so the expensive check runs on full warps; the list
// is drained whenever it holds a full batch, and the first batch with a pass gives the chunk's
// first start (every earlier candidate was verified before it).
constexpr int LIST = 1024 + 64;
constexpr int FIND_SLOTS = 4;  // block starts kept per chunk (a short block can share a chunk with the next)

// ALL: every verified candidate is appended to all_out (in no order; all_n counts them, past
// all_cap too) instead of the chunk's first FIND_SLOTS going to `first`
template <bool ALL>
__global__ void __launch_bounds__(FIND_WARPS * 32) k_find(const uint32_t* __restrict__ w, uint64_t bit_lo,
                                                          uint64_t bit_hi, uint64_t end_word, uint64_t end_bit,
                                                          uint32_t chunk_bits, uint64_t nchunks,
                                                          uint64_t* __restrict__ first,
                                                          const uint8_t* __restrict__ skip,
                                                          uint64_t* __restrict__ all_out, unsigned* __restrict__ all_n,
                                                          unsigned all_cap) {
    __shared__ uint32_t cand[FIND_WARPS][LIST];  // candidate bit, relative to the chunk's first word
    __shared__ uint16_t cl4[CL4_ENTRIES];         // Kraft contributions of four code-length fields
    for (int i = threadIdx.x; i < CL4_ENTRIES; i += blockDim.x) cl4[i] = cl4_entry((uint32_t)i);
    __syncthreads();
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    uint32_t* list = cand[wib];
    const uint64_t nwarps = (uint64_t)gridDim.x * FIND_WARPS;
    for (uint64_t c = (uint64_t)blockIdx.x * FIND_WARPS + wib; c < nchunks; c += nwarps) {
        uint64_t cb = bit_lo + c * chunk_bits;
        uint64_t lo = cb > bit_lo ? cb : bit_lo + 1;  // candidates are strictly after bit_lo
        uint64_t hi = cb + chunk_bits < bit_hi ? cb + chunk_bits : bit_hi;
        int nfound = 0;
        uint64_t found = UINT64_MAX;  // lane j < FIND_SLOTS holds hit j
        if (lo < hi && !(skip && (skip[c] & SKIP_CHUNK))) {
            // a chunk near the end of a stream also keeps headers of a final block (BFINAL 1)
            const bool finals = ALL || (skip && (skip[c] & FINAL_CHUNK));
            const uint64_t w0 = lo >> 5, w1 = (hi + 31) >> 5;
            int nlist = 0;
            // verifies list[0 .. n) in batches of 32 (n a multiple of 32 unless final), keeping the
            // hits in bit order; true once FIND_SLOTS hits are kept
            auto drain = [&](int n) -> bool {
                for (int b0 = 0; b0 < n; b0 += 32) {
                    bool ok = false;
                    uint64_t bit = 0;
                    if (b0 + lane < n) {
                        bit = w0 * 32 + list[b0 + lane];
                        ok = verify_header(w, end_word, end_bit, bit);
                    }
                    uint32_t bal = __ballot_sync(FULL, ok);
                    if (ALL) {
                        if (ok) {
                            unsigned q = atomicAdd(all_n, 1u);
                            if (q < all_cap) all_out[q] = bit;
                        }
                        continue;
                    }
                    while (bal && nfound < FIND_SLOTS) {
                        uint64_t b = __shfl_sync(FULL, bit, __ffs(bal) - 1);
                        if (lane == nfound) found = b;
                        nfound++;
                        bal &= bal - 1;
                    }
                    if (nfound == FIND_SLOTS) return true;
                }
                return false;
            };
            bool done = false;
            for (uint64_t ws = w0; ws < w1 && !done; ws += 32) {
                uint64_t wi = ws + lane;
                uint32_t mask = 0;
                if (wi < w1) {
                    uint64_t a = ldw(w, wi, end_word), b = ldw(w, wi + 1, end_word);
                    uint64_t c2 = ldw(w, wi + 2, end_word), d = ldw(w, wi + 3, end_word);
                    uint64_t lo64 = a | b << 32, hi64 = c2 | d << 32;
                    // bit-sliced: bit o of m is the test for the offset wi*32+o
                    uint64_t m = ~(lo64 >> 1) & (lo64 >> 2);                          // BTYPE = 2
                    m &= ~((lo64 >> 4) & (lo64 >> 5) & (lo64 >> 6) & (lo64 >> 7));    // HLIT <= 29
                    m &= ~((lo64 >> 9) & (lo64 >> 10) & (lo64 >> 11) & (lo64 >> 12)); // HDIST <= 29
                    // BFINAL = 0 for the decode paths: only a stream's last block is final, so
                    // final-block headers are looked for only near a stream's end (the rescue keeps
                    // every header)
                    if (!finals) m &= ~lo64;
                    mask = (uint32_t)m;
                    uint64_t base = wi * 32;
                    if (base < lo) mask &= ~0u << (uint32_t)(lo - base);
                    if (base + 32 > hi) mask &= (1u << (uint32_t)(hi - base)) - 1;

                    uint32_t keep = 0, mm = mask;
                    while (mm) {
                        int o = __ffs(mm) - 1;
                        mm &= mm - 1;
                        uint64_t v1 = o ? (lo64 >> o) | (hi64 << (64 - o)) : lo64;
                        uint64_t v2 = hi64 >> o;
                        if (cl_complete_tab(v1, v2, cl4)) keep |= 1u << o;
                    }
                    mask = keep;
                }
                // survivors, in bit order, appended to the warp's list
                int n = __popc(mask), incl = n;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    int v = __shfl_up_sync(FULL, incl, d);
                    if (lane >= d) incl += v;
                }
                int total = __shfl_sync(FULL, incl, 31);
                int j = nlist + incl - n;
                uint32_t rel = (uint32_t)((wi - w0) * 32);
                for (uint32_t mm = mask; mm; mm &= mm - 1) list[j++] = rel + (uint32_t)(__ffs(mm) - 1);
                nlist += total;
                __syncwarp();
                if (nlist >= 32) {
                    int full = nlist & ~31;
                    done = drain(full);
                    if (!done) {
                        // keep the unverified tail at the front
                        int rest = nlist - full;
                        uint32_t v = lane < rest ? list[full + lane] : 0;
                        __syncwarp();
                        if (lane < rest) list[lane] = v;
                        nlist = rest;
                        __syncwarp();
                    }
                }
            }
            if (!done && nlist) drain(nlist);
        }
        if (!ALL && lane < FIND_SLOTS) first[c * FIND_SLOTS + lane] = found;
    }
}

// Stored-block signatures: every byte position in [byte_lo, byte_hi) whose 16-bit LEN is
// followed by NLEN = ~LEN (RFC 1951 3.2.4). One thread per 32-bit word, four positions each;
// hits are rare (one per stored block, and 1 in 65,536 positions of other data).
__global__ void k_stored_scan(const uint32_t* __restrict__ w, uint64_t byte_lo, uint64_t byte_hi, uint64_t end_word,
                              uint64_t end_byte, StoredCand* __restrict__ out, unsigned* __restrict__ n, unsigned cap) {
    uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t wi = (byte_lo >> 2) + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; wi * 4 < byte_hi; wi += stride) {
        uint64_t v = (uint64_t)ldw(w, wi, end_word) | (uint64_t)ldw(w, wi + 1, end_word) << 32;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            uint32_t len = (uint32_t)(v >> (8 * k)) & 0xffff;
            uint32_t nlen = (uint32_t)(v >> (8 * k + 16)) & 0xffff;
            uint64_t byte = wi * 4 + k;
            if (len == (~nlen & 0xffff) && byte >= byte_lo && byte < byte_hi && byte + 4 + len <= end_byte) {
                unsigned q = atomicAdd(n, 1u);
                if (q < cap) out[q] = StoredCand{byte, len};
            }
        }
    }
}

// ---------------------------------------------------------------- block density
//
// How many output bytes and how many codes a block yields per compressed bit, predicted from its
// header alone: a Huffman code of length L is taken to occur with probability 2^-L, so a dynamic
// block yields E[output] / E[bits] bytes and 1 / E[bits] codes per bit, a match's bits including
// its length's extra bits and its distance code's average cost. The planner prices a decoder's
// job from them (its time follows the codes it decodes and, less, the bytes it writes), and
// places no probe points in a block whose codes barely compress (a near-flat code: a decode
// started off the symbol boundaries does not fall back onto them).

__device__ const uint16_t c_len_base[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                                            31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
__device__ const uint8_t c_len_extra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
constexpr float FIXED_DENSITY = 0.2f;  // a fixed-code block: taken as about 1.6 bytes of output per input byte

__device__ float2 header_density(const uint32_t* w, uint64_t end_word, uint64_t bit) {
    const float2 none = make_float2(0.f, 0.f);
    LaneBits b;
    b.init(w, end_word, bit);
    b.drop(1);
    const int type = (int)b.get(2);
    if (type == 0) return make_float2(0.125f, 0.f);  // stored: copied, no codes
    if (type == 1) return make_float2(FIXED_DENSITY, FIXED_DENSITY / 1.6f);
    if (type != 2) return none;
    const int hlit = (int)b.get(5) + 257, hdist = (int)b.get(5) + 1, hclen = (int)b.get(4) + 4;
    if (hlit > 286 || hdist > 30) return none;
    uint8_t cl[19] = {};
    for (int i = 0; i < hclen; i++) cl[c_cl_order[i]] = (uint8_t)b.get(3);
    uint16_t ccount[16] = {};
    for (int i = 0; i < 19; i++) ccount[cl[i]]++;
    ccount[0] = 0;
    if (kraft_counts(ccount) != 0) return none;
    uint8_t sorted[19];
    {
        uint8_t offs[8];
        offs[1] = 0;
        for (int l = 1; l < 7; l++) offs[l + 1] = (uint8_t)(offs[l] + ccount[l]);
        for (int s = 0; s < 19; s++)
            if (cl[s]) sorted[offs[cl[s]]++] = (uint8_t)s;
    }
    float out = 0.f, bits = 0.f, p_match = 0.f, dist_bits = 0.f, p_dist = 0.f;
    const int total = hlit + hdist;
    int prev = 0;
    for (int i = 0; i < total;) {
        const uint32_t peek = b.peek(7);
        int code = 0, first = 0, index = 0, sym = -1;
        for (int len = 1; len <= 7; len++) {  // canonical decode, one bit at a time
            code |= (int)((peek >> (len - 1)) & 1);
            const int c = ccount[len];
            if (code - c < first) {
                b.drop(len);
                sym = sorted[index + (code - first)];
                break;
            }
            index += c;
            first = (first + c) << 1;
            code <<= 1;
        }
        if (sym < 0) return none;
        int rep = 1, val = sym;
        if (sym == 16) {
            if (i == 0) return none;
            val = prev;
            rep = 3 + (int)b.get(2);
        } else if (sym == 17) {
            val = 0;
            rep = 3 + (int)b.get(3);
        } else if (sym == 18) {
            val = 0;
            rep = 11 + (int)b.get(7);
        }
        if (i + rep > total) return none;
        if (val) {
            const float pr = exp2f(-(float)val);
            for (int q = i; q < i + rep; q++) {
                if (q < 256) {
                    out += pr;
                    bits += pr * (float)val;
                } else if (q == 256) {
                    bits += pr * (float)val;
                } else if (q < hlit) {
                    const int s = q - 257 < 28 ? q - 257 : 28;
                    const int x = c_len_extra[s];
                    out += pr * ((float)c_len_base[s] + 0.5f * (float)((1 << x) - 1));
                    bits += pr * (float)(val + x);
                    p_match += pr;
                } else {
                    const int d = q - hlit;
                    dist_bits += pr * (float)(val + (d < 4 ? 0 : (d - 2) / 2));
                    p_dist += pr;
                }
            }
        }
        prev = val;
        i += rep;
    }
    if (p_dist > 0.f) bits += p_match * dist_bits / p_dist;
    return bits > 0.f ? make_float2(out / bits, 1.f / bits) : none;
}

__global__ void k_density(const uint32_t* __restrict__ w, uint64_t end_word, const uint64_t* __restrict__ bits, uint64_t n,
                          float2* __restrict__ out) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = bits[i] == UINT64_MAX ? make_float2(0.f, 0.f) : header_density(w, end_word, bits[i]);
}

}  // namespace

int launch_density(const uint8_t* d_in, uint64_t end_word, const uint64_t* bits, uint64_t n, float2* out, void* stream) {
    if (!n) return 0;
    const uint64_t want = (n + 127) / 128, cap = (uint64_t)sm_count() * 16;
    k_density<<<(unsigned)(want < cap ? want : cap), 128, 0, (cudaStream_t)stream>>>((const uint32_t*)d_in, end_word, bits, n,
                                                                                     out);
    return 1;
}

int launch_stored_scan(const uint8_t* d_in, uint64_t byte_lo, uint64_t byte_hi, uint64_t end_word, uint64_t end_byte,
                       StoredCand* out, unsigned* n, unsigned cap, void* stream) {
    if (byte_hi <= byte_lo) return 0;
    uint64_t words = (byte_hi - byte_lo) / 4 + 2;
    uint64_t blocks = (words + 255) / 256;
    const uint64_t max_blocks = (uint64_t)sm_count() * 32;
    if (blocks > max_blocks) blocks = max_blocks;
    k_stored_scan<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>((const uint32_t*)d_in, byte_lo, byte_hi, end_word,
                                                                       end_byte, out, n, cap);
    return 1;
}

int launch_find(const uint8_t* d_in, uint64_t bit_lo, uint64_t bit_hi, uint64_t end_word, uint32_t chunk_bits,
                uint64_t nchunks, uint64_t* d_first, uint64_t end_bit, const uint8_t* skip, void* stream) {
    if (!nchunks) return 0;
    int dev = 0, nsm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    uint64_t blocks = (nchunks + FIND_WARPS - 1) / FIND_WARPS;
    uint64_t cap = (uint64_t)nsm * 8;
    k_find<false><<<(unsigned)(blocks < cap ? blocks : cap), FIND_WARPS * 32, 0, (cudaStream_t)stream>>>(
        (const uint32_t*)d_in, bit_lo, bit_hi, end_word, end_bit, chunk_bits, nchunks, d_first, skip, nullptr, nullptr, 0);
    return 1;
}

int launch_find_all(const uint8_t* d_in, uint64_t bit_lo, uint64_t bit_hi, uint64_t end_word, uint64_t end_bit,
                    uint64_t* out, unsigned* n, unsigned cap, void* stream) {
    if (bit_hi <= bit_lo + 1) return 0;
    const uint32_t chunk_bits = 4096 * 8;
    uint64_t nchunks = (bit_hi - bit_lo + chunk_bits - 1) / chunk_bits;
    int dev = 0, nsm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    uint64_t blocks = (nchunks + FIND_WARPS - 1) / FIND_WARPS;
    uint64_t gcap = (uint64_t)nsm * 8;
    k_find<true><<<(unsigned)(blocks < gcap ? blocks : gcap), FIND_WARPS * 32, 0, (cudaStream_t)stream>>>(
        (const uint32_t*)d_in, bit_lo, bit_hi, end_word, end_bit, chunk_bits, nchunks, nullptr, nullptr, out, n, cap);
    return 1;
}

}  // namespace gz
