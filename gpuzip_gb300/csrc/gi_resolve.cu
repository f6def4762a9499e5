// gi_resolve.cu - from decoded symbols to bytes, and the CRC-32 of the bytes.
//
// The decoders leave one 16-bit symbol per output position: a byte, or REF + d for "the byte d
// back" (gpuinflate/inflate.cuh:31). The reference resolves those by writing a 32-bit entry per
// position and pointer jumping over all of them (gpuinflate/gpuinflate.cu:366-421); on text,
// where most bytes are copies of copies hundreds deep, that costs several rounds of dependent
// gathers per byte. Here the output is cut into spans (512 KiB) and resolved in three passes
// that never follow a chain through memory:
//   1. k_local, one block per span, walks the span in order in tiles of 2048 positions: a copy
//      whose source is in an earlier tile reads that tile's (already resolved) value, a copy
//      inside the tile is resolved by pointer doubling in shared memory, and a copy that
//      reaches before the span becomes a marker 256 + m: "byte m of the span's entry window"
//      (the 32 KiB before the span). A copy before the stream's start sets `bad`.
//   2. k_windows, one block, walks the spans in order: span s's entry window is span s-1's last
//      32 KiB with its markers looked up in span s-1's entry window (one 32 KiB gather a span).
//   3. k_final, parallel over every position: a byte, or its span's window byte.
// Stored blocks skipped by the decoders are copied into the symbol pool first, 8 symbols (16
// bytes) per store. CRC-32 is computed from the output bytes: each warp takes 4 KiB (128 bytes
// per lane, bytewise table in shared memory), lane CRCs are merged by the GF(2) identity
//     crc(A || B) = crc(A) * x^(8|B|) mod P  xor  crc(B)
// (carry-less multiplication modulo the CRC polynomial), then 4 KiB CRCs are merged 1024 at a
// time by the same identity until one is left. The multipliers x^(8n) for the fixed sizes are
// computed on the host.
#include <cuda_runtime.h>

#include <atomic>

#include "gi_common.cuh"

namespace gz {
namespace {

constexpr uint32_t POLY = 0xEDB88320u;

unsigned blocks_for(uint64_t n, unsigned per) {
    uint64_t b = (n + per - 1) / per;
    return (unsigned)(b ? b : 1);
}

// ---------------------------------------------------------------- stored blocks

// one block of threads per stored block; 8 output symbols (16 bytes) per thread per step where
// the destination is aligned
__global__ void k_stored(const uint8_t* __restrict__ in, uint16_t* __restrict__ pool, const StoredCopy* list, int n) {
    for (int b = blockIdx.x; b < n; b += gridDim.x) {
        StoredCopy c = list[b];
        uint16_t* dst = pool + c.dst;
        const uint8_t* src = in + c.src;
        uint32_t head = (uint32_t)((8 - (c.dst & 7)) & 7);
        if (head > c.len) head = c.len;
        if (threadIdx.x < head) dst[threadIdx.x] = src[threadIdx.x];
        uint32_t body = (c.len - head) / 8;
        for (uint32_t i = threadIdx.x; i < body; i += blockDim.x) {
            const uint8_t* s = src + head + i * 8;
            uint4 q;
            q.x = (uint32_t)s[0] | ((uint32_t)s[1] << 16);
            q.y = (uint32_t)s[2] | ((uint32_t)s[3] << 16);
            q.z = (uint32_t)s[4] | ((uint32_t)s[5] << 16);
            q.w = (uint32_t)s[6] | ((uint32_t)s[7] << 16);
            *(uint4*)(dst + head + i * 8) = q;
        }
        for (uint32_t i = head + body * 8 + threadIdx.x; i < c.len; i += blockDim.x) dst[i] = src[i];
    }
}

// ---------------------------------------------------------------- resolution

constexpr int R1_THREADS = 512;
constexpr int TILE = 2048;  // positions per tile: 4 per thread
constexpr int TPT = TILE / R1_THREADS;
constexpr uint16_t PENDING = 0xFFFF;

// pass 1: every span resolved on its own (see the file comment). Position i of a tile belongs to
// thread i % R1_THREADS (consecutive threads, consecutive positions: coalesced loads and stores,
// no shared-memory bank conflicts). The span's pieces are staged in shared memory once, by all
// threads, when there are at most SPAN_PIECES of them (else each thread searches the span's range
// of the global list). Blocks take spans from a queue (`work`, zero at launch).
constexpr int SPAN_PIECES = 512;

// the piece holding position p among list[0 .. n) (sorted, back to back, list[0].dst <= p)
__device__ __forceinline__ int piece_at(const Piece* list, int n, uint64_t p) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (list[mid].dst <= p) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__global__ void __launch_bounds__(R1_THREADS, 4) k_local(const uint16_t* __restrict__ pool,
                                                         const Piece* __restrict__ pieces, int npieces,
                                                         const SpanDesc* __restrict__ spans, uint64_t nspans,
                                                         uint16_t* out16, int* bad, unsigned* work) {
    __shared__ uint16_t val[TILE];
    __shared__ uint16_t ptr[TILE];
    __shared__ Piece sp_pieces[SPAN_PIECES];
    __shared__ unsigned next_span;
    (void)npieces;
    uint64_t sp = blockIdx.x;
    while (sp < nspans) {
        const SpanDesc sd = spans[sp];
        const uint64_t s0 = sd.start, s1 = sd.end;
        const bool staged = sd.npiece <= (uint32_t)SPAN_PIECES;
        const Piece* list = staged ? sp_pieces : pieces + sd.piece0;
        const int nlist = (int)sd.npiece;
        __syncthreads();  // the previous span's threads are done with sp_pieces and next_span
        if (staged)
            for (int i = threadIdx.x; i < nlist; i += blockDim.x) sp_pieces[i] = pieces[sd.piece0 + i];
        if (threadIdx.x == 0) next_span = atomicAdd(work, 1u) + gridDim.x;
        int j = -1;  // this thread's current piece (its positions only move forward)
        uint64_t end = 0, delta = 0;
        for (uint64_t tb = s0; tb < s1; tb += TILE) {
            const int n = (int)(s1 - tb < (uint64_t)TILE ? s1 - tb : (uint64_t)TILE);
            const uint32_t t0 = (uint32_t)(tb - s0);
            __syncthreads();  // pieces staged; the previous tile's stores visible, its shared values read
#pragma unroll
            for (int k = 0; k < TPT; k++) {
                const int i = k * R1_THREADS + (int)threadIdx.x;
                if (i >= n) continue;
                const uint64_t p = tb + i;
                if (j < 0) {
                    j = piece_at(list, nlist, p);
                    end = list[j].dst + list[j].len;
                    delta = list[j].src - list[j].dst;  // pool index = position + delta
                }
                while (p >= end) {  // the next piece starts where this one ends
                    j++;
                    end = list[j].dst + list[j].len;
                    delta = list[j].src - list[j].dst;
                }
                const uint32_t v = pool[p + delta];
                // the next tile's symbols of this piece into L2 while this tile resolves (one
                // request per warp and step: the warp's 32 positions share a 64-byte line)
                if ((threadIdx.x & 31) == 0 && p + TILE < end) {
                    const uint16_t* nxt = pool + p + TILE + delta;
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(nxt));
                }
                uint32_t r = v, q = (uint32_t)i;
                if (v > REF) {
                    const int32_t src = (int32_t)(t0 + (uint32_t)i) - (int32_t)(v - REF);  // relative to s0
                    if (src < 0) {
                        if (src < -(int32_t)sd.W) {
                            bad[sd.stream] = 1;  // a match before the stream's start
                            r = 0;
                        } else {
                            r = (uint32_t)(256 + (int32_t)WINDOW + src);  // byte of the entry window
                        }
                    } else if ((uint32_t)src < t0) {
                        r = out16[s0 + (uint32_t)src];  // resolved in an earlier tile
                    } else {
                        r = PENDING;
                        q = (uint32_t)src - t0;
                    }
                }
                val[i] = (uint16_t)r;
                ptr[i] = (uint16_t)q;
            }
            __syncthreads();
            // copies inside the tile: pointer doubling until every chain reached a value
            for (int round = 0; round < TILE; round++) {
                int pend = 0;
#pragma unroll
                for (int k = 0; k < TPT; k++) {
                    const int i = k * R1_THREADS + (int)threadIdx.x;
                    if (i < n && val[i] == PENDING) {
                        const uint16_t qq = ptr[i];
                        const uint16_t vq = ((volatile uint16_t*)val)[qq];
                        if (vq != PENDING) {
                            val[i] = vq;
                        } else {
                            ptr[i] = ((volatile uint16_t*)ptr)[qq];
                            pend = 1;
                        }
                    }
                }
                if (!__syncthreads_or(pend)) break;
            }
#pragma unroll
            for (int k = 0; k < TPT; k++) {
                const int i = k * R1_THREADS + (int)threadIdx.x;
                if (i < n) out16[tb + i] = val[i];
            }
        }
        __syncthreads();
        sp = next_span;
    }
}

// pass 2: the entry window of every span. window[s+1] = M_s(window[s]), where M_s is span s's
// last 32 KiB of pass-1 values (a byte, or 256 + an index into window[s]). The chain over spans
// is a scan over these gather maps, done in three phases over groups of L spans:
//   compose: per group, C_g = M_{gL+L-1} o ... o M_{gL} (maps compose into a map of the same form);
//   chain:   one block walks the groups: window[(g+1)L] = C_g(window[gL]);
//   fill:    per group, window[gL+1 .. gL+L-1] one after the other from window[gL].
// Serial steps: 2L + G instead of the span count. Each thread owns 32 consecutive positions.
constexpr int WT = 1024;               // threads of the window kernels
constexpr int WPER = WINDOW / WT;      // 32 positions per thread

__device__ __forceinline__ void load_map(const uint16_t* src, uint16_t (&v)[WPER]) {
    const uint4* p = (const uint4*)(src + threadIdx.x * WPER);
#pragma unroll
    for (int q = 0; q < 4; q++) {
        uint4 x = p[q];
        uint32_t w[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
        for (int k = 0; k < 4; k++) {
            v[q * 8 + 2 * k] = (uint16_t)(w[k] & 0xffff);
            v[q * 8 + 2 * k + 1] = (uint16_t)(w[k] >> 16);
        }
    }
}

// C_g for every group (one block per group); maps[g] gets the composed map
__global__ void __launch_bounds__(WT) k_compose(const uint16_t* __restrict__ out16, uint64_t nmaps, uint64_t span,
                                                uint64_t L, uint16_t* __restrict__ maps) {
    extern __shared__ __align__(16) uint16_t R[];  // the running composition
    const uint64_t g = blockIdx.x, m0 = g * L, m1 = m0 + L < nmaps ? m0 + L : nmaps;
    uint16_t v[WPER];
    load_map(out16 + (m0 + 1) * span - WINDOW, v);
#pragma unroll
    for (int k = 0; k < WPER; k++) R[threadIdx.x * WPER + k] = v[k];
    __syncthreads();
    for (uint64_t m = m0 + 1; m < m1; m++) {
        load_map(out16 + (m + 1) * span - WINDOW, v);
#pragma unroll
        for (int k = 0; k < WPER; k++) v[k] = v[k] < 256 ? v[k] : R[v[k] - 256];
        __syncthreads();
#pragma unroll
        for (int k = 0; k < WPER; k++) R[threadIdx.x * WPER + k] = v[k];
        __syncthreads();
    }
    uint4* dst = (uint4*)(maps + g * WINDOW + threadIdx.x * WPER);
    const uint4* srcv = (const uint4*)(R + threadIdx.x * WPER);
#pragma unroll
    for (int q = 0; q < 4; q++) dst[q] = srcv[q];
}

// applies a map to a window in shared memory (in place across a barrier), and stores the result
__device__ __forceinline__ void apply_map(const uint16_t (&v)[WPER], uint8_t* win, uint8_t* out_global) {
    uint8_t b[WPER];
#pragma unroll
    for (int k = 0; k < WPER; k++) b[k] = v[k] < 256 ? (uint8_t)v[k] : win[v[k] - 256];
    __syncthreads();
    uint32_t pk[WPER / 4];
#pragma unroll
    for (int k = 0; k < WPER / 4; k++)
        pk[k] = (uint32_t)b[4 * k] | (uint32_t)b[4 * k + 1] << 8 | (uint32_t)b[4 * k + 2] << 16 | (uint32_t)b[4 * k + 3] << 24;
    uint4* ws = (uint4*)(win + threadIdx.x * WPER);
    uint4* wg = (uint4*)(out_global + threadIdx.x * WPER);
    ws[0] = wg[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
    ws[1] = wg[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
    __syncthreads();
}

// window[0] from the segment's window, then window[gL] for every group (one block)
__global__ void __launch_bounds__(WT) k_chain(const uint16_t* __restrict__ maps, uint64_t ngroups, uint64_t L,
                                              uint64_t nspans, const uint8_t* __restrict__ seg_window, uint32_t W,
                                              uint8_t* __restrict__ windows) {
    __shared__ __align__(16) uint8_t win[WINDOW];
    for (int j = threadIdx.x; j < (int)WINDOW; j += WT) {
        uint8_t b = j >= (int)(WINDOW - W) ? seg_window[j - (WINDOW - W)] : 0;
        win[j] = b;
        windows[j] = b;
    }
    __syncthreads();
    for (uint64_t g = 0; g + 1 < ngroups && (g + 1) * L < nspans; g++) {
        uint16_t v[WPER];
        load_map(maps + g * WINDOW, v);
        apply_map(v, win, windows + (g + 1) * L * WINDOW);
    }
}

// window[gL+1 .. gL+L-1] (one block per group)
__global__ void __launch_bounds__(WT) k_fill(const uint16_t* __restrict__ out16, uint64_t nspans, uint64_t span,
                                             uint64_t L, uint8_t* __restrict__ windows) {
    __shared__ __align__(16) uint8_t win[WINDOW];
    const uint64_t s0 = blockIdx.x * L;
    const uint4* src = (const uint4*)(windows + s0 * WINDOW + threadIdx.x * WPER);
    uint4* ws = (uint4*)(win + threadIdx.x * WPER);
    ws[0] = src[0];
    ws[1] = src[1];
    __syncthreads();
    for (uint64_t s = s0 + 1; s < s0 + L && s < nspans; s++) {
        uint16_t v[WPER];
        load_map(out16 + s * span - WINDOW, v);
        apply_map(v, win, windows + s * WINDOW);
    }
}

// pass 3: bytes, 16 per thread per step; a block per span (span starts are multiples of 16)
__global__ void k_final(const uint16_t* __restrict__ out16, const SpanDesc* __restrict__ spans, uint64_t nspans,
                        const uint8_t* __restrict__ windows, uint8_t* __restrict__ out) {
    for (uint64_t sp = blockIdx.x; sp < nspans; sp += gridDim.x) {
        const SpanDesc sd = spans[sp];
        const uint8_t* win = windows + sp * WINDOW;
        for (uint64_t i = sd.start + (uint64_t)threadIdx.x * 16; i < sd.end; i += (uint64_t)blockDim.x * 16) {
            if (i + 16 <= sd.end) {
                const uint4* src = (const uint4*)(out16 + i);
                uint4 a = src[0], b = src[1];
                uint32_t w[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
                uint32_t q[4];
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    uint32_t lo = w[2 * k] & 0xffff, hi = w[2 * k] >> 16, lo2 = w[2 * k + 1] & 0xffff,
                             hi2 = w[2 * k + 1] >> 16;
                    uint32_t b0 = lo < 256 ? lo : win[lo - 256];
                    uint32_t b1 = hi < 256 ? hi : win[hi - 256];
                    uint32_t b2 = lo2 < 256 ? lo2 : win[lo2 - 256];
                    uint32_t b3 = hi2 < 256 ? hi2 : win[hi2 - 256];
                    q[k] = b0 | b1 << 8 | b2 << 16 | b3 << 24;
                }
                *(uint4*)(out + i) = make_uint4(q[0], q[1], q[2], q[3]);
            } else {
                for (uint64_t k = i; k < sd.end; k++) {
                    uint32_t v = out16[k];
                    out[k] = v < 256 ? (uint8_t)v : win[v - 256];
                }
            }
        }
    }
}

// Entry windows of the spans of many streams (the batched form): a block per stream with more
// than one span walks its spans in order; window[first] is not read (nothing reaches before a
// stream's start without being invalid).
__global__ void __launch_bounds__(WT) k_chain_streams(const uint16_t* __restrict__ out16,
                                                      const SpanDesc* __restrict__ spans,
                                                      const uint32_t* __restrict__ multi, uint32_t nmulti,
                                                      uint8_t* __restrict__ windows) {
    __shared__ __align__(16) uint8_t win[WINDOW];
    for (uint32_t m = blockIdx.x; m < nmulti; m += gridDim.x) {
        const uint32_t first = multi[2 * m], count = multi[2 * m + 1];
        for (int j = threadIdx.x; j < (int)WINDOW; j += WT) win[j] = 0;
        __syncthreads();
        for (uint32_t s = first + 1; s < first + count; s++) {
            uint16_t v[WPER];
            load_map(out16 + spans[s - 1].end - WINDOW, v);
            apply_map(v, win, windows + (uint64_t)s * WINDOW);
        }
        __syncthreads();
    }
}

// The same scan per long stream of the batched form (groups never cross streams): the composed
// map of every group but each stream's last, then a block per stream walks its groups, then a
// block per group fills the windows inside it. A span's map is the last WINDOW values of the span.
__global__ void __launch_bounds__(WT) k_compose_groups(const uint16_t* __restrict__ out16,
                                                       const SpanDesc* __restrict__ spans,
                                                       const SpanGroup* __restrict__ groups, uint32_t ngroups,
                                                       uint16_t* __restrict__ maps) {
    extern __shared__ __align__(16) uint16_t R[];
    for (uint32_t gi = blockIdx.x; gi < ngroups; gi += gridDim.x) {
        const SpanGroup gr = groups[gi];
        if (gr.map == UINT32_MAX) continue;  // a stream's last group: its map is never used
        uint16_t v[WPER];
        load_map(out16 + spans[gr.first_span].end - WINDOW, v);
#pragma unroll
        for (int k = 0; k < WPER; k++) R[threadIdx.x * WPER + k] = v[k];
        __syncthreads();
        for (uint32_t s = gr.first_span + 1; s < gr.first_span + gr.count; s++) {
            load_map(out16 + spans[s].end - WINDOW, v);
#pragma unroll
            for (int k = 0; k < WPER; k++) v[k] = v[k] < 256 ? v[k] : R[v[k] - 256];
            __syncthreads();
#pragma unroll
            for (int k = 0; k < WPER; k++) R[threadIdx.x * WPER + k] = v[k];
            __syncthreads();
        }
        uint4* dst = (uint4*)(maps + (uint64_t)gr.map * WINDOW + threadIdx.x * WPER);
        const uint4* srcv = (const uint4*)(R + threadIdx.x * WPER);
#pragma unroll
        for (int q = 0; q < 4; q++) dst[q] = srcv[q];
        __syncthreads();
    }
}

__global__ void __launch_bounds__(WT) k_chain_groups(const SpanGroup* __restrict__ groups,
                                                     const GroupedStream* __restrict__ grouped, uint32_t ngrouped,
                                                     const uint16_t* __restrict__ maps, uint8_t* __restrict__ windows) {
    __shared__ __align__(16) uint8_t win[WINDOW];
    for (uint32_t m = blockIdx.x; m < ngrouped; m += gridDim.x) {
        const GroupedStream gs = grouped[m];
        uint8_t* w0 = windows + (uint64_t)groups[gs.first_group].first_span * WINDOW;
        for (int j = threadIdx.x; j < (int)WINDOW; j += WT) win[j] = w0[j] = 0;
        __syncthreads();
        for (uint32_t g = gs.first_group; g + 1 < gs.first_group + gs.ngroups; g++) {
            uint16_t v[WPER];
            load_map(maps + (uint64_t)groups[g].map * WINDOW, v);
            apply_map(v, win, windows + (uint64_t)groups[g + 1].first_span * WINDOW);
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(WT) k_fill_groups(const uint16_t* __restrict__ out16,
                                                    const SpanDesc* __restrict__ spans,
                                                    const SpanGroup* __restrict__ groups, uint32_t ngroups,
                                                    uint8_t* __restrict__ windows) {
    __shared__ __align__(16) uint8_t win[WINDOW];
    for (uint32_t gi = blockIdx.x; gi < ngroups; gi += gridDim.x) {
        const SpanGroup gr = groups[gi];
        const uint4* src = (const uint4*)(windows + (uint64_t)gr.first_span * WINDOW + threadIdx.x * WPER);
        uint4* ws = (uint4*)(win + threadIdx.x * WPER);
        ws[0] = src[0];
        ws[1] = src[1];
        __syncthreads();
        for (uint32_t s = gr.first_span + 1; s < gr.first_span + gr.count; s++) {
            uint16_t v[WPER];
            load_map(out16 + spans[s - 1].end - WINDOW, v);
            apply_map(v, win, windows + (uint64_t)s * WINDOW);
        }
        __syncthreads();
    }
}

// the window for the next segment: the last 32 KiB of (old window ++ this segment's output)
__global__ void k_next_window(const uint8_t* __restrict__ out, uint64_t total, const uint8_t* __restrict__ old,
                              uint32_t W, uint8_t* __restrict__ nw, uint32_t newW) {
    uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= newW) return;
    int64_t pos = (int64_t)total - (int64_t)newW + j;  // in this segment's output; negative: in the old window
    nw[j] = pos >= 0 ? out[pos] : old[(int64_t)W + pos];
}

// ---------------------------------------------------------------- CRC-32

__device__ __forceinline__ uint32_t mulmod(uint32_t a, uint32_t b) {
    uint32_t p = 0;
#pragma unroll 4
    for (int i = 0; i < 32; i++) {
        if (a & (0x80000000u >> i)) p ^= b;
        b = (b & 1) ? (b >> 1) ^ POLY : b >> 1;
    }
    return p;
}

struct CrcConsts {
    uint32_t lane[5];   // x^(8 * 128 * 2^k): merging lane CRCs
    uint32_t level[12]; // x^(8 * 4096 * 1024^L * 2^k) for the tree levels (k = 0..9) of level L, per call
};

__device__ __forceinline__ uint32_t crc_bytes(const uint32_t* table, const uint8_t* p, int n, uint32_t c) {
    for (int i = 0; i < n; i++) c = table[(c ^ p[i]) & 255] ^ (c >> 8);
    return c;
}

// CRC-32 of every full 4 KiB tile of data[0..ntiles*4096)
__global__ void k_crc_tiles(const uint8_t* __restrict__ data, uint64_t ntiles, uint32_t* __restrict__ out,
                            CrcConsts k) {
    __shared__ uint32_t table[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) {
        uint32_t c = (uint32_t)i;
        for (int b = 0; b < 8; b++) c = c & 1 ? POLY ^ (c >> 1) : c >> 1;
        table[i] = c;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t t = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); t < ntiles; t += warps) {
        const uint4* p = (const uint4*)(data + t * 4096 + lane * 128);
        uint32_t c = 0xffffffffu;
#pragma unroll 2
        for (int q = 0; q < 8; q++) {
            uint4 v = p[q];
            uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int j = 0; j < 4; j++) {
                c = table[(c ^ w[j]) & 255] ^ (c >> 8);
                c = table[(c ^ (w[j] >> 8)) & 255] ^ (c >> 8);
                c = table[(c ^ (w[j] >> 16)) & 255] ^ (c >> 8);
                c = table[(c ^ (w[j] >> 24)) & 255] ^ (c >> 8);
            }
        }
        c = ~c;
        // merge neighbours: lane i (multiple of 2^(s+1)) takes lane i + 2^s
#pragma unroll
        for (int s = 0; s < 5; s++) {
            uint32_t other = __shfl_down_sync(0xffffffffu, c, 1 << s);
            if ((lane & ((2 << s) - 1)) == 0) c = mulmod(c, k.lane[s]) ^ other;
        }
        if (lane == 0) out[t] = c;
    }
}

// One tree level: merges groups of 1024 consecutive CRCs (each of an item of equal size; the
// item count is padded at the FRONT with empty items, so every right-hand operand is full-size
// and its multiplier a constant). mult[s] = x^(8 * item_bytes * 2^s).
__global__ void k_crc_merge(const uint32_t* __restrict__ in, uint64_t n, uint32_t* __restrict__ out, CrcConsts k) {
    __shared__ uint32_t v[1024];
    uint64_t groups = (n + 1023) / 1024;
    uint64_t pad = groups * 1024 - n;
    for (uint64_t g = blockIdx.x; g < groups; g += gridDim.x) {
        for (int i = threadIdx.x; i < 1024; i += blockDim.x) {
            uint64_t vi = g * 1024 + i;
            v[i] = vi < pad ? 0u : in[vi - pad];
        }
        __syncthreads();
        for (int s = 0; s < 10; s++) {
            int step = 1 << s;
            for (int i = threadIdx.x * (2 * step); i < 1024; i += blockDim.x * (2 * step))
                v[i] = mulmod(v[i], k.level[s]) ^ v[i + step];
            __syncthreads();
        }
        if (threadIdx.x == 0) out[g] = v[0];
        __syncthreads();
    }
}

// the tail (under 4 KiB) after the full tiles, by one thread, merged with the full part
__global__ void k_crc_tail(const uint8_t* data, uint64_t full_bytes, uint32_t tail, const uint32_t* full_crc,
                           uint32_t x8tail, uint32_t* result) {
    __shared__ uint32_t table[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) {
        uint32_t c = (uint32_t)i;
        for (int b = 0; b < 8; b++) c = c & 1 ? POLY ^ (c >> 1) : c >> 1;
        table[i] = c;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    uint32_t c = ~crc_bytes(table, data + full_bytes, (int)tail, 0xffffffffu);
    uint32_t a = full_bytes ? *full_crc : 0u;
    *result = tail ? mulmod(a, x8tail) ^ c : a;
}

// CRC-32 of many streams (the batched form): span CRCs (k_crc_spans), then stream CRCs
// (k_crc_streams); lengths that are not a constant of the launch take x^(8n) by square-and-multiply
// over the table below.
__constant__ uint32_t c_x8pow[48];  // x^(8 * 2^k) mod P

__device__ uint32_t x8n_dev(uint64_t n) {
    uint32_t p = 1u << 31;  // x^0
    for (int k = 0; n; k++, n >>= 1)
        if (n & 1) p = mulmod(p, c_x8pow[k]);
    return p;
}

__device__ __forceinline__ uint32_t crc_combine_dev(uint32_t a, uint32_t b, uint64_t len_b) {
    return len_b ? mulmod(a, x8n_dev(len_b)) ^ b : a;
}

// CRC-32 of every span of the batched form: a block per span, whose warps take the span's 4 KiB
// tiles in turn (32 lanes x 128 contiguous bytes, merged with constant multipliers, as
// k_crc_tiles), a partial last tile lane by lane with x^(8n) for its lengths; thread 0 then merges
// the tile CRCs in order (x^(8*4096) for every full tile).
__global__ void __launch_bounds__(256) k_crc_spans(const uint8_t* __restrict__ data, const SpanDesc* __restrict__ spans,
                                                    uint64_t nspans, uint32_t* __restrict__ span_crc, CrcConsts k,
                                                    uint32_t x4096) {
    __shared__ uint32_t table[256];
    __shared__ uint32_t tcrc[SPAN / 4096];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) {
        uint32_t c = (uint32_t)i;
        for (int b = 0; b < 8; b++) c = c & 1 ? POLY ^ (c >> 1) : c >> 1;
        table[i] = c;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (uint64_t sp = blockIdx.x; sp < nspans; sp += gridDim.x) {
        const SpanDesc sd = spans[sp];
        const uint64_t len = sd.end - sd.start;  // at most SPAN; the start is 16-byte aligned
        const uint32_t nfull = (uint32_t)(len / 4096), tail = (uint32_t)(len % 4096);
        const uint32_t ntiles = nfull + (tail != 0);
        for (uint32_t t = w; t < ntiles; t += 8) {
            const uint8_t* base = data + sd.start + (uint64_t)t * 4096;
            uint32_t c;
            if (t < nfull) {
                const uint4* p = (const uint4*)(base + lane * 128);
                c = 0xffffffffu;
#pragma unroll 2
                for (int q = 0; q < 8; q++) {
                    uint4 v = p[q];
                    uint32_t wv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        c = table[(c ^ wv[j]) & 255] ^ (c >> 8);
                        c = table[(c ^ (wv[j] >> 8)) & 255] ^ (c >> 8);
                        c = table[(c ^ (wv[j] >> 16)) & 255] ^ (c >> 8);
                        c = table[(c ^ (wv[j] >> 24)) & 255] ^ (c >> 8);
                    }
                }
                c = ~c;
#pragma unroll
                for (int s = 0; s < 5; s++) {
                    uint32_t other = __shfl_down_sync(0xffffffffu, c, 1 << s);
                    if ((lane & ((2 << s) - 1)) == 0) c = mulmod(c, k.lane[s]) ^ other;
                }
            } else {
                const uint32_t a = lane * 128 < tail ? lane * 128 : tail;
                const uint32_t b = lane * 128 + 128 < tail ? lane * 128 + 128 : tail;
                uint32_t cl = ~crc_bytes(table, base + a, (int)(b - a), 0xffffffffu);
                if (b == a) cl = 0;
                c = 0;
                for (int l = 0; l < 32; l++) {
                    uint32_t x = __shfl_sync(0xffffffffu, cl, l);
                    uint32_t n = __shfl_sync(0xffffffffu, b - a, l);
                    if (lane == 0) c = crc_combine_dev(c, x, n);
                }
            }
            if (lane == 0) tcrc[t] = c;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t acc = 0;
            for (uint32_t t = 0; t < nfull; t++) acc = mulmod(acc, x4096) ^ tcrc[t];
            if (tail) acc = crc_combine_dev(acc, tcrc[nfull], tail);
            span_crc[sp] = acc;
        }
        __syncthreads();
    }
}

// a thread per stream merges its spans' CRCs in order: every span but the last is SPAN bytes
__global__ void k_crc_streams(const SpanDesc* __restrict__ spans, const uint32_t* __restrict__ span_crc,
                              const uint32_t* __restrict__ first_span, const uint32_t* __restrict__ span_count,
                              uint32_t nstreams, uint32_t xspan, uint32_t* __restrict__ crc) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nstreams) return;
    uint32_t c = 0;
    for (uint32_t k = first_span[s]; k < first_span[s] + span_count[s]; k++) {
        const uint64_t len = spans[k].end - spans[k].start;
        c = len == SPAN ? mulmod(c, xspan) ^ span_crc[k] : crc_combine_dev(c, span_crc[k], len);
    }
    crc[s] = c;
}

}  // namespace

// ---------------------------------------------------------------- host side

void span_pieces(SpanDesc* spans, uint64_t nspans, const Piece* pieces, uint64_t npieces) {
    uint64_t p = 0;
    for (uint64_t k = 0; k < nspans; k++) {
        while (p < npieces && pieces[p].dst + pieces[p].len <= spans[k].start) p++;
        uint64_t q = p;
        while (q < npieces && pieces[q].dst < spans[k].end) q++;
        spans[k].piece0 = (uint32_t)p;
        spans[k].npiece = (uint32_t)(q - p);
    }
}

static uint32_t mulmod_host(uint32_t a, uint32_t b) {
    uint32_t p = 0;
    for (int i = 0; i < 32; i++) {
        if (a & (0x80000000u >> i)) p ^= b;
        b = (b & 1) ? (b >> 1) ^ POLY : b >> 1;
    }
    return p;
}

// x^(8n) mod P
static uint32_t x8n_host(uint64_t n) {
    uint32_t sq = 1u << 30;  // x^1
    uint32_t p = 1u << 31;   // x^0
    uint64_t e = n;          // exponent 8n = n << 3: start from x^8
    for (int i = 0; i < 3; i++) sq = mulmod_host(sq, sq);
    while (e) {
        if (e & 1) p = mulmod_host(p, sq);
        sq = mulmod_host(sq, sq);
        e >>= 1;
    }
    return p;
}

uint32_t crc32_combine_host(uint32_t crc1, uint32_t crc2, uint64_t len2) {
    return mulmod_host(crc1, x8n_host(len2)) ^ crc2;
}

// words launch_crc writes: one CRC per 4 KiB tile, then one per 1024 of the level below until one
// is left
uint64_t crc_scratch_words(uint64_t n) {
    uint64_t level = n / 4096, words = level;
    while (level > 1) {
        level = (level + 1023) / 1024;
        words += level;
    }
    return words + 4;
}

int crc_prepare() {
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, k_crc_tiles);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_crc_merge);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_crc_tail);
    return (int)e;
}

int sm_count() {
    static std::atomic<int> counts[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return 1;
    if (dev < 64 && counts[dev].load(std::memory_order_relaxed) > 0) return counts[dev].load(std::memory_order_relaxed);
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) n = 1;
    if (dev < 64) counts[dev].store(n, std::memory_order_relaxed);
    return n;
}

int launch_crc(const uint8_t* data, uint64_t n, uint32_t* scratch, uint64_t scratch_words, uint32_t* result,
               void* stream) {
    if (scratch_words < crc_scratch_words(n)) return -1;
    int launches = 1;
    cudaStream_t st = (cudaStream_t)stream;
    CrcConsts k{};
    for (int s = 0; s < 5; s++) k.lane[s] = x8n_host(128ull << s);
    uint64_t ntiles = n / 4096;
    uint32_t* cur = scratch;
    uint64_t cnt = ntiles;
    uint64_t item = 4096;
    if (ntiles) {
        unsigned grid = (unsigned)((ntiles + 7) / 8);
        const unsigned cap = (unsigned)sm_count() * 16;
        if (grid > cap) grid = cap;
        k_crc_tiles<<<grid, 256, 0, st>>>(data, ntiles, cur, k);
        launches++;
        while (cnt > 1) {
            for (int s = 0; s < 10; s++) k.level[s] = x8n_host(item << s);
            uint64_t groups = (cnt + 1023) / 1024;
            uint32_t* nxt = cur + cnt;
            k_crc_merge<<<(unsigned)(groups < 4096 ? groups : 4096), 512, 0, st>>>(cur, cnt, nxt, k);
            launches++;
            cur = nxt;
            cnt = groups;
            item *= 1024;
        }
    }
    uint32_t tail = (uint32_t)(n - ntiles * 4096);
    k_crc_tail<<<1, 256, 0, st>>>(data, ntiles * 4096, tail, cur, x8n_host(tail), result);
    return launches;
}

// ---------------------------------------------------------------- gather

// a block per piece: 16-byte loads and stores where source and destination agree modulo 16,
// 4-byte ones where they agree modulo 4, bytes otherwise (the destination offsets are 4 KiB-aligned)
__global__ void k_gather(const GatherPiece* __restrict__ pieces, uint64_t n, uint8_t* __restrict__ dst) {
    for (uint64_t b = blockIdx.x; b < n; b += gridDim.x) {
        const GatherPiece pc = pieces[b];
        const uint8_t* src = pc.src;
        uint8_t* d = dst + pc.dst;
        const uint64_t len = pc.len;
        const uintptr_t mis = ((uintptr_t)src ^ (uintptr_t)d);
        if ((mis & 15) == 0) {
            const uint64_t head = ((16 - ((uintptr_t)d & 15)) & 15) < len ? ((16 - ((uintptr_t)d & 15)) & 15) : len;
            if (threadIdx.x < head) d[threadIdx.x] = src[threadIdx.x];
            const uint64_t body = (len - head) / 16;
            const uint4* s4 = (const uint4*)(src + head);
            uint4* d4 = (uint4*)(d + head);
            for (uint64_t i = threadIdx.x; i < body; i += blockDim.x) d4[i] = s4[i];
            for (uint64_t i = head + body * 16 + threadIdx.x; i < len; i += blockDim.x) d[i] = src[i];
        } else if ((mis & 3) == 0) {
            const uint64_t head = ((4 - ((uintptr_t)d & 3)) & 3) < len ? ((4 - ((uintptr_t)d & 3)) & 3) : len;
            if (threadIdx.x < head) d[threadIdx.x] = src[threadIdx.x];
            const uint64_t body = (len - head) / 4;
            const uint32_t* s4 = (const uint32_t*)(src + head);
            uint32_t* d4 = (uint32_t*)(d + head);
            for (uint64_t i = threadIdx.x; i < body; i += blockDim.x) d4[i] = s4[i];
            for (uint64_t i = head + body * 4 + threadIdx.x; i < len; i += blockDim.x) d[i] = src[i];
        } else {
            for (uint64_t i = threadIdx.x; i < len; i += blockDim.x) d[i] = src[i];
        }
    }
}

int launch_gather(const GatherPiece* pieces, uint64_t n, uint8_t* dst, void* stream) {
    if (!n) return 0;
    const uint64_t cap = (uint64_t)sm_count() * 8;
    uint64_t grid = n < cap ? n : cap;
    k_gather<<<(unsigned)grid, 256, 0, (cudaStream_t)stream>>>(pieces, n, dst);
    return 1;
}

int launch_stored(const uint8_t* d_in, uint16_t* pool, const StoredCopy* list, int n, void* stream) {
    if (n <= 0) return 0;
    k_stored<<<n < 65535 ? n : 65535, 256, 0, (cudaStream_t)stream>>>(d_in, pool, list, n);
    return 1;
}

// k_local's grid: as many blocks as fit on the GPU at once (they take spans from a queue)
static unsigned local_grid(uint64_t nspans) {
    int dev = 0, nsm = 1, per_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_local, R1_THREADS, 0) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    uint64_t g = (uint64_t)nsm * (uint64_t)per_sm;
    return (unsigned)(nspans < g ? nspans : g);
}

uint64_t span_length(uint64_t total) {
    uint64_t s = SPAN;
    while (s > (64u << 10) && (total + s - 1) / s < (uint64_t)sm_count()) s >>= 1;
    return s;
}

int launch_resolve(const uint16_t* pool, const Piece* pieces, int npieces, const SpanDesc* spans, uint64_t nspans,
                   uint64_t span_len, uint64_t total, uint32_t W, const uint8_t* seg_window, uint16_t* out16,
                   uint8_t* windows, int* bad, uint8_t* out, int passes, unsigned* work, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (!total || npieces <= 0) return 0;
    int launches = 0;
    int dev = 0, nsm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (passes & 1) {
        cudaMemsetAsync(work, 0, sizeof(unsigned), st);
        k_local<<<local_grid(nspans), R1_THREADS, 0, st>>>(pool, pieces, npieces, spans, nspans, out16, bad, work);
        launches++;
    }
    if (passes & 2) {
        // one stream, spans of span_len: groups of L spans, L about sqrt(spans) balances the three phases
        uint64_t L = 1;
        while (L * L < nspans) L++;
        uint64_t ngroups = (nspans + L - 1) / L;
        uint64_t nmaps = nspans - 1;  // M_s for s < nspans - 1
        uint16_t* maps = out16 + ((total + 63) & ~63ull);
        if (nmaps) {
            k_compose<<<(unsigned)((nmaps + L - 1) / L), WT, 2 * WINDOW, st>>>(out16, nmaps, span_len, L, maps);
            launches++;
        }
        k_chain<<<1, WT, 0, st>>>(maps, ngroups, L, nspans, seg_window, W, windows);
        k_fill<<<(unsigned)ngroups, WT, 0, st>>>(out16, nspans, span_len, L, windows);
        uint64_t fgrid = nspans < (uint64_t)nsm * 8 ? nspans : (uint64_t)nsm * 8;
        k_final<<<(unsigned)fgrid, 256, 0, st>>>(out16, spans, nspans, windows, out);
        launches += 3;
    }
    return launches;
}

int launch_resolve_streams(const uint16_t* pool, const Piece* pieces, int npieces, const SpanDesc* spans,
                           uint64_t nspans, const StreamWindows& sw, uint16_t* out16, uint8_t* windows, int* bad,
                           uint8_t* out, int passes, unsigned* work, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (!nspans || npieces <= 0) return 0;
    int launches = 0;
    int dev = 0, nsm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (passes & 1) {
        cudaMemsetAsync(work, 0, sizeof(unsigned), st);
        k_local<<<local_grid(nspans), R1_THREADS, 0, st>>>(pool, pieces, npieces, spans, nspans, out16, bad, work);
        launches++;
    }
    if (passes & 2) {
        const uint32_t cap = (uint32_t)nsm * 2;
        if (sw.nmulti) {
            k_chain_streams<<<sw.nmulti < cap ? sw.nmulti : cap, WT, 0, st>>>(out16, spans, sw.multi, sw.nmulti,
                                                                              windows);
            launches++;
        }
        if (sw.ngrouped) {
            k_compose_groups<<<sw.ngroups < cap ? sw.ngroups : cap, WT, 2 * WINDOW, st>>>(out16, spans, sw.groups,
                                                                                         sw.ngroups, sw.maps);
            k_chain_groups<<<sw.ngrouped < cap ? sw.ngrouped : cap, WT, 0, st>>>(sw.groups, sw.grouped, sw.ngrouped,
                                                                                 sw.maps, windows);
            k_fill_groups<<<sw.ngroups < cap ? sw.ngroups : cap, WT, 0, st>>>(out16, spans, sw.groups, sw.ngroups,
                                                                             windows);
            launches += 3;
        }
        uint64_t fgrid = nspans < (uint64_t)nsm * 8 ? nspans : (uint64_t)nsm * 8;
        k_final<<<(unsigned)fgrid, 256, 0, st>>>(out16, spans, nspans, windows, out);
        launches++;
    }
    return launches;
}

int resolve_setup() {
    uint32_t pw[48];
    for (int k = 0; k < 48; k++) pw[k] = x8n_host(1ull << k);
    cudaError_t e = cudaMemcpyToSymbol(c_x8pow, pw, sizeof pw);
    if (e != cudaSuccess) return (int)e;
    e = cudaFuncSetAttribute(k_compose, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * WINDOW);
    if (e != cudaSuccess) return (int)e;
    return (int)cudaFuncSetAttribute(k_compose_groups, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * WINDOW);
}

int launch_crc_streams(const uint8_t* data, const SpanDesc* spans, uint64_t nspans, uint32_t* span_crc,
                       const uint32_t* first_span, const uint32_t* span_count, uint32_t nstreams, uint32_t* crc,
                       void* stream) {
    if (!nstreams) return 0;
    cudaStream_t st = (cudaStream_t)stream;
    int launches = 0;
    CrcConsts k{};
    for (int s = 0; s < 5; s++) k.lane[s] = x8n_host(128ull << s);
    if (nspans) {
        const uint64_t cap = (uint64_t)sm_count() * 8;
        k_crc_spans<<<(unsigned)(nspans < cap ? nspans : cap), 256, 0, st>>>(data, spans, nspans, span_crc, k,
                                                                                     x8n_host(4096));
        launches++;
    }
    k_crc_streams<<<(nstreams + 255) / 256, 256, 0, st>>>(spans, span_crc, first_span, span_count, nstreams,
                                                          x8n_host(SPAN), crc);
    return launches + 1;
}

// 16-bit slots after the segment's symbols that hold the composed maps (one per group)
uint64_t resolve_map_slots(uint64_t seg_out_max) {
    uint64_t nspans = (seg_out_max + SPAN - 1) / SPAN + 1;
    uint64_t L = 1;
    while (L * L < nspans) L++;
    return 64 + ((nspans + L - 1) / L + 1) * WINDOW;
}

int launch_next_window(const uint8_t* out, uint64_t total, const uint8_t* old, uint32_t W, uint8_t* nw, uint32_t newW,
                       void* stream) {
    if (!newW) return 0;
    k_next_window<<<blocks_for(newW, 256), 256, 0, (cudaStream_t)stream>>>(out, total, old, W, nw, newW);
    return 1;
}

}  // namespace gz
