// gi_resolve.cu - from decoded symbols to bytes, and the CRC-32 of the bytes.
//
// The resolution scheme is the reference's (gpuinflate/gpuinflate.cu:366-421): every output
// position becomes a 32-bit entry, either LIT | byte or the absolute position it copies (the
// 32 KiB window before the segment sits in front), a reference before the stream's start is
// invalid data, and pointer jumping (up to 8 hops per entry per round, in place, the unresolved
// entries carried to the next round in a list) resolves every chain.
// Stored blocks skipped by the decoders are copied here 16 bytes of output at a time.
// CRC-32 is computed from the output bytes: each warp takes 4 KiB (128 bytes per lane,
// bytewise table in shared memory), lane CRCs are merged by the GF(2) identity
//     crc(A || B) = crc(A) * x^(8|B|) mod P  xor  crc(B)
// (carry-less multiplication modulo the CRC polynomial), then 4 KiB CRCs are merged 1024 at a
// time by the same identity until one is left. The multipliers x^(8n) for the fixed sizes are
// computed on the host.
#include <cuda_runtime.h>

#include "gi_common.cuh"

namespace gz {
namespace {

constexpr int HOPS = 8;
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

// ---------------------------------------------------------------- entries

__global__ void k_window(uint32_t* e32, const uint8_t* window, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) e32[i] = LIT | window[i];
}

// every position of every piece as LIT | byte or the absolute position it copies. bad_limit:
// only references at output positions below it count as "before the start" (positions are
// counted from the window's start)
__global__ void k_absolute(const uint16_t* __restrict__ pool, const Piece* __restrict__ pieces, uint64_t W,
                           uint32_t* __restrict__ e32, int* bad, uint64_t bad_limit) {
    Piece p = pieces[blockIdx.y];
    uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < p.len; i += stride) {
        uint32_t v = pool[p.src + i];
        uint64_t pos = W + p.dst + i;
        uint32_t e = LIT | v;
        if (v > REF) {
            uint64_t d = v - REF;
            if (d <= pos) {
                e = (uint32_t)(pos - d);
            } else {
                e = LIT;
                if (pos < bad_limit) *bad = 1;
            }
        }
        e32[pos] = e;
    }
}

__device__ __forceinline__ uint32_t jump(const uint32_t* e32, uint32_t e) {
#pragma unroll 1
    for (int h = 0; h < HOPS && !(e & LIT); h++) e = e32[e];
    return e;
}

__global__ void k_jump(uint32_t* e32, uint64_t n, const uint32_t* list, uint32_t* next, unsigned* nnext, uint64_t cap) {
    uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    uint32_t i = list ? list[t] : (uint32_t)t;
    uint32_t e = e32[i];
    if (e & LIT) return;
    e = jump(e32, e);
    e32[i] = e;
    if (!(e & LIT)) {
        unsigned q = atomicAdd(nnext, 1u);
        if (q < cap) next[q] = i;
    }
}

// bytes of entries, 16 per thread
__global__ void k_narrow(const uint32_t* __restrict__ e32, uint64_t n, uint8_t* __restrict__ out) {
    uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint64_t i = t * 16;
    if (i + 16 <= n && ((uintptr_t)(out + i) & 15) == 0 && ((uintptr_t)(e32 + i) & 15) == 0) {
        const uint4* s = (const uint4*)(e32 + i);
        uint4 a = s[0], b = s[1], c = s[2], d = s[3];
        uint4 q;
        q.x = (a.x & 255) | (a.y & 255) << 8 | (a.z & 255) << 16 | (a.w & 255) << 24;
        q.y = (b.x & 255) | (b.y & 255) << 8 | (b.z & 255) << 16 | (b.w & 255) << 24;
        q.z = (c.x & 255) | (c.y & 255) << 8 | (c.z & 255) << 16 | (c.w & 255) << 24;
        q.w = (d.x & 255) | (d.y & 255) << 8 | (d.z & 255) << 16 | (d.w & 255) << 24;
        *(uint4*)(out + i) = q;
    } else {
        for (uint64_t k = i; k < n && k < i + 16; k++) out[k] = (uint8_t)e32[k];
    }
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

}  // namespace

// ---------------------------------------------------------------- host side

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

uint64_t crc_scratch_words(uint64_t n) {
    uint64_t t = n / 4096;
    uint64_t total = 0;
    while (t > 1) {
        total += t;
        t = (t + 1023) / 1024;
    }
    return total + 4;
}

int launch_crc(const uint8_t* data, uint64_t n, uint32_t* scratch, uint64_t scratch_words, uint32_t* result,
               void* stream) {
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
        if (grid > 152 * 16) grid = 152 * 16;
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
    (void)scratch_words;
    uint32_t tail = (uint32_t)(n - ntiles * 4096);
    k_crc_tail<<<1, 256, 0, st>>>(data, ntiles * 4096, tail, cur, x8n_host(tail), result);
    return launches;
}

int launch_stored(const uint8_t* d_in, uint16_t* pool, const StoredCopy* list, int n, void* stream) {
    if (n <= 0) return 0;
    k_stored<<<n < 65535 ? n : 65535, 256, 0, (cudaStream_t)stream>>>(d_in, pool, list, n);
    return 1;
}

int launch_absolute(const uint16_t* pool, const Piece* pieces, int npieces, uint64_t W, uint32_t* e32, int* bad,
                    uint64_t bad_limit, void* stream) {
    if (npieces <= 0) return 0;
    int launches = 0;
    // blockIdx.y: the piece; blockIdx.x strides over it
    for (int p0 = 0; p0 < npieces; p0 += 65535) {
        int np = npieces - p0 < 65535 ? npieces - p0 : 65535;
        dim3 grid(8, np);
        k_absolute<<<grid, 256, 0, (cudaStream_t)stream>>>(pool, pieces + p0, W, e32, bad, bad_limit);
        launches++;
    }
    return launches;
}

int launch_window(uint32_t* e32, const uint8_t* window, uint32_t W, void* stream) {
    if (!W) return 0;
    k_window<<<blocks_for(W, 256), 256, 0, (cudaStream_t)stream>>>(e32, window, W);
    return 1;
}

int launch_jump(uint32_t* e32, uint64_t n, const uint32_t* list, uint32_t* next, unsigned* nnext, uint64_t cap,
                void* stream) {
    if (!n) return 0;
    k_jump<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(e32, n, list, next, nnext, cap);
    return 1;
}

int launch_narrow(const uint32_t* e32, uint64_t n, uint8_t* out, void* stream) {
    if (!n) return 0;
    k_narrow<<<blocks_for((n + 15) / 16, 256), 256, 0, (cudaStream_t)stream>>>(e32, n, out);
    return 1;
}

}  // namespace gz
