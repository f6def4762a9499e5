// gi_decode.cu - the speculative decoders.
//
// Semantics per job follow the reference's Decoder::run (gpuinflate/inflate.cuh:474-581): start
// at a block header or inside a block, decode blocks (stored, fixed, dynamic) until the position
// at a block boundary equals a later target's bit (landing), the stream's final block ends, the
// stop bit is reached, or the data is invalid; write one 16-bit symbol per output byte, either the
// byte or REF + d for "the byte d back". Error classes and the points where the input end is
// checked are the reference's (inflate.cuh:432-441, :515-524, :536-546, :571).
//
// The execution model is this file's own. A decoder is a whole warp: all 32 lanes carry the same
// bit-reader state and take the same branches, so nothing diverges; the lanes are used where
// there is parallel work:
//   * tables: the canonical code is built by the warp (histogram, ranks by __match_any_sync,
//     one lookup entry per lane per step) into the warp's shared memory;
//   * output: lane i holds the symbol for position i of the current 32-symbol group, so every
//     group leaves in one 64-byte store, and long matches are written 256 symbols per
//     instruction with 16-byte stores;
//   * lookups: one 32-bit entry per code gives the literal, or a length/distance base with its
//     extra-bit count, so a match costs two shared-memory reads.
// A decoder whose extent fills takes a new one from the pool (an atomic on the pool's fill
// level), so no decode needs a second launch; the extent records the exact decoder state where
// it begins, so the host can cut a segment at any extent boundary.
// Warps take jobs from a device queue (longest first), the grid is persistent: one wave of
// blocks sized from the occupancy of this kernel.
#include <cuda_runtime.h>

#include "gi_common.cuh"

namespace gz {
namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int NWARPS = DECODE_WARPS;  // decoders per block
constexpr int LB = 10;     // literal/length lookup bits
constexpr int DB = 8;      // distance lookup bits
constexpr int CB = 7;      // code-length code lookup bits (its codes are at most 7 bits)

// lookup entry: bits 0-3 code length (0: longer than the lookup, or no code), 4-7 extra bits,
// 8-23 value (literal byte, length base, distance base, code-length symbol), 24-25 kind
constexpr uint32_t K_LIT = 0u << 24, K_LEN = 1u << 24, K_EOB = 2u << 24, K_BAD = 3u << 24;
constexpr uint32_t E_LONG = K_BAD;  // kind BAD with code length 0: take the slow path

struct Code {  // canonical code data for codes longer than the lookup
    uint16_t first[16];  // first code of each length (MSB-first numbering)
    uint16_t count[16];
    uint16_t offs[16];   // index of the first symbol of each length in syms
};

struct Job1 {
    uint64_t stop;
    uint64_t limit;     // min(stop, end_bit + 1): one comparison per symbol checks both
    uint64_t end_bit;
    uint64_t end_byte;
    const Start* tg;
    int t, tend;        // next target, end of the stream's targets
    uint64_t tbit;      // targets[t].bit, or UINT64_MAX
    int passed;         // block-start targets passed without landing (DecodeArgs.give_up)
    int give_up;        // 0: never
};

// per-warp shared memory: the decoder's tables, and the state of its current job that the hot loop
// does not touch (kept out of registers)
struct __align__(16) Tables {
    uint32_t lit[1 << LB];
    uint32_t dist[1 << DB];
    uint16_t lit_syms[288];
    uint16_t dist_syms[32];
    Code litc, distc, clc;
    uint16_t cl_syms[19];
    uint16_t running[16];
    uint8_t lens[320];
    uint8_t clh[1 << CB];  // (length << 5) | symbol
    int32_t state;         // which tables are loaded: 0 none, 1 fixed, 2 dynamic
    uint32_t pad;
    Job1 j;                // the job's limits and target cursor
    JobResult r;           // the job's result, written as it goes
};

__device__ const uint16_t c_lbase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                                         31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
__device__ const uint8_t c_lext[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
__device__ const uint16_t c_dbase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,    65,    97,    129,
                                         193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
__device__ const uint8_t c_dext[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
__device__ const uint8_t c_order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

enum Alphabet { A_LIT = 0, A_DIST = 1, A_CL = 2 };

// the lookup entry of symbol s (without its code length)
__device__ __forceinline__ uint32_t entry_of(int alphabet, int s) {
    if (alphabet == A_LIT) {
        if (s < 256) return K_LIT | ((uint32_t)s << 8);
        if (s == 256) return K_EOB;
        if (s < 286) return K_LEN | ((uint32_t)c_lbase[s - 257] << 8) | ((uint32_t)c_lext[s - 257] << 4);
        return K_BAD;
    }
    if (alphabet == A_DIST) {
        if (s < 30) return ((uint32_t)c_dbase[s] << 8) | ((uint32_t)c_dext[s] << 4);
        return K_BAD;
    }
    return (uint32_t)s << 8;
}

struct Built {
    int kraft;    // 0 complete, 1 incomplete, -1 over-subscribed
    int nonzero;  // codes
    int ones;     // codes of length 1
};

// Builds a canonical code from lens[0..n) (shared memory) with the whole warp: the lookup of
// `root` bits (entries for codes up to root bits; E_LONG elsewhere), and Code/syms for longer
// codes. The result is the same in every lane.
__device__ Built build_code(const uint8_t* lens, int n, int alphabet, int root, uint32_t* lut, uint8_t* lut8, Code& c,
                            uint16_t* syms, uint16_t* running, int lane) {
    // histogram
    if (lane < 16) c.count[lane] = 0;
    __syncwarp();
    for (int s0 = 0; s0 < n; s0 += 32) {
        int s = s0 + lane;
        int l = s < n ? lens[s] : -1;
        unsigned peers = __match_any_sync(FULL, l);
        int leader = __ffs(peers) - 1;
        if (lane == leader && l >= 0) c.count[l] += (uint16_t)__popc(peers);
        __syncwarp();
    }
    Built b;
    b.nonzero = n - c.count[0];
    b.ones = c.count[1];
    int left = 1;
    b.kraft = 0;
    for (int len = 1; len < 16; len++) {
        left = (left << 1) - c.count[len];
        if (left < 0) {
            b.kraft = -1;
            break;
        }
    }
    if (b.kraft < 0) return b;
    b.kraft = left > 0 ? 1 : 0;
    __syncwarp();
    if (lane == 0) {
        c.count[0] = 0;
        uint16_t off = 0, code = 0;
        for (int len = 1; len < 16; len++) {
            code = (uint16_t)((code + (len > 1 ? c.count[len - 1] : 0)) << 1);
            if (len == 1) code = 0;
            c.first[len] = code;
            c.offs[len] = off;
            off = (uint16_t)(off + c.count[len]);
        }
    }
    if (lane < 16) running[lane] = 0;
    __syncwarp();
    // symbols in canonical order (length, then symbol)
    for (int s0 = 0; s0 < n; s0 += 32) {
        int s = s0 + lane;
        int l = s < n ? lens[s] : 0;
        unsigned peers = __match_any_sync(FULL, l);
        int rank = __popc(peers & ((1u << lane) - 1));
        if (l) syms[c.offs[l] + running[l] + rank] = (uint16_t)s;
        __syncwarp();
        if (l && lane == 31 - __clz(peers)) running[l] += (uint16_t)__popc(peers);
        __syncwarp();
    }
    // lookup entries: every (code of length <= root, filler bits) pair
    const int size = 1 << root;
    if (lut8) {
        for (int i = lane; i < size; i += 32) lut8[i] = 0;
    } else {
        for (int i = lane; i < size; i += 32) lut[i] = E_LONG;
    }
    __syncwarp();
    int ebase[16];
    int e_total = 0;
#pragma unroll
    for (int len = 1; len < 16; len++) {
        ebase[len] = e_total;
        if (len <= root) e_total += c.count[len] << (root - len);
    }
    for (int e = lane; e < e_total; e += 32) {
        int len = 1;
        while (len < root && e >= ebase[len + 1]) len++;
        int rel = e - ebase[len];
        int r = rel >> (root - len);
        int fill = rel & ((1 << (root - len)) - 1);
        uint32_t j = ((uint32_t)(c.first[len] + r) << (root - len)) | (uint32_t)fill;  // MSB-first
        uint32_t idx = __brev(j) >> (32 - root);                                        // stream order
        int sym = syms[c.offs[len] + r];
        if (lut8)
            lut8[idx] = (uint8_t)((len << 5) | sym);
        else
            lut[idx] = entry_of(alphabet, sym) | (uint32_t)len;
    }
    __syncwarp();
    return b;
}

struct Ctx {
    DecodeArgs a;
    Tables* T;
    int lane;
};

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Bit reader, identical in every lane
struct Bits {
    const uint32_t* w;
    uint64_t end_word;
    uint64_t next;  // next word to load
    uint64_t buf;
    int cnt;

    __device__ __forceinline__ void refill1() {
        uint32_t v = next < end_word ? __ldg(w + next) : 0u;
        buf |= (uint64_t)v << cnt;
        next++;
        cnt += 32;
    }
    __device__ __forceinline__ void init(const uint8_t* in, uint64_t endw, uint64_t bit) {
        w = (const uint32_t*)in;
        end_word = endw;
        next = bit >> 5;
        buf = 0;
        cnt = 0;
        refill1();
        refill1();
        int s = (int)(bit & 31);
        buf >>= s;
        cnt -= s;
    }
    __device__ __forceinline__ void need(int n) {
        if (cnt < n) refill1();
    }
    __device__ __forceinline__ uint32_t get(int n) {  // n <= 32
        need(n);
        uint32_t v = (uint32_t)(buf & ((1ull << n) - 1));
        buf >>= n;
        cnt -= n;
        return v;
    }
    __device__ __forceinline__ uint64_t pos() const { return next * 32 - (uint64_t)cnt; }
};

// symbol of a code longer than the lookup (or -1 entry)
__device__ __forceinline__ uint32_t slow_decode(const Code& c, const uint16_t* syms, int alphabet, uint64_t buf,
                                                int root) {
    uint32_t rev = __brev((uint32_t)buf);
    for (int len = root + 1; len < 16; len++) {
        uint32_t code = rev >> (32 - len);
        uint32_t d = code - c.first[len];
        if (d < c.count[len]) return entry_of(alphabet, syms[c.offs[len] + d]) | (uint32_t)len;
    }
    return 0;  // no code: invalid data
}

// Reads a dynamic header's tables (after BFINAL/BTYPE). 0 ok, -1 invalid (inflate.cuh:231-265
// and :393-402 state the rules).
__device__ int dynamic_tables(Tables& T, Bits& br, int lane) {
    T.state = 0;
    int hlit = (int)br.get(5) + 257;
    int hdist = (int)br.get(5) + 1;
    int hclen = (int)br.get(4) + 4;
    if (hlit > 286 || hdist > 30) return -1;
    // the code-length code's lengths: read by every lane, each lane keeps one
    uint32_t cl_bits = 0;
    for (int i = 0; i < hclen; i++) {
        uint32_t v = br.get(3);
        if (lane < 19 && c_order[i] == lane) cl_bits = v;
    }
    if (lane < 19) T.lens[lane] = (uint8_t)cl_bits;
    __syncwarp();
    Built cb = build_code(T.lens, 19, A_CL, CB, nullptr, T.clh, T.clc, T.cl_syms, T.running, lane);
    if (cb.kraft != 0) return -1;
    int total = hlit + hdist;
    int prev = 0;
    for (int i = 0; i < total;) {
        br.need(CB + 7);
        uint32_t e = T.clh[br.buf & ((1u << CB) - 1)];
        int len = (int)(e >> 5), sym = (int)(e & 31);
        br.buf >>= len;
        br.cnt -= len;
        int rep = 1, val = sym;
        if (sym >= 16) {
            if (sym == 16) {
                if (i == 0) return -1;
                val = prev;
                rep = 3 + (int)(br.buf & 3);
                br.buf >>= 2;
                br.cnt -= 2;
            } else if (sym == 17) {
                val = 0;
                rep = 3 + (int)(br.buf & 7);
                br.buf >>= 3;
                br.cnt -= 3;
            } else {
                val = 0;
                rep = 11 + (int)(br.buf & 127);
                br.buf >>= 7;
                br.cnt -= 7;
            }
            if (i + rep > total) return -1;
        }
        for (int k = lane; k < rep; k += 32) T.lens[i + k] = (uint8_t)val;
        prev = val;
        i += rep;
    }
    __syncwarp();
    if (T.lens[256] == 0) return -1;
    Built lb = build_code(T.lens, hlit, A_LIT, LB, T.lit, nullptr, T.litc, T.lit_syms, T.running, lane);
    if (lb.kraft < 0 || (lb.kraft > 0 && !(lb.nonzero == 1 && lb.ones == 1))) return -1;
    // distance lengths follow the literal/length ones
    __syncwarp();
    Built db = build_code(T.lens + hlit, hdist, A_DIST, DB, T.dist, nullptr, T.distc, T.dist_syms, T.running, lane);
    if (db.kraft < 0 || (db.kraft > 0 && !(db.nonzero == 0 || (db.nonzero == 1 && db.ones == 1)))) return -1;
    T.state = 2;
    __syncwarp();
    return 0;
}

__device__ void fixed_tables(Tables& T, int lane) {
    if (T.state == 1) return;
    __syncwarp();
    for (int i = lane; i < 288; i += 32) T.lens[i] = (uint8_t)(i < 144 ? 8 : i < 256 ? 9 : i < 280 ? 7 : 8);
    __syncwarp();
    build_code(T.lens, 288, A_LIT, LB, T.lit, nullptr, T.litc, T.lit_syms, T.running, lane);
    __syncwarp();
    for (int i = lane; i < 30; i += 32) T.lens[i] = 5;
    __syncwarp();
    build_code(T.lens, 30, A_DIST, DB, T.dist, nullptr, T.distc, T.dist_syms, T.running, lane);
    T.state = 1;
    __syncwarp();
}

// the output side of a decoder: 32-symbol groups staged across the lanes
struct Out {
    uint16_t* base;   // current extent
    uint32_t op;      // symbols in the current extent (an extent holds at most 16 Mi + 65,793)
    uint32_t cap;
    uint64_t done;    // symbols in earlier extents
    int ext;          // current extent index
    uint16_t stage;   // this lane's symbol of the current group
    bool discard;     // JOB_DISCARD: the extent is written over instead of growing
};

__device__ __forceinline__ void flush_partial(Out& o, int lane) {
    uint32_t r = o.op & 31;
    if (r && (uint32_t)lane < r) o.base[(o.op & ~31u) + lane] = o.stage;
}

__device__ __forceinline__ void emit_lit(Out& o, uint32_t v, int lane) {
    uint32_t r = o.op & 31;
    if ((uint32_t)lane == r) o.stage = (uint16_t)v;
    o.op++;
    if (r == 31) o.base[o.op - 32 + lane] = o.stage;
}

__device__ __forceinline__ void emit_run(Out& o, uint32_t len, uint16_t v, int lane) {
    uint32_t r = o.op & 31;
    if ((uint32_t)lane - r < len) o.stage = v;
    if (r + len < 32) {
        o.op += len;
        return;
    }
    uint32_t g = o.op & ~31u;
    o.base[g + lane] = o.stage;
    uint32_t p = g + 32;
    uint32_t rem = r + len - 32;
    // 16-byte stores: 256 symbols per instruction (p is a multiple of 32: 64-byte aligned)
    uint32_t w = (uint32_t)v | ((uint32_t)v << 16);
    uint4 q = make_uint4(w, w, w, w);
    uint32_t k = 0;
    for (; k + 256 <= rem; k += 256) *(uint4*)(o.base + p + k + lane * 8) = q;
    for (; k + 32 <= rem; k += 32) o.base[p + k + lane] = v;
    o.stage = v;
    o.op += len;
}


// Starts a new extent for the decoder at `state`; false when the pool or the extent list is full.
__device__ bool new_extent(Ctx& C, Out& o, uint64_t need, const Start& state, int job) {
    int lane = C.lane;
    flush_partial(o, lane);
    if (o.discard) {  // start the same extent over (it holds DISCARD_EXTENT >= need)
        o.done += o.op;
        o.op = 0;
        return need <= o.cap;
    }
    uint64_t want = o.cap * 2;
    if (want < (64ull << 10)) want = 64ull << 10;
    if (want > (16ull << 20)) want = 16ull << 20;
    if (want < need) want = (need + 31) & ~31ull;
    unsigned long long off = 0;
    int e = 0;
    if (lane == 0) {
        off = atomicAdd(&C.a.ctr->pool_used, (unsigned long long)want);
        e = off + want <= C.a.pool_cap ? atomicAdd(&C.a.ctr->n_ext, 1) : -1;
        if (e >= C.a.ext_cap) e = -1;
    }
    e = __shfl_sync(FULL, e, 0);
    off = __shfl_sync(FULL, off, 0);
    if (e < 0) return false;
    if (lane == 0) {
        C.a.ext[o.ext].len = o.op;
        C.a.ext[o.ext].next = e;
        Extent x;
        x.pool_off = off;
        x.len = 0;
        x.cap = want;
        x.start = state;
        x.next = -1;
        x.job = job;
        C.a.ext[e] = x;
    }
    o.done += o.op;
    o.op = 0;
    o.cap = (uint32_t)want;
    o.base = C.a.pool + off;
    o.ext = e;
    return true;
}

// Decodes one symbol of the current block and writes its output: 0 a literal or a match, 1 the
// end-of-block code, -1 invalid data with no code at all, -2 invalid data after a length symbol
// was read (a length or distance symbol that does not exist, or - check_refs - a match reaching
// before the stream's start). The reference counts a symbol at its length code, before the rest
// is checked (inflate.cuh:449-457), so a -2 is one more symbol read. As there, a code that is in
// the table but names no length (286, 287) or no distance (30, 31) is read before it is refused,
// and a bit pattern that is no code at all is not: where the decode ends on an error is the same.
__device__ __forceinline__ int one_symbol(const Tables& T, Bits& br, Out& o, int lane, bool check_refs) {
    br.need(32);
    uint32_t e = T.lit[(uint32_t)br.buf & ((1u << LB) - 1)];
    if (e < (1u << 24)) {  // literal
        int n = (int)(e & 15);
        br.buf >>= n;
        br.cnt -= n;
        emit_lit(o, (e >> 8) & 255, lane);
        return 0;
    }
    if ((e & 15) == 0) {
        e = slow_decode(T.litc, T.lit_syms, A_LIT, br.buf, LB);
        if (e == 0) return -1;
        if (e < (1u << 24)) {
            int n = (int)(e & 15);
            br.buf >>= n;
            br.cnt -= n;
            emit_lit(o, (e >> 8) & 255, lane);
            return 0;
        }
    }
    uint32_t kind = e & (3u << 24);
    if (kind == K_EOB) {
        int n = (int)(e & 15);
        br.buf >>= n;
        br.cnt -= n;
        return 1;
    }
    if (kind == K_BAD) {
        const int n = (int)(e & 15);
        br.buf >>= n;
        br.cnt -= n;
        return -2;
    }
    int n = (int)(e & 15), x = (int)((e >> 4) & 15);
    uint32_t len = ((e >> 8) & 0xffff) + (uint32_t)((br.buf >> n) & ((1u << x) - 1));
    br.buf >>= n + x;
    br.cnt -= n + x;
    br.need(32);
    uint32_t de = T.dist[(uint32_t)br.buf & ((1u << DB) - 1)];
    if ((de & 15) == 0) {
        de = de == E_LONG ? slow_decode(T.distc, T.dist_syms, A_DIST, br.buf, DB) : 0;
        if (de == 0) return -2;
    }
    if ((de & (3u << 24)) == K_BAD) {
        const int dn = (int)(de & 15);
        br.buf >>= dn;
        br.cnt -= dn;
        return -2;
    }
    int dn = (int)(de & 15), dx = (int)((de >> 4) & 15);
    uint32_t d = ((de >> 8) & 0xffff) + (uint32_t)((br.buf >> dn) & ((1u << dx) - 1));
    br.buf >>= dn + dx;
    br.cnt -= dn + dx;
    if (check_refs && d > o.done + o.op) return -2;
    emit_run(o, len, (uint16_t)(REF + d), lane);
    return 0;
}

__device__ void decode_job(Ctx& C, int k) {
    const int lane = C.lane;
    const long long t_begin = clock64();
    Tables& T = *C.T;
    const Job J = C.a.jobs[k];
    const StreamDesc S = C.a.streams[J.stream];
    Job1& j = T.j;
    j.stop = S.stop;
    j.end_bit = S.end_bit;
    j.end_byte = S.end_bit >> 3;
    j.limit = S.stop < S.end_bit + 1 ? S.stop : S.end_bit + 1;
    j.tg = C.a.targets;
    j.t = J.tfirst;
    j.tend = S.target_end;
    j.tbit = j.t < j.tend ? j.tg[j.t].bit : UINT64_MAX;
    j.passed = 0;
    j.give_up = (J.flags & JOB_TRUSTED) || J.start.mode == AT_BLOCK ? 0 : C.a.give_up;
    const bool check_refs = (J.flags & JOB_CHECK_REFS) != 0;

    JobResult& r = T.r;
    r.t_begin = global_ns();
    r.t_end = r.t_begin;
    r.eob_bit = UINT64_MAX;
    r.eob_out = 0;
    r.status = S_OK;
    r.landed = -1;
    r.end_final = J.start.mode == AT_BLOCK ? -1 : J.start.final;
    r.blocks = 0;
    r.resume = J.start;
    r.hdr0 = UINT64_MAX;
    r.symbols = 0;
    r.last_block_bit = UINT64_MAX;
    r.last_block_out = 0;

    Out o;
    o.base = C.a.pool + J.pool_off;
    o.op = 0;
    o.cap = J.cap;
    o.done = 0;
    o.ext = k;
    o.stage = 0;
    o.discard = (J.flags & JOB_DISCARD) != 0;
    if (lane == 0) {
        Extent x;
        x.pool_off = J.pool_off;
        x.len = 0;
        x.cap = J.cap;
        x.start = J.start;
        x.next = -1;
        x.job = k;
        C.a.ext[k] = x;
    }

    Bits br;
    bool in_block = false, fixed = false;
    uint64_t header = J.start.header;
    if (J.start.mode == IN_FIXED) {
        fixed_tables(T, lane);
        in_block = fixed = true;
    } else if (J.start.mode == IN_DYNAMIC) {
        br.init(C.a.in, S.end_word, J.start.header);
        br.get(3);
        if (dynamic_tables(T, br, lane) != 0) {
            r.status = S_DATA;
            r.end_bit = J.start.bit;
            r.out_len = 0;
            r.cycles = 0;
            if (lane == 0) C.a.res[k] = r;
            return;
        }
        in_block = true;
    }
    br.init(C.a.in, S.end_word, J.start.bit);

    for (;;) {
        if (!in_block) {
            uint64_t p = br.pos();
            while (j.tbit < p) {
                j.passed += j.tg[j.t].mode == AT_BLOCK;
                j.t++;
                j.tbit = j.t < j.tend ? j.tg[j.t].bit : UINT64_MAX;
            }
            if (j.tbit == p && j.tg[j.t].mode == AT_BLOCK) {
                r.landed = j.t;
                break;
            }
            if (p >= j.stop || (j.give_up && j.passed >= j.give_up)) {
                r.status = S_STOPPED;
                r.resume = Start{p, p, AT_BLOCK, -1, {0, 0, 0, 0, 0, 0}};
                break;
            }
            if (o.op + MAX_SYMBOL_OUT > o.cap) {
                Start st = Start{p, p, AT_BLOCK, -1, {0, 0, 0, 0, 0, 0}};
                if (!new_extent(C, o, MAX_SYMBOL_OUT, st, k)) {
                    r.status = S_OVERFLOW;
                    r.resume = st;
                    break;
                }
            }
            if (p >= j.end_bit) {
                r.status = S_INPUT;
                break;
            }
            header = p;
            r.last_block_bit = p;
            r.last_block_out = o.done + o.op;
            int fin = (int)br.get(1);
            int type = (int)br.get(2);
            r.blocks++;
            r.end_final = fin;
            if (type == 0) {
                uint32_t rb = (uint32_t)(br.pos() & 7);
                if (rb) br.get(8 - (int)rb);
                uint32_t len = br.get(16), nlen = br.get(16);
                if (len != (~nlen & 0xffffu)) {
                    r.status = S_DATA;
                    break;
                }
                uint64_t byte = br.pos() >> 3;
                if (byte + len > j.end_byte) {
                    r.status = S_INPUT;
                    break;
                }
                if (o.op + len > o.cap) {
                    Start st = Start{p, p, AT_BLOCK, -1, {0, 0, 0, 0, 0, 0}};
                    if (!new_extent(C, o, len + MAX_SYMBOL_OUT, st, k)) {
                        r.status = S_OVERFLOW;
                        r.resume = st;
                        break;
                    }
                }
                if (len) {
                    flush_partial(o, lane);
                    bool queued = false;
                    if (lane == 0) {
                        int i = atomicAdd(&C.a.ctr->n_stored, 1);
                        if (i < C.a.stored_cap) {
                            StoredCopy sc;
                            sc.src = byte;
                            sc.dst = (uint64_t)(o.base - C.a.pool) + o.op;
                            sc.len = len;
                            sc.pad = 0;
                            C.a.stored[i] = sc;
                            queued = true;
                        }
                    }
                    queued = __shfl_sync(FULL, queued, 0);
                    if (!queued) {  // list full: the warp copies the bytes itself
                        for (uint32_t q = lane; q < len; q += 32) o.base[o.op + q] = C.a.in[byte + q];
                        __syncwarp();
                    }
                    o.op += len;
                    // the group the block ends in: its staged symbols must not overwrite its bytes
                    if (!queued && (uint32_t)lane < (uint32_t)(o.op & 31)) o.stage = o.base[(o.op & ~31ull) + lane];
                }
                br.init(C.a.in, S.end_word, (byte + len) * 8);
                if (fin) break;
                continue;
            }
            if (type == 3) {
                r.status = S_DATA;
                break;
            }
            if (type == 1) {
                fixed_tables(T, lane);
                fixed = true;
            } else {
                if (dynamic_tables(T, br, lane) != 0) {
                    r.status = S_DATA;
                    break;
                }
                fixed = false;
            }
            in_block = true;
        }
        // ---- the block's symbols
        const uint8_t mode = fixed ? IN_FIXED : IN_DYNAMIC;
        if (r.hdr0 == UINT64_MAX) r.hdr0 = header;
        bool eob = false;
        // one comparison per symbol covers the stop bit, the input's end and the next target
        uint64_t lim2 = j.tbit < j.limit ? j.tbit : j.limit;
        for (;;) {
            uint64_t p = br.pos();
            if (p >= lim2) {
                if (p >= j.limit) {
                    if (p > j.end_bit) {
                        r.status = S_INPUT;
                    } else {
                        r.status = S_STOPPED;
                        r.resume = Start{p, header, mode, (int8_t)r.end_final, {0, 0, 0, 0, 0, 0}};
                    }
                    break;
                }
                // a target at or before this symbol boundary: land on it when it is a boundary
                // of this block (same tables), else pass it
                while (j.tbit < p) {
                    j.passed += j.tg[j.t].mode == AT_BLOCK;
                    j.t++;
                    j.tbit = j.t < j.tend ? j.tg[j.t].bit : UINT64_MAX;
                }
                if (j.tbit == p) {
                    const Start& tt = j.tg[j.t];
                    if (tt.mode == mode && tt.header == header) {
                        r.landed = j.t;
                        break;
                    }
                    j.passed += tt.mode == AT_BLOCK;
                    j.t++;
                    j.tbit = j.t < j.tend ? j.tg[j.t].bit : UINT64_MAX;
                }
                if (j.give_up && j.passed >= j.give_up) {  // out of step: stop where it is
                    r.status = S_STOPPED;
                    r.resume = Start{p, header, mode, (int8_t)r.end_final, {0, 0, 0, 0, 0, 0}};
                    break;
                }
                lim2 = j.tbit < j.limit ? j.tbit : j.limit;
                continue;
            }
            if (o.op + MAX_SYMBOL_OUT > o.cap) {
                Start st = Start{p, header, mode, (int8_t)r.end_final, {0, 0, 0, 0, 0, 0}};
                if (!new_extent(C, o, MAX_SYMBOL_OUT, st, k)) {
                    r.status = S_OVERFLOW;
                    r.resume = st;
                    break;
                }
            }
            // a run of symbols with no per-symbol position or room checks: a symbol takes at most
            // 48 bits and writes at most 258 positions, so these cannot pass the next check point
            // (the first one starts before it), the stop bit or the extent's end
            const uint64_t left = lim2 - p;
            const uint32_t room = o.cap - o.op;
            uint32_t run = (uint32_t)(left / 48 < (uint64_t)(room / MAX_SYMBOL_OUT) ? left / 48 : room / MAX_SYMBOL_OUT);
            if (run == 0) run = 1;
            const bool chk = check_refs && r.blocks <= FIRST_RUN_BLOCKS;
            int rc;
            const uint32_t run0 = run;
            do {
                rc = one_symbol(T, br, o, lane, chk);
            } while (rc == 0 && --run);
            r.symbols += run0 - run;  // every symbol but the one that ended the run early was a literal or match
            if (rc > 0) {
                eob = true;
                break;
            }
            if (rc < 0) {
                r.status = S_DATA;
                r.symbols += rc == -2;
                break;
            }
        }
        if (!eob) break;
        in_block = false;
        if (br.pos() > j.end_bit) {
            r.status = S_INPUT;
            break;
        }
        if (r.eob_bit == UINT64_MAX) {
            r.eob_bit = br.pos();
            r.eob_out = o.done + o.op;
        }
        if (r.end_final == 1) break;
    }
    flush_partial(o, lane);
    r.end_bit = br.pos();
    r.out_len = o.done + o.op;
    r.cycles = (uint64_t)(clock64() - t_begin);
    r.t_end = global_ns();
    if (lane == 0) {
        C.a.ext[o.ext].len = o.op;
        C.a.res[k] = r;
    }
}

// ---------------------------------------------------------------- probes
//
// Huffman codes resynchronize: decoding from an arbitrary bit soon falls onto the real symbol
// boundaries (the reference's Decoder::probe, gpuinflate/inflate.cuh:583-648, uses the same
// property). A probe decodes, writing nothing, from LEAD bits before a point with the tables of
// the block the span begins in, restarting one bit later when the data makes no sense, and
// reports the first symbol boundary at or after the point (or the block boundary there). A
// wrong report is harmless: a decoder lands only on a position its own decode reaches with the
// same tables. One warp takes all points of a span, so the span's tables are built once.

// the tables a span starts with; header and final of its block (final -1 when unknown)
__device__ __forceinline__ bool span_tables(Tables& T, const uint8_t* in, uint64_t end_word, const Start& s, int lane,
                                            uint64_t& header, bool& fixed, int& final) {
    if (s.mode == IN_FIXED) {
        fixed_tables(T, lane);
        header = s.header;
        fixed = true;
        final = s.final;
        return true;
    }
    uint64_t h = s.mode == AT_BLOCK ? s.bit : s.header;
    Bits hb;
    hb.init(in, end_word, h);
    final = (int)hb.get(1);
    int type = (int)hb.get(2);
    header = h;
    if (type == 1) {
        fixed_tables(T, lane);
        fixed = true;
        return true;
    }
    if (type != 2) return false;
    fixed = false;
    return dynamic_tables(T, hb, lane) == 0;
}

// the tables of a block whose header is known: fixed, or the dynamic header at `header`
__device__ __forceinline__ bool block_tables(Tables& T, const uint8_t* in, uint64_t end_word, uint64_t header, bool fixed,
                                             int lane) {
    if (fixed) {
        fixed_tables(T, lane);
        return true;
    }
    Bits hb;
    hb.init(in, end_word, header);
    hb.get(1);
    if (hb.get(2) != 2) return false;
    return dynamic_tables(T, hb, lane) == 0;
}

__global__ void __launch_bounds__(NWARPS * 32, 4) k_probe(ProbeArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    Tables& T = ((Tables*)smem)[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    if (lane == 0) T.state = 0;
    __syncwarp();
    const uint64_t nwarps = (uint64_t)gridDim.x * NWARPS;
    for (uint64_t w = (uint64_t)blockIdx.x * NWARPS + (threadIdx.x >> 5); w < (uint64_t)a.nspans; w += nwarps) {
        const ProbeSpan ps = a.spans[w];
        // base: the block a point's probe starts in (the span's, then the block the last probe
        // ended in); cur: the block being decoded
        uint64_t span_header = 0;
        bool span_fixed = false;
        int span_final = -1;
        const bool ok = span_tables(T, a.in, a.end_word, ps.start, lane, span_header, span_fixed, span_final);
        uint64_t base_header = span_header;
        bool base_fixed = span_fixed;
        int base_final = span_final;
        bool have = ok;  // the loaded tables are base's
        for (uint32_t i = 0; i < ps.npoints; i++) {
            const uint64_t at = ps.first_point + (uint64_t)i * ps.spacing;
            Start res = Start{UINT64_MAX, UINT64_MAX, AT_BLOCK, -1, {0, 0, 0, 0, 0, 0}};
            uint64_t header = base_header;
            bool fixed = base_fixed;
            int final = base_final;
            if (ok) {
                uint64_t start = at - a.lead > ps.start.bit ? at - a.lead : ps.start.bit;
                for (uint32_t attempt = 0; attempt < a.attempts && start < at && res.bit == UINT64_MAX; attempt++) {
                    if (!have) {
                        have = block_tables(T, a.in, a.end_word, base_header, base_fixed, lane);
                        if (!have) break;
                    }
                    header = base_header;
                    fixed = base_fixed;
                    final = base_final;
                    Bits br;
                    br.init(a.in, a.end_word, start);
                    uint64_t p;
                    for (;;) {
                        p = br.pos();
                        if (p >= at) {
                            res = Start{p, header, (uint8_t)(fixed ? IN_FIXED : IN_DYNAMIC), (int8_t)final,
                                        {0, 0, 0, 0, 0, 0}};
                            break;
                        }
                        br.need(32);
                        uint32_t e = T.lit[br.buf & ((1u << LB) - 1)];
                        if ((e & 15) == 0) e = slow_decode(T.litc, T.lit_syms, A_LIT, br.buf, LB);
                        if (e == 0 || (e & (3u << 24)) == K_BAD) break;
                        int n = (int)(e & 15);
                        uint32_t kind = e & (3u << 24);
                        if (kind == K_LIT) {
                            br.buf >>= n;
                            br.cnt -= n;
                            continue;
                        }
                        if (kind == K_EOB) {
                            br.buf >>= n;
                            br.cnt -= n;
                            uint64_t h = br.pos();
                            if (h >= at) {
                                res = Start{h, h, AT_BLOCK, -1, {0, 0, 0, 0, 0, 0}};
                                break;
                            }
                            int fin = (int)br.get(1);
                            int ty = (int)br.get(2);
                            header = h;
                            final = fin;
                            have = false;  // the loaded tables are no longer base's
                            if (ty == 1) {
                                fixed_tables(T, lane);
                                fixed = true;
                            } else if (ty == 2 && dynamic_tables(T, br, lane) == 0) {
                                fixed = false;
                            } else {
                                break;
                            }
                            continue;
                        }
                        int x = (int)((e >> 4) & 15);
                        br.buf >>= n + x;
                        br.cnt -= n + x;
                        br.need(32);
                        uint32_t de = T.dist[br.buf & ((1u << DB) - 1)];
                        if ((de & 15) == 0) de = de == E_LONG ? slow_decode(T.distc, T.dist_syms, A_DIST, br.buf, DB) : 0;
                        if (de == 0 || (de & (3u << 24)) == K_BAD) break;
                        int dn = (int)(de & 15), dx = (int)((de >> 4) & 15);
                        br.buf >>= dn + dx;
                        br.cnt -= dn + dx;
                    }
                    start = p + 1;
                }
            }
            if (res.bit != UINT64_MAX && res.mode != AT_BLOCK) {
                // the next point starts in the block this one ended in (its tables are loaded)
                base_header = header;
                base_fixed = fixed;
                base_final = final;
                have = true;
            } else if (base_header != span_header || base_fixed != span_fixed) {
                base_header = span_header;
                base_fixed = span_fixed;
                base_final = span_final;
                have = false;
            }
            if (lane == 0) a.out[ps.out_index + i] = res;
        }
    }
}

__global__ void __launch_bounds__(NWARPS * 32, 4) k_decode(DecodeArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    Tables* tabs = (Tables*)smem;
    Ctx C;
    C.a = a;
    C.lane = threadIdx.x & 31;
    C.T = &tabs[threadIdx.x >> 5];
    if (C.lane == 0) C.T->state = 0;
    __syncwarp();
    for (;;) {
        int q = 0;
        if (C.lane == 0) q = atomicAdd(&a.ctr->next_job, 1);
        q = __shfl_sync(FULL, q, 0);
        if (q >= a.njobs) break;
        int k = a.order ? a.order[q] : q;
        decode_job(C, k);
    }
}

}  // namespace

int decode_blocks_per_sm() {
    int n = 0;
    cudaFuncSetAttribute(k_probe, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(NWARPS * sizeof(Tables)));
    cudaFuncSetAttribute(k_decode, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(NWARPS * sizeof(Tables)));
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_decode, NWARPS * 32, NWARPS * sizeof(Tables));
    return n > 0 ? n : 1;
}

int launch_probe(const ProbeArgs& a, int grid, void* stream) {
    if (a.nspans <= 0) return 0;
    k_probe<<<grid, NWARPS * 32, NWARPS * sizeof(Tables), (cudaStream_t)stream>>>(a);
    return 1;
}

int launch_decode(const DecodeArgs& a, int grid, void* stream) {
    k_decode<<<grid, NWARPS * 32, NWARPS * sizeof(Tables), (cudaStream_t)stream>>>(a);
    return 1;
}

}  // namespace gz
