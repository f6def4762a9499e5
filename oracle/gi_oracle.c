/* gi_oracle.c - CPU oracle for the Deflate decode path. TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this file's
 * library (liboracle.so), and only as the checker or as the timed CPU baseline. The product
 * (gpuzip_gb300/, libgpuinflate.so) never links, loads or calls it.
 *
 * What it restates, in plain C, from gpuzip's reference decoder:
 *   - the sequential decode that the reference's test harness uses as its CPU oracle
 *     (gpuinflate/gi_test.cpp:47-91): Decoder::run from bit 0 (gpuinflate/inflate.cuh:474-581),
 *     continuing after every 65,536 blocks (MAX_BLOCKS, inflate.cuh:71) with stream_start
 *     cleared, and a final pass that rejects matches reaching before the stream's start
 *     (gi_test.cpp:78-89);
 *   - the error classes: reading past the input returns zero bits (inflate.cuh:116-123);
 *     "truncated" is reported only where the reference checks the position
 *     (inflate.cuh:434, :521, :542, :571); every other failure is "invalid data";
 *   - the table rules zlib applies (inflate.cuh:162-196, :231-265, :393-402): complete
 *     code-length code, at most 286/30 codes, an end-of-block code, an incomplete
 *     literal/length code only as one 1-bit code, an incomplete distance code only as none
 *     or one 1-bit code;
 *   - in_used = (bit after the final block + 7) / 8 (gi_test.cpp:74);
 *   - the block-start tests: header_prefilter128 (inflate.cuh:300-311) and
 *     plausible_dynamic_header with its kraft() checks (inflate.cuh:268-281, :315-332);
 *   - CRC-32 (gzip's trailer check, src/gz.rs:207-247 via crc32fast): the reflected
 *     polynomial 0xEDB88320, bytewise table.
 * Output is produced as plain bytes (matches copied), which is what the reference's oracle
 * yields after its resolution pass.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define O_OK 0
#define O_DATA 1
#define O_TRUNCATED 2
#define O_TOO_BIG 7

#define O_WINDOW 32768u
#define O_MAX_BLOCKS 65536u
#define O_LB 10 /* first-level lookup bits; longer codes take the canonical slow path */

static const uint16_t len_base[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                                      31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
static const uint8_t len_extra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
static const uint16_t dist_base[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,    65,    97,    129,
                                       193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
static const uint8_t dist_extra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
/* RFC 1951 3.2.7: the order code-length code lengths are sent in */
static const uint8_t cl_order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

/* ------------------------------------------------------------------ bits */

/* LSB-first reader over a copy of the input followed by 16 zero bytes; bits past the input
 * read as zero, as the reference's reader does (inflate.cuh:116-123). */
typedef struct {
    const uint8_t* p;
    uint64_t size;      /* input bytes */
    uint64_t size_bits; /* size * 8 */
    uint64_t pos;       /* next bit */
} obits;

static inline uint64_t load64(const uint8_t* p) {
    uint64_t v;
    memcpy(&v, p, 8);
    return v; /* little-endian hosts only (x86-64, aarch64) */
}

static inline uint32_t peek(const obits* b, int n) {
    uint64_t byte = b->pos >> 3;
    uint64_t v;
    if (byte + 8 <= b->size + 16) {
        v = load64(b->p + byte);
    } else {
        v = 0; /* far past the end: every bit is zero */
        if (byte < b->size + 16) memcpy(&v, b->p + byte, (size_t)(b->size + 16 - byte));
    }
    v >>= (b->pos & 7);
    return n >= 32 ? (uint32_t)v : (uint32_t)(v & ((1ull << n) - 1));
}

static inline uint32_t getbits(obits* b, int n) {
    if (n == 0) return 0;
    uint32_t v = peek(b, n);
    b->pos += (uint64_t)n;
    return v;
}

/* ------------------------------------------------------------------ canonical Huffman */

typedef struct {
    uint16_t count[16];
    uint16_t symbol[288];
    uint16_t lut[1 << O_LB]; /* (length << 9) | symbol for codes of <= O_LB bits; 0 = longer or none */
    int nonzero;
} ohuff;

/* 0: complete; 1: incomplete; -1: over-subscribed (inflate.cuh:162-196 returns the same) */
static int huff_build(ohuff* h, const uint8_t* lens, int n) {
    for (int i = 0; i < 16; i++) h->count[i] = 0;
    for (int s = 0; s < n; s++) h->count[lens[s]]++;
    h->nonzero = n - h->count[0];
    h->count[0] = 0;
    int left = 1;
    for (int len = 1; len < 16; len++) {
        left = (left << 1) - h->count[len];
        if (left < 0) return -1;
    }
    uint16_t offs[16], next[16];
    offs[1] = 0;
    for (int len = 1; len < 15; len++) offs[len + 1] = (uint16_t)(offs[len] + h->count[len]);
    int code = 0;
    for (int len = 1; len < 16; len++) {
        code = (code + h->count[len - 1]) << 1;
        next[len] = (uint16_t)code;
    }
    memset(h->lut, 0, sizeof h->lut);
    for (int s = 0; s < n; s++) {
        int len = lens[s];
        if (!len) continue;
        h->symbol[offs[len]++] = (uint16_t)s;
        int c = next[len]++;
        if (len <= O_LB) {
            int rev = 0;
            for (int b = 0; b < len; b++) rev |= ((c >> b) & 1) << (len - 1 - b);
            for (int k = rev; k < (1 << O_LB); k += 1 << len) h->lut[k] = (uint16_t)((len << 9) | s);
        }
    }
    return left > 0 ? 1 : 0;
}

static inline int single_code(const ohuff* h) { return h->nonzero == 1 && h->count[1] == 1; }

/* symbol, or -1 for bits that start no code of up to 15 bits */
static inline int huff_decode(const ohuff* h, obits* b) {
    uint32_t bits = peek(b, 16);
    uint16_t e = h->lut[bits & ((1u << O_LB) - 1)];
    if (e) {
        b->pos += e >> 9;
        return e & 511;
    }
    int code = 0, first = 0, index = 0;
    for (int len = 1; len < 16; len++) {
        code |= (int)((bits >> (len - 1)) & 1);
        int c = h->count[len];
        if (code - c < first) {
            b->pos += (uint64_t)len;
            return h->symbol[index + (code - first)];
        }
        index += c;
        first = (first + c) << 1;
        code <<= 1;
    }
    return -1;
}

/* a dynamic block's code lengths, after BFINAL and BTYPE: 0 valid, -1 invalid
 * (inflate.cuh:231-265) */
static int read_code_lengths(obits* b, ohuff* clh, uint8_t* lens, int* hlit_out, int* hdist_out) {
    int hlit = (int)getbits(b, 5) + 257;
    int hdist = (int)getbits(b, 5) + 1;
    int hclen = (int)getbits(b, 4) + 4;
    if (hlit > 286 || hdist > 30) return -1;
    uint8_t cl[19];
    memset(cl, 0, sizeof cl);
    for (int i = 0; i < hclen; i++) cl[cl_order[i]] = (uint8_t)getbits(b, 3);
    if (huff_build(clh, cl, 19) != 0) return -1;
    int total = hlit + hdist;
    for (int i = 0; i < total;) {
        int s = huff_decode(clh, b);
        if (s < 0) return -1;
        if (s < 16) {
            lens[i++] = (uint8_t)s;
            continue;
        }
        int rep;
        uint8_t val = 0;
        if (s == 16) {
            if (i == 0) return -1;
            val = lens[i - 1];
            rep = 3 + (int)getbits(b, 2);
        } else if (s == 17) {
            rep = 3 + (int)getbits(b, 3);
        } else {
            rep = 11 + (int)getbits(b, 7);
        }
        if (i + rep > total) return -1;
        while (rep--) lens[i++] = val;
    }
    if (lens[256] == 0) return -1;
    *hlit_out = hlit;
    *hdist_out = hdist;
    return 0;
}

typedef struct {
    ohuff lit, dist, clh;
    uint8_t lens[320];
    int have_fixed;
} otables;

static int dynamic_tables(otables* t, obits* b) {
    t->have_fixed = 0;
    int hlit, hdist;
    if (read_code_lengths(b, &t->clh, t->lens, &hlit, &hdist) != 0) return -1;
    int r = huff_build(&t->lit, t->lens, hlit);
    if (r < 0 || (r > 0 && !single_code(&t->lit))) return -1;
    r = huff_build(&t->dist, t->lens + hlit, hdist);
    if (r < 0 || (r > 0 && !(t->dist.nonzero == 0 || single_code(&t->dist)))) return -1;
    return 0;
}

static void fixed_tables(otables* t) {
    if (t->have_fixed) return;
    t->have_fixed = 1;
    for (int i = 0; i < 288; i++) t->lens[i] = (uint8_t)(i < 144 ? 8 : i < 256 ? 9 : i < 280 ? 7 : 8);
    huff_build(&t->lit, t->lens, 288);
    for (int i = 0; i < 30; i++) t->lens[i] = 5;
    huff_build(&t->dist, t->lens, 30);
}

/* ------------------------------------------------------------------ inflate */

/* Decodes the raw Deflate stream at in[0..size). Returns O_OK, O_DATA, O_TRUNCATED, or
 * O_TOO_BIG when the output would exceed out_cap. *out_len gets the bytes written (on
 * success), *in_used the stream's length in bytes (on success). */
int oracle_inflate(const uint8_t* in, uint64_t size, uint8_t* out, uint64_t out_cap, uint64_t* out_len,
                   uint64_t* in_used) {
    uint8_t* pad = (uint8_t*)calloc((size_t)size + 16, 1);
    if (!pad) return -1;
    if (size) memcpy(pad, in, (size_t)size);
    otables* t = (otables*)calloc(1, sizeof(otables));
    if (!t) {
        free(pad);
        return -1;
    }
    obits b = {pad, size, size * 8, 0};
    uint64_t op = 0;         /* bytes written */
    uint64_t run_start = 0;  /* output position where the current run began */
    uint32_t run_blocks = 0; /* blocks decoded in the current run */
    int first_run = 1;       /* stream_start of the reference's run() */
    int deferred_bad = 0;    /* a match before the start seen in a later run: invalid if all else decodes */
    int status = O_OK;
    for (;;) {
        /* at a block boundary */
        if (run_blocks >= O_MAX_BLOCKS) { /* the reference starts a new run here */
            run_blocks = 0;
            first_run = 0;
            run_start = op;
        }
        if (b.pos >= b.size_bits) {
            status = O_TRUNCATED;
            break;
        }
        int final = (int)getbits(&b, 1);
        int type = (int)getbits(&b, 2);
        run_blocks++;
        if (type == 0) {
            if (b.pos & 7) getbits(&b, 8 - (int)(b.pos & 7));
            uint32_t len = getbits(&b, 16), nlen = getbits(&b, 16);
            if (len != (~nlen & 0xffffu)) {
                status = O_DATA;
                break;
            }
            uint64_t byte = b.pos >> 3;
            if (byte + len > size) {
                status = O_TRUNCATED;
                break;
            }
            if (op + len > out_cap) {
                status = O_TOO_BIG;
                break;
            }
            memcpy(out + op, in + byte, len);
            op += len;
            b.pos = (byte + len) * 8;
            if (final) break;
            continue;
        }
        if (type == 3) {
            status = O_DATA;
            break;
        }
        if (type == 1) {
            fixed_tables(t);
        } else if (dynamic_tables(t, &b) != 0) {
            status = O_DATA;
            break;
        }
        /* the block's symbols (inflate.cuh:418-466) */
        for (;;) {
            if (b.pos > b.size_bits) {
                status = O_TRUNCATED;
                break;
            }
            int sym = huff_decode(&t->lit, &b);
            if (sym < 0) {
                status = O_DATA;
                break;
            }
            if (sym < 256) {
                if (op >= out_cap) {
                    status = O_TOO_BIG;
                    break;
                }
                out[op++] = (uint8_t)sym;
                continue;
            }
            if (sym == 256) break;
            sym -= 257;
            if (sym >= 29) {
                status = O_DATA;
                break;
            }
            uint32_t len = len_base[sym] + getbits(&b, len_extra[sym]);
            int ds = huff_decode(&t->dist, &b);
            if (ds < 0 || ds >= 30) {
                status = O_DATA;
                break;
            }
            uint32_t d = dist_base[ds] + getbits(&b, dist_extra[ds]);
            if (first_run && d > op - run_start) {
                status = O_DATA;
                break;
            }
            if (op + len > out_cap) {
                status = O_TOO_BIG;
                break;
            }
            if (d > op) { /* only in a later run: the reference flags it in its final pass */
                deferred_bad = 1;
                memset(out + op, 0, len);
            } else {
                const uint8_t* src = out + op - d;
                for (uint32_t k = 0; k < len; k++) out[op + k] = src[k];
            }
            op += len;
        }
        if (status != O_OK) break;
        if (b.pos > b.size_bits) {
            status = O_TRUNCATED;
            break;
        }
        if (final) break;
    }
    if (status == O_OK && deferred_bad) status = O_DATA;
    if (status == O_OK) {
        *out_len = op;
        *in_used = (b.pos + 7) / 8;
    }
    free(t);
    free(pad);
    return status;
}

/* ------------------------------------------------------------------ block-start tests */

/* cheap test of a dynamic-block start from the 128 bits at it (inflate.cuh:300-311) */
int oracle_prefilter128(uint64_t v1, uint64_t v2) {
    if (((v1 >> 1) & 3) != 2 || ((v1 >> 3) & 31) > 29 || ((v1 >> 8) & 31) > 29) return 0;
    int hclen = (int)((v1 >> 13) & 15) + 4;
    int sum = 0;
    for (int i = 0; i < hclen; i++) {
        int p = 17 + 3 * i;
        uint32_t l;
        if (p + 3 <= 64)
            l = (uint32_t)(v1 >> p);
        else if (p >= 64)
            l = (uint32_t)(v2 >> (p - 64));
        else
            l = (uint32_t)((v1 >> p) | (v2 << (64 - p)));
        l &= 7;
        if (l) sum += 128 >> l;
    }
    return sum == 128;
}

static int kraft(const uint8_t* lens, int n, int* nonzero, int* ones) {
    int count[16] = {0};
    for (int s = 0; s < n; s++) count[lens[s]]++;
    *nonzero = n - count[0];
    *ones = count[1];
    int left = 1;
    for (int len = 1; len < 16; len++) {
        left = (left << 1) - count[len];
        if (left < 0) return -1;
    }
    return left > 0 ? 1 : 0;
}

/* does bit look like the start of a dynamic block (inflate.cuh:315-332); pad: the input followed
 * by at least 16 zero bytes */
static int plausible_padded(const uint8_t* pad, uint64_t size, uint64_t bit) {
    obits b = {pad, size, size * 8, bit};
    uint32_t h = peek(&b, 17);
    int ok = 0;
    if (((h >> 1) & 3) == 2 && ((h >> 3) & 31) <= 29 && ((h >> 8) & 31) <= 29) {
        b.pos += 3;
        ohuff clh_store;
        ohuff* clh = &clh_store;
        uint8_t lens[320];
        int hlit, hdist, nz, ones;
        if (read_code_lengths(&b, clh, lens, &hlit, &hdist) == 0) {
            int r = kraft(lens, hlit, &nz, &ones);
            if (!(r < 0 || (r > 0 && !(nz == 1 && ones == 1)))) {
                r = kraft(lens + hlit, hdist, &nz, &ones);
                if (!(r < 0 || (r > 0 && !(nz == 0 || (nz == 1 && ones == 1))))) ok = b.pos <= b.size_bits;
            }
        }
    }
    return ok;
}

int oracle_plausible_dynamic_header(const uint8_t* in, uint64_t size, uint64_t bit) {
    uint8_t* pad = (uint8_t*)calloc((size_t)size + 16, 1);
    if (!pad) return 0;
    memcpy(pad, in, (size_t)size);
    const int ok = plausible_padded(pad, size, bit);
    free(pad);
    return ok;
}

/* For every chunk of chunk_bits bits from bit_lo, the first bit in (bit_lo, bit_hi) that passes
 * both tests, or UINT64_MAX; the order of the reference's finder (gpuinflate.cu:291-319). */
void oracle_first_headers(const uint8_t* in, uint64_t size, uint64_t bit_lo, uint64_t bit_hi, uint64_t chunk_bits,
                          uint64_t* first, uint64_t nchunks) {
    uint8_t* pad = (uint8_t*)calloc((size_t)size + 32, 1);
    memcpy(pad, in, (size_t)size);
    for (uint64_t c = 0; c < nchunks; c++) first[c] = UINT64_MAX;
    for (uint64_t bit = bit_lo + 1; bit < bit_hi; bit++) {
        uint64_t c = (bit - bit_lo) / chunk_bits;
        if (c >= nchunks || first[c] != UINT64_MAX) continue;
        uint64_t byte = bit >> 3;
        uint64_t v1 = 0, v2 = 0;
        uint8_t tmp[24] = {0};
        uint64_t avail = size + 32 > byte ? size + 32 - byte : 0;
        memcpy(tmp, pad + byte, (size_t)(avail < 24 ? avail : 24));
        uint64_t a = load64(tmp), bb = load64(tmp + 8), cc = load64(tmp + 16);
        int o = (int)(bit & 7);
        v1 = o ? (a >> o) | (bb << (64 - o)) : a;
        v2 = o ? (bb >> o) | (cc << (64 - o)) : bb;
        if (oracle_prefilter128(v1, v2) && oracle_plausible_dynamic_header(in, size, bit)) first[c] = bit;
    }
    free(pad);
}

/* ------------------------------------------------------------------ CRC-32 */

static uint32_t crc_table[256];
static int crc_ready;

static void crc_init(void) {
    for (uint32_t n = 0; n < 256; n++) {
        uint32_t c = n;
        for (int k = 0; k < 8; k++) c = c & 1 ? 0xEDB88320u ^ (c >> 1) : c >> 1;
        crc_table[n] = c;
    }
    crc_ready = 1;
}

/* gzip's CRC-32, continued from crc (0 to start) */
uint32_t oracle_crc32(uint32_t crc, const uint8_t* p, uint64_t n) {
    if (!crc_ready) crc_init();
    uint32_t c = ~crc;
    for (uint64_t i = 0; i < n; i++) c = crc_table[(c ^ p[i]) & 0xff] ^ (c >> 8);
    return ~c;
}
