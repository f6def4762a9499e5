/* gi_oracle_parallel.c - TEST INFRASTRUCTURE ONLY: the CPU baseline timed beside the GPU path.
 *
 * A multi-threaded CPU inflate of one raw Deflate stream, restating the reference's own
 * multi-threaded CPU decoder of a single stream (cpu_speculative, research/gpu-inflate/
 * gpuinflate.cu:258-347) on the oracle's sequential decoder (gi_oracle.c, included below so the
 * two share one translation unit and its helpers; the Makefile builds liboracle.so from this file):
 *   1. block starts: every 4 KiB chunk of input is searched, in parallel, for its first bit that
 *      passes the reference's prefilter and the full dynamic-header check (gpuinflate.cu:271-283);
 *   2. one job per start, in parallel: a decode from the start until it reaches another start at
 *      a block boundary (it "lands" there), the final block ends, or the data fails; a byte it
 *      copies from before its own start is written as a marker 256 + w, "the w-th byte before
 *      the job's start" (gpuinflate.cu:304-316 decodes its jobs with the same meaning);
 *   3. the chain from the stream's start: each job's landing names the next job (gpuinflate.cu:
 *      318-322 stitches the same way);
 *   4. every output position gets a LIT-tagged byte or the absolute position it copies, and each
 *      one follows its chain back to a byte, in parallel (gpuinflate.cu:323-341 resolves by
 *      pointer jumping over the same 32-bit entries).
 * The reference also resynchronizes inside long blocks with probes; the blocks of the streams
 * measured here hold at most 32 Ki symbols, so jobs from block starts alone keep every thread busy.
 *
 * Only tests and bench.py's CPU-baseline leg load it.
 */
#include "gi_oracle.c"

#include <pthread.h>
#include <time.h>

#define P_LIT 0x80000000u

enum { J_LANDED = 0, J_FINAL = 1, J_FAILED = 2, J_STOPPED = 3 };

typedef struct {
    uint16_t* sym; /* a byte (< 256), or 256 + w: the w-th byte before the job's start */
    uint64_t n, cap;
    int status;
    int64_t landed; /* the start it landed on */
} pjob;

typedef struct {
    const uint8_t* pad;       /* the input followed by 32 zero bytes */
    uint64_t size;
    uint64_t scan_bits;       /* starts are searched in [0, scan_bits) */
    uint64_t chunk_bits;      /* one start per chunk of this many bits */
    uint64_t* first;          /* per chunk: its first start, or UINT64_MAX */
    uint64_t nchunks;
    uint64_t* starts;         /* sorted */
    uint64_t nstarts;
    pjob* jobs;
    uint64_t* piece_job;      /* the chain: the job of each piece, and where its output goes */
    uint64_t* piece_at;
    uint64_t npieces;
    uint32_t* e;              /* per output position: P_LIT | byte, or the position it copies */
    uint8_t* out;
    uint64_t out_len;
    uint64_t next;            /* the shared work counter of the current phase */
    int phase;
    int failed;
} pstate;

static int reserve(pjob* j, uint64_t need) {
    uint64_t cap = j->cap ? j->cap : 16384;
    while (cap < need) cap *= 2;
    uint16_t* s = (uint16_t*)realloc(j->sym, cap * sizeof(uint16_t));
    if (!s) return -1;
    j->sym = s;
    j->cap = cap;
    return 0;
}

static inline int push_sym(pjob* j, uint16_t v) {
    if (j->n == j->cap && reserve(j, j->n + 1)) return -1;
    j->sym[j->n++] = v;
    return 0;
}

/* job k: a decode from starts[k] until it lands on a later start at a block boundary */
static void run_job(const pstate* st, uint64_t k, otables* t) {
    pjob* j = &st->jobs[k];
    obits b = {st->pad, st->size, st->size * 8, st->starts[k]};
    uint64_t next = k + 1;
    const int stream_start = k == 0;
    j->status = J_FAILED;
    j->landed = -1;
    for (;;) {
        while (next < st->nstarts && st->starts[next] < b.pos) next++;
        if (next < st->nstarts && st->starts[next] == b.pos) {
            j->status = J_LANDED;
            j->landed = (int64_t)next;
            return;
        }
        if (b.pos >= st->scan_bits && st->scan_bits < st->size * 8) { /* past the last start searched */
            j->status = J_STOPPED;
            return;
        }
        if (b.pos >= b.size_bits) return;
        const int final = (int)getbits(&b, 1);
        const int type = (int)getbits(&b, 2);
        if (type == 0) {
            if (b.pos & 7) getbits(&b, 8 - (int)(b.pos & 7));
            const uint32_t len = getbits(&b, 16), nlen = getbits(&b, 16);
            const uint64_t byte = b.pos >> 3;
            if (len != (~nlen & 0xffffu) || byte + len > st->size) return;
            for (uint32_t q = 0; q < len; q++)
                if (push_sym(j, st->pad[byte + q])) return;
            b.pos = (byte + len) * 8;
        } else {
            if (type == 3) return;
            if (type == 1) fixed_tables(t);
            else if (dynamic_tables(t, &b) != 0) return;
            for (;;) {
                if (b.pos > b.size_bits) return;
                int sym = huff_decode(&t->lit, &b);
                if (sym < 0) return;
                if (sym < 256) {
                    if (push_sym(j, (uint16_t)sym)) return;
                    continue;
                }
                if (sym == 256) break;
                sym -= 257;
                if (sym >= 29) return;
                const uint32_t len = len_base[sym] + getbits(&b, len_extra[sym]);
                const int ds = huff_decode(&t->dist, &b);
                if (ds < 0 || ds >= 30) return;
                const uint32_t d = dist_base[ds] + getbits(&b, dist_extra[ds]);
                if (stream_start && d > j->n) return; /* a match before the stream's start */
                if (j->n + len > j->cap && reserve(j, j->n + len)) return;
                uint16_t* o = j->sym + j->n;
                for (uint32_t q = 0; q < len; q++) {
                    const int64_t src = (int64_t)(j->n + q) - (int64_t)d;
                    o[q] = src >= 0 ? j->sym[src] : (uint16_t)(256 + (uint64_t)(-src));
                }
                j->n += len;
            }
        }
        if (final) {
            j->status = J_FINAL;
            return;
        }
    }
}

static void* worker(void* arg) {
    pstate* st = (pstate*)arg;
    otables* t = (otables*)calloc(1, sizeof(otables));
    if (!t) {
        st->failed = 1;
        return NULL;
    }
    for (;;) {
        const uint64_t i = __atomic_fetch_add(&st->next, 1, __ATOMIC_RELAXED);
        if (st->phase == 0) { /* the first start of chunk i */
            if (i >= st->nchunks) break;
            const uint64_t lo = i * st->chunk_bits, hi = lo + st->chunk_bits < st->scan_bits ? lo + st->chunk_bits : st->scan_bits;
            st->first[i] = UINT64_MAX;
            /* 32 offsets at a time: the first test (BTYPE 2, HLIT and HDIST at most 29) on the
             * bits of a 64-bit window at once, the prefilter's code-length test and the full
             * header check on the offsets that pass it */
            for (uint64_t base = lo & ~31ull; base < hi && st->first[i] == UINT64_MAX; base += 32) {
                const uint64_t w = load64(st->pad + (base >> 3));
                uint32_t m = (uint32_t)(~(w >> 1) & (w >> 2) & ~((w >> 4) & (w >> 5) & (w >> 6) & (w >> 7)) &
                                        ~((w >> 9) & (w >> 10) & (w >> 11) & (w >> 12)));
                while (m) {
                    const int o = __builtin_ctz(m);
                    m &= m - 1;
                    const uint64_t bit = base + (uint64_t)o;
                    if (bit < lo || bit >= hi || bit == 0) continue;
                    const uint8_t* q = st->pad + (bit >> 3);
                    const int sh = (int)(bit & 7);
                    const uint64_t a = load64(q), b8 = load64(q + 8), c = load64(q + 16);
                    const uint64_t v1 = sh ? (a >> sh) | (b8 << (64 - sh)) : a;
                    const uint64_t v2 = sh ? (b8 >> sh) | (c << (64 - sh)) : b8;
                    if (oracle_prefilter128(v1, v2) && plausible_padded(st->pad, st->size, bit)) {
                        st->first[i] = bit;
                        break;
                    }
                }
            }
        } else if (st->phase == 1) { /* job i */
            if (i >= st->nstarts) break;
            run_job(st, i, t);
        } else if (st->phase == 2) { /* the entries of piece i */
            if (i >= st->npieces) break;
            const pjob* j = &st->jobs[st->piece_job[i]];
            const uint64_t at = st->piece_at[i];
            const uint64_t n = i + 1 < st->npieces ? st->piece_at[i + 1] - at : st->out_len - at;
            for (uint64_t q = 0; q < n; q++) {
                const uint16_t v = j->sym[q];
                st->e[at + q] = v < 256 ? (P_LIT | v) : (uint32_t)(at - (uint64_t)(v - 256));
            }
        } else { /* positions [i * 2^20, ...): each follows its chain back to a byte */
            const uint64_t a = i << 20;
            if (a >= st->out_len) break;
            const uint64_t end = a + (1u << 20) < st->out_len ? a + (1u << 20) : st->out_len;
            for (uint64_t p = a; p < end; p++) {
                uint32_t v = __atomic_load_n(&st->e[p], __ATOMIC_RELAXED);
                while (!(v & P_LIT)) v = __atomic_load_n(&st->e[v], __ATOMIC_RELAXED);
                __atomic_store_n(&st->e[p], v, __ATOMIC_RELAXED);
                st->out[p] = (uint8_t)v;
            }
        }
    }
    free(t);
    return NULL;
}

static void run_phase(pstate* st, int phase, int threads) {
    st->phase = phase;
    st->next = 0;
    pthread_t th[256];
    int n = threads < 1 ? 1 : threads > 256 ? 256 : threads;
    for (int i = 0; i < n; i++)
        if (pthread_create(&th[i], NULL, worker, st) != 0) {
            n = i;
            break;
        }
    if (n == 0) worker(st);
    for (int i = 0; i < n; i++) pthread_join(th[i], NULL);
}

static double seconds_since(struct timespec* t0) {
    struct timespec t1;
    clock_gettime(CLOCK_MONOTONIC, &t1);
    const double s = (double)(t1.tv_sec - t0->tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0->tv_nsec);
    *t0 = t1;
    return s;
}

/* The first up to out_cap bytes of the raw Deflate stream in[0..size), decoded by `threads`
 * threads; one block start is searched per chunk of chunk_bytes (the reference's chunk size
 * argument) in the first scan_bytes of input (jobs from them must cover out_cap bytes of output). *out_len: bytes written. Returns O_OK; O_DATA when the chain from the
 * stream's start breaks before out_cap bytes or the stream's end; -1 when memory runs out. phase_s
 * (if given) gets the seconds of the block-start search, the jobs, and the resolution. */
int oracle_inflate_parallel(const uint8_t* in, uint64_t size, uint64_t scan_bytes, uint64_t chunk_bytes, uint8_t* out,
                            uint64_t out_cap, uint64_t* out_len, int threads, double* phase_s) {
    pstate st;
    memset(&st, 0, sizeof st);
    double secs[3] = {0, 0, 0};
    struct timespec t0;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    int rc = O_OK;
    uint8_t* pad = (uint8_t*)calloc((size_t)size + 32, 1);
    if (!pad) return -1;
    memcpy(pad, in, (size_t)size);
    st.pad = pad;
    st.size = size;
    st.scan_bits = (scan_bytes < size ? scan_bytes : size) * 8;
    st.chunk_bits = (chunk_bytes ? chunk_bytes : 4096) * 8;
    st.nchunks = (st.scan_bits + st.chunk_bits - 1) / st.chunk_bits;
    if (!st.nchunks) st.nchunks = 1;
    st.first = (uint64_t*)malloc(st.nchunks * sizeof(uint64_t));
    st.starts = (uint64_t*)malloc((st.nchunks + 1) * sizeof(uint64_t));
    if (!st.first || !st.starts) {
        rc = -1;
        goto done;
    }
    run_phase(&st, 0, threads);
    st.starts[0] = 0;
    st.nstarts = 1;
    for (uint64_t c = 0; c < st.nchunks; c++)
        if (st.first[c] != UINT64_MAX && st.first[c] > st.starts[st.nstarts - 1]) st.starts[st.nstarts++] = st.first[c];
    secs[0] = seconds_since(&t0);
    st.jobs = (pjob*)calloc(st.nstarts, sizeof(pjob));
    st.piece_job = (uint64_t*)malloc(st.nstarts * sizeof(uint64_t));
    st.piece_at = (uint64_t*)malloc(st.nstarts * sizeof(uint64_t));
    if (!st.jobs || !st.piece_job || !st.piece_at) {
        rc = -1;
        goto done;
    }
    run_phase(&st, 1, threads);
    secs[1] = seconds_since(&t0);
    { /* the chain from the stream's start, up to out_cap bytes */
        uint64_t k = 0, at = 0;
        for (;;) {
            st.piece_job[st.npieces] = k;
            st.piece_at[st.npieces++] = at;
            at += st.jobs[k].n;
            if (at >= out_cap) {
                at = out_cap;
                break;
            }
            if (st.jobs[k].status == J_FINAL) break;
            if (st.jobs[k].status != J_LANDED || st.npieces == st.nstarts) {
                rc = O_DATA;
                goto done;
            }
            k = (uint64_t)st.jobs[k].landed;
        }
        st.out_len = at;
    }
    if (st.out_len >= P_LIT) { /* entries hold positions below 2^31 */
        rc = -1;
        goto done;
    }
    st.e = (uint32_t*)malloc((st.out_len + 1) * sizeof(uint32_t));
    if (!st.e) {
        rc = -1;
        goto done;
    }
    st.out = out;
    run_phase(&st, 2, threads);
    run_phase(&st, 3, threads);
    secs[2] = seconds_since(&t0);
    *out_len = st.out_len;
    if (st.failed) rc = -1;
done:
    if (st.jobs)
        for (uint64_t k = 0; k < st.nstarts; k++) free(st.jobs[k].sym);
    free(st.jobs);
    free(st.e);
    free(st.piece_job);
    free(st.piece_at);
    free(st.first);
    free(st.starts);
    free(pad);
    if (phase_s)
        for (int i = 0; i < 3; i++) phase_s[i] = secs[i];
    return rc;
}
