// gi_common.cuh - types shared by the host orchestration and the kernels of libgpuinflate.
//
// The speculative scheme follows gpuzip's gpuinflate (gpuinflate/inflate.cuh:43-68,
// gpuinflate/gpuinflate.cu:1-17): decoders start at guessed block starts, each runs until it
// lands exactly on a later start, and writes 16-bit symbols (a byte, or "the byte d back")
// that are resolved afterwards. What differs is where the work happens: a decoder is a whole
// warp (uniform control flow, lanes cooperate on tables and stores), a decoder whose buffer
// fills takes a new extent from a device pool instead of waiting for another round, and the
// finder tests 32 bit offsets per lane with bit-sliced masks.
#pragma once
#include <stdint.h>

namespace gz {

constexpr uint32_t WINDOW = 32768;
constexpr uint32_t MAX_SYMBOL_OUT = 258;       // most positions one symbol writes
constexpr uint32_t REF = 255;                  // symbol values above REF: the byte (value - REF) back
constexpr uint32_t FIRST_RUN_BLOCKS = 65536;   // references before the start are checked at once in these blocks
constexpr uint32_t LIT = 0x80000000u;          // resolved entry: a byte (low 8 bits); else the position it copies

// where a decoder starts, or a state an extent starts in (inflate.cuh:43-53 has the same three)
enum : uint8_t { AT_BLOCK = 0, IN_FIXED = 1, IN_DYNAMIC = 2 };

// how a decode ended (the values of inflate.cuh:41)
enum : int32_t { S_OK = 0, S_DATA = 1, S_OVERFLOW = 2, S_INPUT = 3, S_STOPPED = 4 };

struct Start {
    uint64_t bit;
    uint64_t header;  // IN_DYNAMIC: the block's header; AT_BLOCK: = bit; IN_FIXED: unused
    uint8_t mode;
    int8_t final;     // BFINAL of the block it is inside: 0, 1, or -1 unknown
    uint8_t pad[6];
};
static_assert(sizeof(Start) == 24, "Start layout");

// a stream (or the current segment of one) inside the device input buffer, in bits of that buffer
struct StreamDesc {
    uint64_t end_bit;   // the input ends here: reading past it gives zero bits and an input error
    uint64_t end_word;  // first 32-bit word past the input (loads from it on return zero)
    uint64_t stop;      // decoders stop at the first block or symbol boundary at or after this bit
    int32_t target_end; // the stream's targets are [first target, target_end)
    int32_t check_refs; // its first job starts the stream: a reference before the start is invalid at once
};

struct Job {
    Start start;
    int32_t stream;
    int32_t tfirst;     // may land on targets[tfirst .. target_end)
    uint64_t pool_off;  // its first extent, in 16-bit symbols (a multiple of 32)
    uint32_t cap;       // the first extent's size (a multiple of 32)
    uint32_t flags;     // JOB_CHECK_REFS
};
constexpr uint32_t JOB_CHECK_REFS = 1;
// the job's output is not kept: it writes over its first extent again and again (which must hold
// DISCARD_EXTENT symbols: a stored block and a match), for decodes only their results are wanted from
constexpr uint32_t JOB_DISCARD = 2;
// a job whose start is known to be in step (a segment's or a stream's start): never given up
constexpr uint32_t JOB_TRUSTED = 4;
constexpr int32_t GIVE_UP_AFTER = 2;  // DecodeArgs.give_up of the segmented path (0 in batched passes and the rescue)
constexpr uint32_t DISCARD_EXTENT = 65536 + 512;

struct JobResult {
    uint64_t end_bit;    // where it stopped
    uint64_t eob_bit;    // just past its first end-of-block code (UINT64_MAX: none)
    uint64_t out_len;    // symbols written, all extents
    uint64_t eob_out;    // symbols written before eob_bit
    Start resume;        // S_OVERFLOW / S_STOPPED: the exact state to go on from
    int32_t status;
    int32_t landed;      // target index it landed on, -1: none (end of stream, stop or error)
    int32_t end_final;   // BFINAL of the block it ended in, -1 unknown
    uint32_t blocks;     // block headers read
    uint64_t cycles;     // SM clock cycles the job took (diagnostics)
    uint64_t hdr0;       // header of the first block it decoded symbols of (diagnostics)
    uint64_t symbols;    // literals and matches decoded (an encoder's blocks hold a regular number)
    uint64_t last_block_bit;  // header of the last block it began (UINT64_MAX: none)
    uint64_t last_block_out;  // symbols written before that header
    uint64_t t_begin, t_end;  // the GPU's global timer (ns) when the job began and ended (diagnostics)
};

// a run of a job's output in the pool; job k's first extent is extent k
struct Extent {
    uint64_t pool_off;
    uint64_t len;
    uint64_t cap;
    Start start;         // the decoder's exact state where the extent begins
    int32_t next;        // the job's next extent, -1: last
    int32_t job;
};

// a stored block the decoder skipped: its bytes go to the pool later, 16 bytes at a time
struct StoredCopy {
    uint64_t src;        // byte offset in the device input
    uint64_t dst;        // symbol offset in the pool
    uint32_t len;
    uint32_t pad;
};

// device counters of one decode launch
struct Counters {
    int32_t next_job;
    int32_t n_ext;
    int32_t n_stored;
    int32_t pad;
    unsigned long long pool_used;
};

struct DecodeArgs {
    const uint8_t* in;
    const StreamDesc* streams;
    const Job* jobs;
    const Start* targets;
    const int32_t* order;   // job order (longest first)
    int32_t njobs;
    int32_t ext_cap;
    int32_t stored_cap;
    // a job that starts inside a block (at a probe point), is not JOB_TRUSTED, and passes this
    // many targets at block starts (AT_BLOCK) without landing on one stops there (S_STOPPED, its
    // exact state in resume): a decoder in step lands on every real block start it reaches, so it
    // is out of step, decoding garbage that a periodic code stream can keep valid for hundreds of
    // kilobytes. (Jobs from block starts never give up: the finder's spurious hits inside a block
    // of near-random codes would stop correct ones.) 0: never.
    int32_t give_up;
    uint16_t* pool;
    uint64_t pool_cap;
    JobResult* res;
    Extent* ext;
    StoredCopy* stored;
    Counters* ctr;
};

// probe points of one span: first_point + i * spacing for i < npoints, with the tables of `start`
struct ProbeSpan {
    Start start;
    uint64_t first_point;
    uint64_t spacing;
    uint32_t npoints;
    uint32_t out_index;  // results go to out[out_index + i]
};

struct ProbeArgs {
    const uint8_t* in;
    uint64_t end_word;
    const ProbeSpan* spans;
    int32_t nspans;
    uint32_t lead;      // bits decoded before a point to fall into step
    Start* out;
    uint32_t attempts;  // restarts one bit later a probe makes before giving up on a point
};

// a run of the segment's output: pool[src .. src+len) goes to output position dst
struct Piece {
    uint64_t src;
    uint64_t dst;
    uint64_t len;
};

// launchers (each file owns its kernels)
// a byte position whose 16-bit LEN and NLEN fields look like a stored block's (NLEN = ~LEN)
struct StoredCand {
    uint64_t byte;
    uint64_t len;
};

// each launcher returns how many kernels it launched
// d_first gets FIND_SLOTS_PER_CHUNK entries per chunk: the chunk's first block starts in bit order,
// UINT64_MAX where there are fewer. skip (may be null): chunks flagged nonzero are not scanned
// (they lie inside stored blocks)
constexpr int FIND_SLOTS_PER_CHUNK = 4;
// per-chunk flags of launch_find's `skip` (may be NULL): a chunk wholly inside trusted stored
// blocks (not searched); a chunk near a stream's end (final-block headers kept too)
constexpr uint8_t SKIP_CHUNK = 1, FINAL_CHUNK = 2;
constexpr uint64_t FINAL_TAIL_BITS = (256ull << 10) * 8;  // how near: the last 256 KiB of a stream's input
int launch_find(const uint8_t* d_in, uint64_t bit_lo, uint64_t bit_hi, uint64_t end_word, uint32_t chunk_bits,
                uint64_t nchunks, uint64_t* d_first, uint64_t end_bit, const uint8_t* skip, void* stream);
// every position in (bit_lo, bit_hi) that passes the full dynamic-header check, appended to out
// in no order (*n counts them all, including those past cap)
int launch_find_all(const uint8_t* d_in, uint64_t bit_lo, uint64_t bit_hi, uint64_t end_word, uint64_t end_bit,
                    uint64_t* out, unsigned* n, unsigned cap, void* stream);
// for the block starting at each bits[i]: (output bytes, codes) per compressed bit, predicted
// from its header's code lengths ((0, 0) for UINT64_MAX or no valid header)
int launch_density(const uint8_t* d_in, uint64_t end_word, const uint64_t* bits, uint64_t n, float2* out, void* stream);
int launch_stored_scan(const uint8_t* d_in, uint64_t byte_lo, uint64_t byte_hi, uint64_t end_word, uint64_t end_byte,
                       StoredCand* out, unsigned* n, unsigned cap, void* stream);
constexpr int DECODE_WARPS = 8;  // decoders (warps) per block of k_decode
int decode_blocks_per_sm();
int launch_decode(const DecodeArgs& a, int grid, void* stream);
int launch_probe(const ProbeArgs& a, int grid, void* stream);
int launch_stored(const uint8_t* d_in, uint16_t* pool, const StoredCopy* list, int n, void* stream);
// byte ranges the GPU reads directly (page-locked host or device memory) copied into dst: one
// kernel for all of them; each piece at most GATHER_PIECE bytes
constexpr uint64_t GATHER_PIECE = 256 << 10;
struct GatherPiece {
    const uint8_t* src;
    uint64_t dst;  // offset in dst
    uint64_t len;
};
int launch_gather(const GatherPiece* pieces, uint64_t n, uint8_t* dst, void* stream);
// the output is resolved in spans of at most this many positions (a multiple of 16, at least WINDOW)
constexpr uint64_t SPAN = 512 * 1024;
// a span of output positions [start, end) of one stream; W: bytes of that stream before start that
// the span may copy from (0 at the stream's start, at most WINDOW); start is a multiple of 16
struct SpanDesc {
    uint64_t start, end;
    uint32_t W;
    uint32_t stream;  // bad[stream] is set for a match before the stream's start
    uint32_t piece0;  // the pieces that overlap the span: piece0 .. piece0 + npiece - 1
    uint32_t npiece;
};
// fills piece0/npiece of every span (spans and pieces both sorted, the pieces back to back)
void span_pieces(SpanDesc* spans, uint64_t nspans, const Piece* pieces, uint64_t npieces);
// passes: 1 = local resolution (and the check for matches before the start), 2 = windows and bytes.
// One stream in spans of span_len bytes (a power of two from 64 KiB to SPAN; the first span with W
// bytes of seg_window before it):
// work: one word of device memory the launch uses as the span queue of k_local
int launch_resolve(const uint16_t* pool, const Piece* pieces, int npieces, const SpanDesc* spans, uint64_t nspans,
                   uint64_t span_len, uint64_t total, uint32_t W, const uint8_t* seg_window, uint16_t* out16,
                   uint8_t* windows, int* bad, uint8_t* out, int passes, unsigned* work, void* stream);
// the spans of one stream of `total` output bytes: SPAN, halved (not below 64 KiB, twice a window)
// while the stream has fewer spans than the GPU has SMs, so a small stream's spans are resolved on
// as many blocks as its decode ran on
uint64_t span_length(uint64_t total);
// Many streams (every stream starting at its first span, W 0). A stream of fewer than
// GROUPED_SPANS spans (but more than one) is listed in multi as (first span, span count); a longer
// one is cut into groups of consecutive spans (about the square root of its span count each),
// listed in groups, and its entry in grouped gives its first group and group count.
constexpr uint32_t GROUPED_SPANS = 16;
struct SpanGroup {
    uint32_t first_span, count;
    uint32_t map;  // slot of the group's composed map in `maps` (unused for a stream's last group)
    uint32_t pad;
};
struct GroupedStream {
    uint32_t first_group, ngroups;
};
struct StreamWindows {
    const uint32_t* multi;
    uint32_t nmulti;
    const SpanGroup* groups;
    uint32_t ngroups;
    const GroupedStream* grouped;
    uint32_t ngrouped;
    uint16_t* maps;  // WINDOW 16-bit slots per composed map
};
int launch_resolve_streams(const uint16_t* pool, const Piece* pieces, int npieces, const SpanDesc* spans,
                           uint64_t nspans, const StreamWindows& sw, uint16_t* out16, uint8_t* windows, int* bad,
                           uint8_t* out, int passes, unsigned* work, void* stream);
int resolve_setup();  // once per device: kernel attributes (returns a cudaError_t)
uint64_t resolve_map_slots(uint64_t seg_out_max);  // extra 16-bit slots out16 needs after the output
int launch_next_window(const uint8_t* out, uint64_t total, const uint8_t* old, uint32_t W, uint8_t* nw, uint32_t newW,
                       void* stream);
// CRC-32 of data[0..n) into *result: returns the kernels launched, or -1 (nothing launched) when
// scratch_words words of scratch are fewer than crc_scratch_words(n)
int launch_crc(const uint8_t* data, uint64_t n, uint32_t* scratch, uint64_t scratch_words, uint32_t* result,
                void* stream);
uint64_t crc_scratch_words(uint64_t n);
// loads launch_crc's kernels on the current device now (a cudaError_t), so that a later launch_crc
// takes no device memory for them under lazy module loading
int crc_prepare();

// the current device's SM count (queried once per device)
int sm_count();
// CRC-32 of each of nstreams streams laid out as spans (stream s: spans first_span[s] .. + span_count[s])
int launch_crc_streams(const uint8_t* data, const SpanDesc* spans, uint64_t nspans, uint32_t* span_crc,
                       const uint32_t* first_span, const uint32_t* span_count, uint32_t nstreams, uint32_t* crc,
                       void* stream);

// host-side CRC-32 arithmetic (reflected polynomial 0xEDB88320)
uint32_t crc32_combine_host(uint32_t crc1, uint32_t crc2, uint64_t len2);

}  // namespace gz
