/* gpuinflate.h - C interface of the GB300-native Deflate decoder (libgpuinflate.so).
 *
 * Part 1 is interface version 1 of gpuzip's gpuinflate library, kept symbol for symbol and
 * byte for byte so that gpuzip's Rust host (src/inflate.rs) loads this library unchanged:
 * the same names, the same argument meaning, the same return codes and the same struct
 * layouts. Part 2 adds entry points that the reference does not have; adding symbols does not
 * change version 1.
 *
 * One context serves one call at a time; use one context per host thread. */
#ifndef GPUINFLATE_H
#define GPUINFLATE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(GI_BUILD) && defined(__GNUC__)
#define GI_API __attribute__((visibility("default")))
#else
#define GI_API
#endif

/* ------------------------------------------------------------------ part 1: interface 1 */

/* reference: gpuinflate/gpuinflate.h:31 */
#define GI_ABI_VERSION 1

/* Return codes. reference: gpuinflate/gpuinflate.h:33-40 (same values) */
enum {
    GI_OK = 0,
    GI_ERR_DATA = 1,      /* not a valid Deflate stream (a match reaching before the start included) */
    GI_ERR_TRUNCATED = 2, /* the input stops before the stream's final block ends (or is empty) */
    GI_ERR_ABORTED = 3,   /* the sink asked to stop */
    GI_ERR_GPU = 4,       /* no usable GPU, GPU memory exhausted, or a CUDA failure */
    GI_ERR_ARG = 5,       /* an invalid argument */
    GI_ERR_SPACE = 6      /* part 2 only: the output does not fit the caller's buffer */
};

typedef struct gi_ctx gi_ctx;

/* reference: gpuinflate/gpuinflate.h:44-49 (16 bytes; same fields, same order) */
typedef struct {
    uint32_t size;           /* sizeof(gi_config); smaller is an argument error */
    int32_t device;          /* CUDA device ordinal */
    uint32_t segment_out_mb; /* largest output of one segment in MiB; 0 picks it from free GPU memory */
    uint32_t segment_in_kb;  /* compressed input per segment in KiB; 0 picks it from the stream's ratio */
} gi_config;

/* reference: gpuinflate/gpuinflate.h:51-59 (80 bytes; same fields, same order) */
typedef struct {
    uint64_t in_used;  /* input bytes the stream occupies, through its final block, rounded up to a byte */
    uint64_t out_size; /* output bytes produced */
    uint32_t segments; /* segments the stream was decoded in */
    uint32_t rounds;   /* decode launches, all segments */
    uint64_t jobs;     /* speculative decoders started, all segments */
    double seconds;    /* wall time of the whole call */
    double upload_s, find_s, decode_s, resolve_s, download_s; /* GPU time per stage */
} gi_stats;

/* Gets the output in stream order, always from one thread owned by the library, never two
 * calls at once; the bytes are valid only during the call. A nonzero return stops the decode
 * (GI_ERR_ABORTED). reference: gpuinflate/gpuinflate.h:61-63 */
typedef int (*gi_sink)(void* user, const uint8_t* data, size_t len);

/* reference: gpuinflate/gpuinflate.h:65 (returns GI_ABI_VERSION) */
GI_API uint32_t gi_abi_version(void);

/* Creates a context on cfg->device (cfg NULL: device 0, automatic sizes) and allocates its GPU
 * and pinned host buffers. On failure *ctx is NULL and err (if given) describes the cause.
 * reference: gpuinflate/gpuinflate.h:69, gpuinflate/gpuinflate.cu:881-907 */
GI_API int gi_create(const gi_config* cfg, gi_ctx** ctx, char* err, size_t err_len);

/* Decodes the raw Deflate stream that begins at in[0]. Bytes after the final block are
 * allowed and are not read beyond what the stream needs; stats->in_used says where it ended.
 * out_hint is the expected output size or 0; it only sizes the first segment. sink may be
 * NULL (output discarded after it reaches host memory); stats may be NULL and is filled on
 * every return. in NULL with in_size > 0 is GI_ERR_ARG; in_size 0 is GI_ERR_TRUNCATED.
 * reference: gpuinflate/gpuinflate.h:74-75, gpuinflate/gpuinflate.cu:909-940 */
GI_API int gi_inflate(gi_ctx* ctx, const uint8_t* in, uint64_t in_size, uint64_t out_hint, gi_sink sink, void* user,
                      gi_stats* stats);

/* Text of the last failure on ctx, valid until the next call on ctx.
 * reference: gpuinflate/gpuinflate.h:78 */
GI_API const char* gi_last_error(const gi_ctx* ctx);

/* Name of the context's GPU. reference: gpuinflate/gpuinflate.h:81 */
GI_API const char* gi_device_name(const gi_ctx* ctx);

/* Frees the context and its buffers. reference: gpuinflate/gpuinflate.h:83 */
GI_API void gi_destroy(gi_ctx* ctx);

/* ------------------------------------------------------------------ part 2: additions */

/* CRC-32 (gzip's, reflected 0xEDB88320) and byte count mod 2^32 of the output of the last
 * call on ctx that returned GI_OK, both computed on the GPU. No counterpart in the reference:
 * its caller folds every sink chunk into crc32fast (src/gz.rs:207-247). */
GI_API uint32_t gi_last_crc32(const gi_ctx* ctx);
GI_API uint32_t gi_last_isize(const gi_ctx* ctx);

/* Device-resident form: the raw Deflate stream is already in GPU memory (d_in, in_size bytes,
 * on ctx's device) and the output goes to GPU memory (d_out, out_cap bytes). *out_size gets
 * the output length; an output longer than out_cap returns GI_ERR_SPACE. Same error classes
 * and in_used as gi_inflate. No counterpart in the reference (its input always comes from
 * host memory, gpuinflate/gpuinflate.cu:672-692). */
GI_API int gi_inflate_device(gi_ctx* ctx, const void* d_in, uint64_t in_size, void* d_out, uint64_t out_cap,
                             uint64_t* out_size, gi_stats* stats);

/* One gzip member (RFC 1952) at in[0]: header parsed as gpuzip's src/gz.rs:62-110 does, the
 * raw stream decoded as gi_inflate does, then the trailer's CRC-32 and ISIZE checked against
 * the values computed on the GPU (src/gz.rs:236-247 does that check on the host). A mismatch
 * is GI_ERR_DATA. *member_size (may be NULL) gets the member's size including its trailer. */
GI_API int gi_inflate_gzip(gi_ctx* ctx, const uint8_t* in, uint64_t in_size, gi_sink sink, void* user,
                           uint64_t* member_size, gi_stats* stats);

/* The batched form: n independent streams decoded together, in as few passes over the GPU as the
 * context's buffers allow (one launch of each kernel for all streams of a pass). Every stream's
 * output goes to out + out_offset (16-byte aligned, in order), its CRC-32 is computed on the GPU.
 * Returns GI_OK when the call ran; each stream has its own status (GI_ERR_SPACE when its output
 * did not fit out_cap). No counterpart in the reference (one stream per gi_inflate call, a
 * context serving one call at a time: gpuinflate/gpuinflate.h:8); it replaces gpuzip's
 * per-member calls (src/gz.rs:154-264) and its nvCOMP batches for ZIP entries
 * (src/extract.rs:458-597). */
#define GI_STREAM_GZIP 1u /* `in` is a gzip member: header parsed, trailer CRC-32 and ISIZE checked */
#define GI_STREAM_CRC 2u  /* expected_crc holds the output's CRC-32 (a ZIP entry): checked */
#define GI_STREAM_MAPPED 4u /* `in` is memory the GPU reads directly (page-locked host memory from
                             * cudaHostAlloc/cudaHostRegister, or device memory): such streams are
                             * gathered by one kernel instead of one copy call each */

typedef struct {
    const uint8_t* in;     /* the stream (host memory; see GI_STREAM_MAPPED) */
    uint64_t in_size;
    uint32_t flags;        /* GI_STREAM_GZIP, GI_STREAM_CRC */
    uint32_t expected_crc;
    uint64_t out_offset;   /* set: where its output starts in out */
    uint64_t out_size;     /* set */
    uint64_t in_used;      /* set: bytes of in the stream took (a gzip member: through its trailer) */
    uint32_t crc32;        /* set: CRC-32 of its output */
    int32_t status;        /* set: GI_OK or the error of this stream */
} gi_stream;

GI_API int gi_inflate_batch(gi_ctx* ctx, gi_stream* streams, uint32_t n, uint8_t* out, uint64_t out_cap,
                            gi_stats* stats);

/* Where the GPU time of the last call on ctx went, per kernel kind (CUDA events around every
 * launch on the context's stream), and what the call moved. No counterpart in the reference
 * (its gi_stats has only the five stage times, which part 1 keeps). */
typedef struct {
    uint32_t size;          /* sizeof(gi_profile), set by the caller */
    uint32_t launches;      /* kernels the call launched */
    double kernel_ms[7];    /* find (block starts and probes), decode, stored copies, span-local resolution,
                               span windows and bytes, the next segment's window, CRC-32 */
    uint32_t decode_launches, reserved;
    uint64_t in_bytes;      /* compressed bytes uploaded, all segments */
    uint64_t out_bytes;     /* bytes produced */
    uint64_t jobs, extents, stored_blocks;
    uint64_t probes;        /* probe points (resynchronization inside long blocks) */
    /* the planner's setting the call used, chosen by the context's autotuner for this class of
     * stream (gi_inflate, gi_inflate_device, gi_inflate_gzip): the farthest apart probe points
     * are (bits), the bits a probe decodes before its point, the divisor of a decoder's average
     * work that gives one job's share; tuned: 0 while the class's candidates are being tried
     * (one per call), 1 once the fastest was chosen */
    uint32_t probe_spacing_bits, probe_lead_bits;
    float job_share_div;
    uint32_t tuned;
} gi_profile;

GI_API int gi_last_profile(const gi_ctx* ctx, gi_profile* profile);

/* CRC-32 (gzip's) of size bytes already in GPU memory on `device`, written to *d_crc (a device
 * pointer), launched on `stream` (a cudaStream_t; NULL for the default stream) without waiting.
 * For callers that cannot allocate device memory: it allocates nothing, its scratch is a fixed
 * 1 MiB array that every GPU loading this library holds until the process exits. Limits: at
 * most 1 GiB per call, d_data 16-byte aligned (else GI_ERR_ARG, with the reason in err). The
 * first call on a device sets it up there (looks the array up and loads the CRC kernels); under
 * CUDA's lazy module loading that is when the driver places the array and the kernels in device
 * memory, so make that first call (size 0 is enough) before reserving the rest of the device's
 * memory and before any stream capture on that device; later calls take no device memory. Calls
 * that overlap on one device share the array and race. No counterpart in the reference (its CRC
 * is computed on the host by its caller). */
GI_API int gi_crc32_device_noalloc(int device, const void* d_data, uint64_t size, uint32_t* d_crc, void* stream,
                                   char* err, size_t err_len);

/* The entries of a tar archive that lies decoded in GPU memory (by gi_inflate_device, say, from a
 * .tar.gz member): every 512-byte block is tested for a header on the GPU at once, then the
 * chain of headers is walked from the archive's start, GNU long names ('L') and pax records
 * ('x': path, size) applied to the entry that follows them, up to the all-zero block that ends
 * the archive. d_tar must be 16-byte aligned. *tar gets the entries in archive order (free with
 * gi_tar_free); GI_ERR_DATA when a header fails its checksum or the archive ends inside one
 * (gi_last_error says where). No counterpart in the reference, whose host reads the decoded
 * stream through a tar reader (src/gz.rs:622-785). */
typedef struct {
    const char* name;   /* the entry's path: its pax path, else its GNU long name, else its header's
                           (a ustar prefix joined to it); valid until gi_tar_free */
    uint64_t header;    /* offset of its own header in the archive (after any long-name or pax
                           entries that name it, as the tar crate's raw_header_position) */
    uint64_t offset;    /* offset of its data */
    uint64_t size;      /* bytes of data */
    uint32_t type;      /* its typeflag byte: '0' or 0 a file, '5' a folder, '1'/'2' links, ... */
    uint32_t reserved;
} gi_tar_entry;

typedef struct gi_tar gi_tar;

GI_API int gi_tar_index_device(gi_ctx* ctx, const void* d_tar, uint64_t size, gi_tar** tar);
GI_API uint32_t gi_tar_entries(const gi_tar* tar, const gi_tar_entry** entries);
GI_API uint64_t gi_tar_end(const gi_tar* tar);  /* bytes the archive took, through its end block */
GI_API void gi_tar_free(gi_tar* tar);

/* Every gzip member of a file (a .gz, .tgz, a BGZF file, any concatenation of members), decoded
 * as gpuzip's gz::decode does (src/gz.rs:154-264): header rules of parse_header (FHCRC checked,
 * BGZF's "BC" subfield read), each member's trailer CRC-32 and ISIZE checked against values
 * computed on the GPU, the outputs handed to `sink` in order, from a thread the library owns,
 * never two calls at once. After the first member, bytes that are not a gzip member end the
 * file: they are ignored and reported in *info. Members whose size their BGZF header gives are
 * decoded together, many per pass of the batched form (no per-member call); the others one by
 * one through the segmented path; a file in page-locked memory is read by the gather kernel.
 * Errors: GI_ERR_DATA (not gzip, no member, a bad header, invalid Deflate data, a CRC or size
 * mismatch), GI_ERR_TRUNCATED (the input ends inside a member),
 * GI_ERR_ABORTED (the sink stopped), GI_ERR_GPU. No counterpart in the reference, whose host
 * decodes member by member (about 10 ms of GPU call each, src/gz.rs:16-19). */
typedef struct {
    uint32_t size;          /* sizeof(gi_members_info), set by the caller (32) */
    uint32_t members;       /* members decoded */
    uint64_t batched;       /* of which decoded together (their size from a BGZF header) */
    uint64_t trailing;      /* bytes after the last member that are not a gzip member */
    uint32_t trailing_zero; /* 1: those bytes are all zero */
    uint32_t reserved;
} gi_members_info;

GI_API int gi_inflate_members(gi_ctx* ctx, const uint8_t* in, uint64_t in_size, gi_sink sink, void* user,
                              gi_members_info* info, gi_stats* stats);

/* Every entry of a ZIP archive, read as gpuzip's zip.rs reads it (read_central_directory and plan,
 * src/zip.rs:393-540): the end record (Zip64 when present), data prepended to the archive, the
 * central directory with its Zip64 extra fields, each entry's local header, entries whose bytes
 * overlap another's (a zip bomb's trick) left out. Deflate entries are decoded together, many per
 * pass of the batched form, each checked against the directory's CRC-32 and size; stored entries
 * are checked the same way; directories, encrypted entries and other methods are not decoded.
 * The sink gets every entry in directory order, from a thread the library owns, never two calls
 * at once: once per entry (several times, consecutive, for an entry larger than a pass, then
 * once more with data NULL if it failed after its output began), with data NULL when the entry
 * has no output (status says why). A nonzero return stops the call.
 * Returns GI_OK when the directory could be read (entries may fail one by one), GI_ERR_DATA
 * when it cannot ("not a ZIP file", a bad or truncated directory, a bad local header),
 * GI_ERR_ABORTED, GI_ERR_GPU. No counterpart in the reference (its extract.rs sends each large
 * entry to gi_inflate and batches small ones through nvCOMP, src/extract.rs:320-597). */
typedef struct {
    uint32_t size;     /* sizeof(gi_zip_entry) (40) */
    uint32_t index;    /* position in the central directory */
    uint16_t method;   /* 0 stored, 8 deflated, another number: not decoded */
    uint16_t flags;    /* the entry's general-purpose flags (bit 0: encrypted) */
    int32_t status;    /* GI_OK; GI_ERR_DATA (invalid data, or a CRC or size mismatch); GI_ERR_TRUNCATED;
                          GI_ERR_ARG: not decoded (a directory, encrypted, another method, overlapping) */
    uint64_t out_size; /* its size in the directory */
    uint64_t in_size;  /* its compressed size in the directory */
    uint32_t crc32;    /* the directory's CRC-32 */
    uint32_t name_len; /* bytes of the name passed with it */
} gi_zip_entry;

typedef int (*gi_entry_sink)(void* user, const gi_zip_entry* entry, const uint8_t* name, const uint8_t* data,
                             size_t len);

GI_API int gi_inflate_zip(gi_ctx* ctx, const uint8_t* in, uint64_t in_size, gi_entry_sink sink, void* user,
                          gi_stats* stats);

/* ------------------------------------------------------------------ part 3: the request server
 *
 * A request loop over the batched form, for a process that decodes many streams as they come
 * (gpuzip's `test` and `extract` over a stream of archives). No counterpart in the reference,
 * whose host decodes one member per gi_inflate call under a mutex (src/inflate.rs:60, :152).
 *
 * Requests are admitted against an HBM budget: a request's whole input is copied into a
 * resident device arena as soon as the arena has room (in arrival order), so a pass never
 * waits for its uploads. `workers` decode loops, each with its own stream and pass buffers,
 * take every admitted request that fits their next pass when they become free; passes of
 * different workers run on the GPU at the same time, so requests that arrive while a pass is
 * running are decoded beside it, not after it. A request whose output cannot fit a pass is
 * decoded on its own (segmented, from host memory). Results are delivered to a callback. */
typedef struct gi_server gi_server;

typedef struct {
    uint32_t size;          /* sizeof(gi_server_config) (40) */
    int32_t device;
    uint32_t workers;       /* decode loops, i.e. passes that may run at once (0 = 3) */
    uint32_t max_batch;     /* most requests in one pass (0 = 4096) */
    uint32_t pass_out_mb;   /* output of one pass, MiB (0 = 2048, less when the budget is small) */
    uint32_t rescue_workers; /* rescue loops: GI_REQ_RESCUE requests recovered at once (0 = 3, at most 4) */
    uint64_t hbm_budget;    /* device bytes the server may hold: pass buffers + arena + the rescues'
                               allowance (a sixth of the budget, 4-24 GiB; 0 = 120 GB) */
    uint64_t arena_bytes;   /* of which the input arena (0 = the rest of the budget, at most 64 GiB) */
} gi_server_config;

typedef struct {
    uint64_t tag;           /* the caller's tag from gi_server_submit */
    int32_t status;         /* GI_OK, or the error class of gi_inflate / gi_inflate_gzip */
    uint32_t crc32;         /* CRC-32 of the output, computed on the GPU */
    uint64_t out_size;
    uint64_t in_used;       /* bytes of the input the stream took (gzip: through its trailer) */
    double t_submit, t_admit, t_start, t_done;  /* seconds on the server's clock (gi_server_clock) */
    uint32_t pass_requests; /* requests decoded in the same pass (1 for one decoded on its own) */
    uint32_t worker;
} gi_result;

/* data: r->out_size bytes of output (NULL when status != GI_OK), valid only during the call.
 * Called from a thread of the server, never two at once; it may call gi_server_submit, but not
 * gi_server_drain or gi_server_destroy. */
typedef void (*gi_done)(void* user, const gi_result* r, const uint8_t* data);

typedef struct {
    uint32_t size;          /* sizeof(gi_server_stats), set by the caller (104) */
    uint32_t workers;
    uint64_t submitted, completed, failed;
    uint64_t passes;        /* passes run (a request decoded on its own counts as one) */
    uint64_t alone;         /* requests decoded on their own */
    uint64_t overlapped;    /* passes that started while another worker's pass was running */
    uint64_t in_bytes, out_bytes;
    uint64_t device_bytes;  /* device memory the server holds: pass buffers and arena */
    uint64_t arena_bytes, arena_peak;  /* the input arena, and the most of it held at once */
    double busy_s;          /* time during which at least one pass was running */
} gi_server_stats;

GI_API int gi_server_create(const gi_server_config* cfg, gi_done done, void* user, gi_server** server, char* err,
                            size_t err_len);
/* Queues one request; `in` (host memory) must stay valid until its callback has returned.
 * flags: GI_STREAM_GZIP (one gzip member) or GI_STREAM_CRC (raw Deflate with a known CRC-32) or
 * 0 (raw Deflate); or GI_REQ_RESCUE: a damaged gzip member to recover (gzrescue_gb300.h, default
 * options), served in arrival order beside the passes; its callback gets status GI_OK when the
 * rescue gave a result (else GI_ERR_DATA), out_size output bytes followed by out_size mask bytes
 * (GR_UNKNOWN / GR_EXACT / GR_SUSPECT / GR_INFERRED), and crc32 0. A rescue's device memory is taken for
 * the request and given back, outside hbm_budget.
 * Returns GI_OK, or GI_ERR_ARG (no input, or the server is shutting down). */
#define GI_REQ_RESCUE 8
GI_API int gi_server_submit(gi_server* server, const uint8_t* in, uint64_t in_size, uint32_t flags,
                            uint32_t expected_crc, uint64_t tag);
/* Waits until every submitted request has had its callback. */
GI_API int gi_server_drain(gi_server* server);
GI_API double gi_server_clock(const gi_server* server);
GI_API int gi_server_read_stats(const gi_server* server, gi_server_stats* stats);
/* Drains, stops the server's threads and frees its memory. */
GI_API void gi_server_destroy(gi_server* server);

#ifdef __cplusplus
}
#endif

#endif
