/* gzrescue_gb300.h - recovery of damaged gzip data on the GPU: the gr_* entry points of
 * libgpuinflate.so, with the interface of gzrescue's libgzrescue (interface version 4).
 *
 * The names, argument meanings, return codes and struct layouts are those of gzrescue's
 * gpuinflate/rescue.h:38-107, so that gpuzip's Rust host (src/rescue.rs:193-261) binds these
 * symbols unchanged; the layouts are part of that interface and are kept field for field.
 *
 * What differs is where the work runs: every block header of the file is found and every block
 * decoded on the GPU at once (one decode from each header, landing on the next), the decisions
 * of a pass are made on the host from those results, and the bytes, their certainty, the CRC-32
 * checks, the one-flipped-bit trials and the scoring of lost window bytes are computed on the GPU.
 * The calls take no context: the library keeps one device (GPUZIP_RESCUE_DEVICE, default 0); up to
 * four calls of a process run at once (each on a rescue slot of its own: its stream, the device
 * blocks it keeps for its next call, its host tables), further calls wait for a free slot.
 *
 * The search for the CRs a Windows-to-Unix transfer removed from a raw stream with a known size
 * and CRC (gr_rescue_raw) runs its trial decodes on the GPU, thousands in one launch, and counts
 * the input bytes it decoded as the reference does, so that the budget cuts it at the same trial. */
#ifndef GZRESCUE_GB300_H
#define GZRESCUE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(GI_BUILD) && defined(__GNUC__)
#define GR_API __attribute__((visibility("default")))
#else
#define GR_API
#endif

/* reference: gpuinflate/rescue.h:38 */
#define GR_ABI_VERSION 4

/* Return codes and per-byte certainty. reference: gpuinflate/rescue.h:40-43 (same values) */
enum { GR_OK = 0, GR_ERR_NO_DEFLATE = 1, GR_ERR_ABORTED = 2, GR_ERR_ARG = 3, GR_ERR_MEMORY = 4, GR_ERR_TOO_BIG = 5, GR_ERR_INTERNAL = 6 };
enum { GR_UNKNOWN = 0, GR_EXACT = 1, GR_SUSPECT = 2, GR_INFERRED = 3 };

/* reference: gpuinflate/rescue.h:45-56. A field is read only when `size` covers it. */
typedef struct {
    uint32_t size;         /* sizeof(gr_options) */
    uint8_t fill;          /* written where a byte is unknown */
    uint8_t no_infer;      /* 1: leave the bytes copied from lost data unknown, do not infer them */
    uint8_t cr_lost;       /* CR LF to LF transfer: 0 tell from the data, 1 it happened, 2 never */
    uint8_t crs_expected;  /* raw streams with cr_lost 1: CRs lost, when known (1-8; 255 none; 0 unknown) */
    uint64_t max_output;   /* GR_ERR_TOO_BIG when the output would exceed it; 0: no limit */
    uint64_t cr_budget;    /* input bytes the CR search may decode; 0: 1 GiB */
} gr_options;

/* One piece of the output. reference: gpuinflate/rescue.h:58-66 */
typedef struct {
    uint64_t out_offset, length; /* in the output */
    uint64_t decoded, known;     /* bytes the decode produced, of which not unknown */
    uint64_t in_byte_start, in_byte_end;
    int32_t suspect;             /* 1: a damaged block */
    int32_t status;              /* how its decode ended: 0 ok, 1 invalid data, 3 end of input, 4 stopped */
    uint32_t blocks, symbols;
    const char* why;             /* suspect: how the damage showed; else "" */
} gr_piece;

/* reference: gpuinflate/rescue.h:68-86 */
typedef struct {
    uint64_t input_size, output_size;
    uint64_t exact_bytes, suspect_bytes, unknown_bytes;
    uint32_t headers, pieces, damaged, members;
    int32_t crc_check;     /* 1 ok, 0 mismatch, -1 not checkable */
    int64_t length_off;    /* output length minus the trailer's, every block in step; else 0 */
    int32_t truncated;     /* the file ends inside the stream */
    int32_t header_damaged;
    uint64_t input_end;    /* byte after the last decoded block of the first member */
    uint64_t inferred_bytes;
    int32_t ascii_undone;  /* an LF to CR LF transfer was undone */
    uint32_t cr_restored;  /* CRs a raw stream lost in transfer that were put back */
    uint64_t cr_decoded;   /* input bytes the search for them decoded (counted per decode) */
    int32_t hidden_damage; /* damage of a kind that can keep the decoder in step, with no CRC to vouch */
} gr_stats;

/* Receives the output in order, at most 1 MiB at a time, from the calling thread. Nonzero stops.
 * reference: gpuinflate/rescue.h:87-88 */
typedef int (*gr_sink)(void* user, const uint8_t* data, const uint8_t* mask, size_t len);

typedef struct gr_result gr_result;

/* reference: gpuinflate/rescue.h:92 */
GR_API uint32_t gr_abi_version(void);

/* Recovers the gzip data in in[0..size) into the sink; on GR_OK or GR_ERR_ABORTED *result holds the
 * statistics, the pieces and the notes (free with gr_free). reference: gpuinflate/rescue.h:94-96 */
GR_API int gr_rescue(const uint8_t* in, uint64_t size, const gr_options* opt, gr_sink sink, void* user, gr_result** result);

/* The same for a raw Deflate stream at in[0] (a ZIP entry); expected_size UINT64_MAX when unknown,
 * has_crc: expected_crc holds the original's CRC-32. reference: gpuinflate/rescue.h:98-103 */
GR_API int gr_rescue_raw(const uint8_t* in, uint64_t size, uint64_t expected_size, int has_crc, uint32_t expected_crc,
                         const gr_options* opt, gr_sink sink, void* user, gr_result** result);

/* reference: gpuinflate/rescue.h:104-107 */
GR_API const gr_stats* gr_result_stats(const gr_result* r);
GR_API uint32_t gr_result_pieces(const gr_result* r, const gr_piece** pieces);
GR_API uint32_t gr_result_notes(const gr_result* r, const char* const** notes);
GR_API void gr_free(gr_result* r);

/* Added here, no counterpart in the reference: the number of GPU kernels the last gr_rescue or
 * gr_rescue_raw call of the process launched. */
GR_API uint64_t gr_last_launches(void);

/* Added here, no counterpart in the reference: frees the device blocks the rescue slots keep for
 * their next call. Between calls a slot keeps the blocks its last call used, up to a fifth of the
 * device's memory (all slots together up to half of it): a large file's resolve holds 8 bytes per
 * output byte, which costs tens of milliseconds to allocate and free per call. Slots in use by a
 * call keep theirs. The library's decoder calls this itself when a device allocation fails. */
GR_API void gr_release_cached(void);

/* ---- Added here: the tar walk over the rescued output, on the GPU where it lies.
 * gpuzip's Rust host reads a rescued .tar.gz with its TarReader (src/rescue.rs:374-829) and then
 * applies two rules (src/main.rs:546-558): these give the same outcome for the stream gr_rescue
 * produces, without the output leaving the device. A file's status: 0 intact, 1 suspect (its
 * bytes lie in flagged blocks, or the next header is not where its size says), 2 partial
 * (unknown bytes, or cut short), 3 inferred, 4 unverified (intact, but the stream's CRC fails with
 * nothing to blame, or damage that keeps the decoder in step was seen). */
typedef struct {
    uint64_t intact, unverified, repaired, bytes; /* files; headers mended from the one before; file bytes read */
    uint32_t files, suspect, inferred, partial, skipped;
    uint32_t pad;
} gr_tar_stats;

typedef struct {
    const char* name;
    uint64_t offset, size; /* its data in the output, and the size its header gives */
    int32_t status;
    int32_t pad;
} gr_tar_file;

typedef struct gr_tar gr_tar;

/* gr_rescue, then the tar walk: on GR_OK *tar holds every regular file in archive order with its
 * status, and the regions with no readable header (free with gr_tar_free). */
GR_API int gr_rescue_tar(const uint8_t* in, uint64_t size, const gr_options* opt, gr_sink sink, void* user, gr_result** result,
                         gr_tar** tar);
GR_API const gr_tar_stats* gr_tar_result_stats(const gr_tar* t);
GR_API uint32_t gr_tar_result_files(const gr_tar* t, const gr_tar_file** files);
/* (offset, bytes) pairs */
GR_API uint32_t gr_tar_result_skipped(const gr_tar* t, const uint64_t** pairs);
GR_API void gr_tar_free(gr_tar* t);

#ifdef __cplusplus
}
#endif

#endif
