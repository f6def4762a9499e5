// gi_internal.h - entry points of the engine that other files of the library use (not exported).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "gpuinflate.h"

// gi_inflate_batch over inputs already in device memory: dev_in[i] holds a copy of the whole of
// streams[i].in (streams[i].in stays the host copy the gzip header and trailer are read from).
int gi_batch_resident(gi_ctx* g, gi_stream* streams, const uint8_t* const* dev_in, uint32_t n, uint8_t* out,
                      uint64_t out_cap, gi_stats* stats);

// output bytes one pass of the context holds (and, in *in_cap, its compressed input bytes)
uint64_t gi_pass_capacity(const gi_ctx* g, uint64_t* in_cap);

// for the entry points of other files on a context: its device and stream (a cudaStream_t), and
// its last error (cleared, set; refuse sets it and returns code)
int gi_ctx_device(const gi_ctx* g);
void* gi_ctx_stream(const gi_ctx* g);
void gi_ctx_clear_error(gi_ctx* g);
void gi_ctx_set_error(gi_ctx* g, const std::string& why);
int gi_ctx_refuse(gi_ctx* g, int code, const char* why);

namespace gz {
// The request server's rescue (gi_rescue.cu): the gzip member in[0..size) rescued on `device` with
// the default options; `out` gets the output bytes then as many mask bytes, out_size the output's
// length; the rescue's slot keeps at most keep_bytes of device blocks for its next rescue. Up to
// four run at once (one per rescue slot). Returns a GR_* code.
int rescue_for_server(int device, const uint8_t* in, uint64_t size, std::vector<uint8_t>& out, uint64_t& out_size,
                      uint64_t keep_bytes);
}  // namespace gz
