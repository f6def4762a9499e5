// gi_internal.h - entry points of the engine that other files of the library use (not exported).
#pragma once

#include <cstdint>
#include <vector>

#include "gpuinflate.h"

// gi_inflate_batch over inputs already in device memory: dev_in[i] holds a copy of the whole of
// streams[i].in (streams[i].in stays the host copy the gzip header and trailer are read from).
int gi_batch_resident(gi_ctx* g, gi_stream* streams, const uint8_t* const* dev_in, uint32_t n, uint8_t* out,
                      uint64_t out_cap, gi_stats* stats);

// output bytes one pass of the context holds (and, in *in_cap, its compressed input bytes)
uint64_t gi_pass_capacity(const gi_ctx* g, uint64_t* in_cap);

namespace gz {
// The request server's rescue (gi_rescue.cu): the gzip member in[0..size) rescued on `device` with
// the default options; `out` gets the output bytes then as many mask bytes, out_size the output's
// length. Returns a GR_* code.
int rescue_for_server(int device, const uint8_t* in, uint64_t size, std::vector<uint8_t>& out, uint64_t& out_size);
}  // namespace gz
