// gi_noalloc.cu - CRC-32 of a buffer already in GPU memory, for callers that cannot allocate.
//
// Some callers of this library cannot call cudaMalloc: a serving process that reserved all GPU
// memory for its own pool at start-up (an allocation later would fail, or synchronize the whole
// device and stall the streams of other requests), or a host framework that hands out device
// memory only through its own allocator. gi_crc32_device_noalloc gives them the GPU CRC-32 the
// gzip path checks trailers with, using no memory it allocates: its scratch (one CRC per 4 KiB
// tile of the input and the tree that merges them) is the file-scope array below, which every
// GPU that loads this library holds until the process exits (about 1 MiB).
//
// The first call on a device sets the entry point up there, with that device current: it looks up
// the array's address as the GPU sees it and loads the CRC kernels. Under CUDA's lazy module
// loading (the default) that set-up is when the driver places the array and the kernels' code and
// constants in device memory, so the first call on each device, with size 0 if there is nothing
// to check yet, must come before the caller reserves the rest of the device's memory, and before
// any stream capture on that device; later calls take no device memory. Every call on a device
// shares the one array: calls that overlap on the GPU (different host threads, or different
// streams without ordering between them) race on it and corrupt each other's result. Nothing in
// the array needs to start at zero: every word a call reads was written earlier in the same call.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#define GI_BUILD
#include "gpuinflate.h"
#include "gi_common.cuh"

namespace {

// largest input: 1 GiB = 262,144 tiles of 4 KiB; the merge tree adds 256 + 1 words, the result 1
constexpr uint64_t NOALLOC_MAX_BYTES = 1ull << 30;
constexpr uint64_t NOALLOC_WORDS = (NOALLOC_MAX_BYTES / 4096) + 1024;

static __device__ __align__(256) uint32_t g_crc_scratch[NOALLOC_WORDS];

constexpr int MAX_DEVICES = 64;
std::mutex g_mutex;
uint32_t* g_scratch_addr[MAX_DEVICES] = {};

void say(char* err, size_t err_len, const char* msg) {
    if (err && err_len) snprintf(err, err_len, "%s", msg);
}

}  // namespace

extern "C" GI_API int gi_crc32_device_noalloc(int device, const void* d_data, uint64_t size, uint32_t* d_crc,
                                              void* stream, char* err, size_t err_len) {
    if ((!d_data && size) || !d_crc) {
        say(err, err_len, "no buffer");
        return GI_ERR_ARG;
    }
    if (size > NOALLOC_MAX_BYTES) {
        say(err, err_len, "input larger than 1 GiB (the fixed scratch of this entry point)");
        return GI_ERR_ARG;
    }
    if (((uintptr_t)d_data & 15) != 0) {
        say(err, err_len, "input not 16-byte aligned");
        return GI_ERR_ARG;
    }
    if (device < 0 || device >= MAX_DEVICES) {
        say(err, err_len, "device ordinal out of range");
        return GI_ERR_ARG;
    }
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) {
        cudaGetLastError();
        say(err, err_len, "no usable GPU");
        return GI_ERR_GPU;
    }
    cudaError_t e = cudaSetDevice(device);
    uint32_t* scratch = nullptr;
    if (e == cudaSuccess) {
        std::lock_guard<std::mutex> lock(g_mutex);
        if (!g_scratch_addr[device]) {
            // once per device, with the device current: the array's address as the GPU sees it,
            // and the CRC kernels loaded
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_crc_scratch);
            if (e == cudaSuccess) e = (cudaError_t)gz::crc_prepare();
            if (e == cudaSuccess) g_scratch_addr[device] = (uint32_t*)p;
        }
        scratch = g_scratch_addr[device];
    }
    bool too_big = false;
    if (e == cudaSuccess) {
        too_big = gz::launch_crc((const uint8_t*)d_data, size, scratch, NOALLOC_WORDS, d_crc, stream) < 0;
        e = cudaGetLastError();
    }
    cudaSetDevice(prev);
    if (too_big) {
        say(err, err_len, "input larger than the fixed scratch of this entry point");
        return GI_ERR_ARG;
    }
    if (e != cudaSuccess) {
        say(err, err_len, cudaGetErrorString(e));
        return GI_ERR_GPU;
    }
    return GI_OK;
}
