// gi_server.cu - the request server: continuous batching of independent streams on one GPU.
//
// Three kinds of threads share one lock and one condition variable:
//  - callers of gi_server_submit append requests to `waiting`, in arrival order;
//  - the admitter moves the head of `waiting` into the device arena as soon as the arena has room
//    for its whole input (the HBM budget), copies the input there on a stream of its own, and
//    appends the request to `ready`;
//  - a rescue thread takes the damaged members queued for recovery (GI_REQ_RESCUE), one at a
//    time in arrival order, beside the passes;
//  - each worker owns a decode context (its own stream, pass buffers and pinned output buffer);
//    whenever it is free it takes every ready request that fits its next pass (in order, up to
//    max_batch), runs the batched form over their device copies, gives their arena ranges back
//    and delivers the results.
// Passes of different workers run on the GPU at the same time, each on its context's stream, so a
// request that arrives while a pass is running is decoded beside it as soon as a worker is free,
// not after everything queued before it has finished. The host work of one pass (stitching,
// target lists) overlaps the kernels of another.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#define GI_BUILD
#include "gpuinflate.h"
#include "gi_arena.h"
#include "gi_internal.h"
#include "gzrescue_gb300.h"

namespace {

using clk = std::chrono::steady_clock;

constexpr uint64_t DEFAULT_BUDGET = 120000000000ull;  // bytes of device memory
constexpr uint64_t ARENA_MAX = 64ull << 30;
constexpr uint64_t ARENA_MIN = 64ull << 20;
constexpr uint32_t DEFAULT_PASS_MB = 2048;
constexpr uint32_t MIN_PASS_MB = 64;
constexpr double CTX_BYTES_PER_PASS_BYTE = 12.0;  // a context's device memory per output byte of a pass
constexpr uint64_t PASS_GAP = 1024 + 4096 + 8192;  // what a stream adds to a pass's input besides its bytes
constexpr uint32_t MAX_WORKERS = 16;
// a pass holds requests of one size class: large requests (a decode of tens of milliseconds) in
// passes of their own, so small ones never wait for them inside a pass
constexpr uint64_t LARGE_OUT = 32ull << 20;
constexpr uint32_t MAX_BATCH = 65536;

struct Request {
    uint64_t tag;
    const uint8_t* in;
    uint64_t size;
    uint32_t flags, expected_crc;
    uint64_t out_guess;   // output bytes expected (for packing passes)
    bool alone;           // decoded on its own, from host memory
    int pre_status;       // an error met before decoding (the upload failed), else GI_OK
    uint64_t arena_off;
    double t_submit, t_admit, t_start;
};

// the output a request will probably have: a gzip member's ISIZE when it is possible for Deflate
// (at most 1032 bytes out per byte in), else 4 bytes per input byte
uint64_t guess_out(const uint8_t* in, uint64_t size, uint32_t flags) {
    if ((flags & GI_STREAM_GZIP) && size >= 18) {
        const uint8_t* q = in + size - 4;
        uint64_t isz = q[0] | q[1] << 8 | q[2] << 16 | (uint32_t)q[3] << 24;
        if (isz <= 1032 * size) return isz;
    }
    return 4 * size;
}

}  // namespace

struct gi_server {
    gi_server_config cfg{};
    gi_done done = nullptr;
    void* user = nullptr;
    clk::time_point t0;
    std::vector<gi_ctx*> ctx;
    std::vector<uint8_t*> h_out;  // one pinned output buffer per worker
    uint64_t out_buf = 0;         // bytes of each
    uint64_t pass_out = 0, pass_in = 0;
    uint8_t* d_arena = nullptr;
    cudaStream_t copy_st = nullptr;
    gz::Arena arena;

    std::mutex m;
    std::condition_variable cv;
    std::deque<Request*> waiting, ready, rescue;
    uint64_t outstanding = 0;  // submitted, callback not yet returned
    uint32_t running = 0;      // passes running
    double busy_from = 0;
    bool stop = false;
    gi_server_stats st{};
    std::mutex done_m;  // callbacks never run two at once
    std::thread admitter;
    std::vector<std::thread> workers, rescuers;
    // the rescues' device memory: an allowance carved from the budget, used by estimate
    uint64_t rescue_budget = 0, rescue_used = 0;
    uint32_t rescues_running = 0;

    double now() const { return std::chrono::duration<double>(clk::now() - t0).count(); }
};

namespace {

void admit_loop(gi_server* s) {
    cudaSetDevice(s->cfg.device);
    std::unique_lock<std::mutex> l(s->m);
    for (;;) {
        s->cv.wait(l, [&] {
            return s->stop ||
                   (!s->waiting.empty() && (s->waiting.front()->alone || s->arena.fits(s->waiting.front()->size)));
        });
        if (s->stop) return;
        Request* r = s->waiting.front();
        s->waiting.pop_front();
        if (!r->alone) r->arena_off = s->arena.alloc(r->size);
        s->st.arena_peak = std::max(s->st.arena_peak, s->arena.used());
        l.unlock();
        if (!r->alone) {
            cudaError_t e = cudaMemcpyAsync(s->d_arena + r->arena_off, r->in, r->size, cudaMemcpyHostToDevice, s->copy_st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s->copy_st);
            if (e != cudaSuccess) {
                cudaGetLastError();
                r->pre_status = GI_ERR_GPU;
            }
        }
        l.lock();
        r->t_admit = s->now();
        s->ready.push_back(r);
        s->cv.notify_all();
    }
}

struct VecSink {
    std::vector<uint8_t>* v;
    uint64_t cap;
};

int vec_sink(void* user, const uint8_t* data, size_t len) {
    VecSink* vs = (VecSink*)user;
    if (vs->v->size() + len > vs->cap) return 1;
    vs->v->insert(vs->v->end(), data, data + len);
    return 0;
}

// one request decoded on its own through the segmented path, from host memory
void decode_alone(gi_server* s, int w, Request* r, gi_result& res, std::vector<uint8_t>& buf) {
    gi_ctx* g = s->ctx[w];
    buf.clear();
    // a member's trailer gives its exact size when its ISIZE cannot have wrapped
    uint64_t cap = UINT64_MAX;
    if ((r->flags & GI_STREAM_GZIP) && r->size >= 18 && r->size * 1032 < (1ull << 32)) cap = r->out_guess;
    buf.reserve(std::min<uint64_t>(r->out_guess, 1ull << 32));
    VecSink vs{&buf, cap};
    gi_stats stt{};
    int rc;
    if (r->flags & GI_STREAM_GZIP) {
        uint64_t member = 0;
        rc = gi_inflate_gzip(g, r->in, r->size, vec_sink, &vs, &member, &stt);
        res.in_used = member;
    } else {
        rc = gi_inflate(g, r->in, r->size, 0, vec_sink, &vs, &stt);
        res.in_used = stt.in_used;
    }
    if (rc == GI_ERR_ABORTED) rc = GI_ERR_DATA;  // longer than its trailer says
    res.crc32 = rc == GI_OK ? gi_last_crc32(g) : 0;
    if (rc == GI_OK && (r->flags & GI_STREAM_CRC) && res.crc32 != r->expected_crc) rc = GI_ERR_DATA;
    res.status = rc;
    res.out_size = rc == GI_OK ? stt.out_size : 0;
}

// decodes the pass b on worker w and delivers every result
void run_pass(gi_server* s, int w, std::vector<Request*>& b) {
    const uint32_t n = (uint32_t)b.size();
    std::vector<gi_result> res(n);
    std::vector<const uint8_t*> data(n, nullptr);
    std::vector<std::vector<uint8_t>> own;  // outputs of requests decoded on their own
    for (uint32_t i = 0; i < n; i++) {
        res[i] = gi_result{b[i]->tag, GI_OK, 0, 0, 0, b[i]->t_submit, b[i]->t_admit, b[i]->t_start, 0, n, (uint32_t)w};
    }
    std::vector<uint32_t> redo;  // requests whose output did not fit the pass
    if (n == 1 && b[0]->pre_status != GI_OK) {
        res[0].status = b[0]->pre_status;
    } else if (n == 1 && b[0]->alone) {
        redo.push_back(0);
    } else {
        std::vector<gi_stream> items(n);
        std::vector<const uint8_t*> dev(n);
        for (uint32_t i = 0; i < n; i++) {
            items[i] = gi_stream{b[i]->in, b[i]->size, b[i]->flags & (GI_STREAM_GZIP | GI_STREAM_CRC), b[i]->expected_crc,
                                 0, 0, 0, 0, GI_OK};
            dev[i] = s->d_arena + b[i]->arena_off;
        }
        gi_stats stt{};
        int rc = gi_batch_resident(s->ctx[w], items.data(), dev.data(), n, s->h_out[w], s->out_buf, &stt);
        {
            // the pass has finished with its inputs
            std::lock_guard<std::mutex> l(s->m);
            for (uint32_t i = 0; i < n; i++) s->arena.release(b[i]->arena_off, b[i]->size);
            s->cv.notify_all();
        }
        for (uint32_t i = 0; i < n; i++) {
            gi_stream& it = items[i];
            res[i].status = rc != GI_OK ? rc : it.status;
            if (res[i].status == GI_ERR_SPACE) {
                redo.push_back(i);
                continue;
            }
            res[i].crc32 = it.crc32;
            res[i].in_used = it.in_used;
            if (res[i].status == GI_OK) {
                res[i].out_size = it.out_size;
                data[i] = s->h_out[w] + it.out_offset;
            }
        }
    }
    own.resize(redo.size());
    for (size_t k = 0; k < redo.size(); k++) {
        uint32_t i = redo[k];
        decode_alone(s, w, b[i], res[i], own[k]);
        if (res[i].status == GI_OK) data[i] = own[k].data();
    }
    uint64_t out_bytes = 0, failed = 0;
    {
        std::lock_guard<std::mutex> l(s->done_m);
        for (uint32_t i = 0; i < n; i++) {
            res[i].t_done = s->now();
            s->done(s->user, &res[i], res[i].status == GI_OK ? data[i] : nullptr);
            out_bytes += res[i].out_size;
            failed += res[i].status != GI_OK;
        }
    }
    std::lock_guard<std::mutex> l(s->m);
    s->st.alone += redo.size();
    s->st.out_bytes += out_bytes;
    s->st.failed += failed;
    s->st.completed += n;
}

void work_loop(gi_server* s, int w) {
    cudaSetDevice(s->cfg.device);
    std::unique_lock<std::mutex> l(s->m);
    for (;;) {
        s->cv.wait(l, [&] { return s->stop || !s->ready.empty(); });
        if (s->ready.empty()) return;
        // the next pass: the ready requests, in order, while they fit it
        std::vector<Request*> b;
        Request* f = s->ready.front();
        if (f->alone || f->pre_status != GI_OK) {
            b.push_back(f);
            s->ready.pop_front();
        } else {
            // the ready requests of the first one's size class, in order, while they fit the pass
            const bool large = f->out_guess >= LARGE_OUT;
            uint64_t in_b = 0, out_b = 0;
            for (auto it = s->ready.begin(); it != s->ready.end() && b.size() < s->cfg.max_batch;) {
                Request* r = *it;
                if (r->alone || r->pre_status != GI_OK) break;
                if ((r->out_guess >= LARGE_OUT) != large) {
                    ++it;
                    continue;
                }
                if (!b.empty() && (in_b + r->size + PASS_GAP > s->pass_in || out_b + r->out_guess + 16 > s->pass_out))
                    break;
                b.push_back(r);
                it = s->ready.erase(it);
                in_b += r->size + PASS_GAP;
                out_b += r->out_guess + 16;
            }
        }
        const double t = s->now();
        if (s->running++ == 0)
            s->busy_from = t;
        else
            s->st.overlapped++;
        if (b[0]->pre_status == GI_OK) s->st.passes++;
        for (Request* r : b) r->t_start = t;
        l.unlock();
        run_pass(s, w, b);
        l.lock();
        if (--s->running == 0) s->st.busy_s += s->now() - s->busy_from;
        s->outstanding -= b.size();
        for (Request* r : b) delete r;
        s->cv.notify_all();
    }
}

// a rescue's GR_* code as a request status: input with nothing to recover is bad data; running
// out of memory or an internal failure is the GPU's side (retry later, or elsewhere); an output
// past its limit is a lack of space
int rescue_status(int gr) {
    switch (gr) {
        case GR_OK: return GI_OK;
        case GR_ERR_MEMORY:
        case GR_ERR_INTERNAL: return GI_ERR_GPU;
        case GR_ERR_TOO_BIG: return GI_ERR_SPACE;
        case GR_ERR_ARG: return GI_ERR_ARG;
        default: return GI_ERR_DATA;
    }
}

// A rescue's device peak, estimated: about 24 bytes per output byte (the input, the links'
// symbols, the pass's entries, bytes, certainty, output and mask) for its output guess.
uint64_t rescue_need(const Request* r) { return 24 * std::max<uint64_t>(r->out_guess, r->size) + 2 * r->size; }

// The rescue requests, in arrival order, on rescue_workers loops (their GPU work runs beside the
// passes, each on its own stream): the next one starts when its estimated device peak fits what
// the rescues in progress leave of the allowance (or when none is in progress).
void rescue_loop(gi_server* s) {
    cudaSetDevice(s->cfg.device);
    std::unique_lock<std::mutex> l(s->m);
    for (;;) {
        s->cv.wait(l, [&] {
            return s->stop || (!s->rescue.empty() && (s->rescues_running == 0 ||
                                                       s->rescue_used + rescue_need(s->rescue.front()) <= s->rescue_budget));
        });
        if (s->rescue.empty()) return;
        Request* r = s->rescue.front();
        s->rescue.pop_front();
        const uint64_t need = rescue_need(r);
        s->rescue_used += need;
        s->rescues_running++;
        r->t_admit = r->t_start = s->now();
        const uint64_t keep = s->rescue_budget / (4 * std::max<uint32_t>(1, s->cfg.rescue_workers));
        l.unlock();
        std::vector<uint8_t> buf;
        uint64_t out_size = 0;
        int rc = gz::rescue_for_server(s->cfg.device, r->in, r->size, buf, out_size, keep);
        gi_result res{r->tag, rescue_status(rc), 0, rc == 0 ? out_size : 0, r->size, r->t_submit, r->t_admit,
                      r->t_start, 0, 1, s->cfg.workers};
        {
            std::lock_guard<std::mutex> dl(s->done_m);
            res.t_done = s->now();
            s->done(s->user, &res, res.status == GI_OK ? buf.data() : nullptr);
        }
        l.lock();
        s->rescue_used -= need;
        s->rescues_running--;
        s->st.completed++;
        s->st.failed += res.status != GI_OK;
        s->st.out_bytes += res.out_size;
        s->outstanding--;
        delete r;
        s->cv.notify_all();
    }
}

void teardown(gi_server* s) {
    {
        std::lock_guard<std::mutex> l(s->m);
        s->stop = true;
        s->cv.notify_all();
    }
    if (s->admitter.joinable()) s->admitter.join();
    for (auto& t : s->rescuers)
        if (t.joinable()) t.join();
    for (auto& t : s->workers)
        if (t.joinable()) t.join();
    cudaSetDevice(s->cfg.device);
    for (gi_ctx* g : s->ctx) gi_destroy(g);
    for (uint8_t* p : s->h_out) cudaFreeHost(p);
    if (s->d_arena) cudaFree(s->d_arena);
    if (s->copy_st) cudaStreamDestroy(s->copy_st);
    delete s;
}

}  // namespace

extern "C" {

GI_API int gi_server_create(const gi_server_config* cfg, gi_done done, void* user, gi_server** out, char* err,
                            size_t err_len) {
    auto fail = [&](int code, const std::string& m) {
        if (err && err_len) snprintf(err, err_len, "%s", m.c_str());
        return code;
    };
    if (!out) return fail(GI_ERR_ARG, "no server pointer");
    *out = nullptr;
    if (!done) return fail(GI_ERR_ARG, "no callback");
    gi_server_config c{sizeof(gi_server_config), 0, 0, 0, 0, 0, 0, 0};
    if (cfg) {
        if (cfg->size < sizeof(gi_server_config)) return fail(GI_ERR_ARG, "gi_server_config too small");
        c = *cfg;
    }
    if (!c.workers) c.workers = 3;
    if (c.workers > MAX_WORKERS) return fail(GI_ERR_ARG, "too many workers (at most 16)");
    if (!c.max_batch) c.max_batch = 4096;
    c.max_batch = std::min(c.max_batch, MAX_BATCH);
    if (!c.hbm_budget) c.hbm_budget = DEFAULT_BUDGET;
    if (!c.rescue_workers) c.rescue_workers = 3;
    if (c.rescue_workers > 4) return fail(GI_ERR_ARG, "too many rescue workers (at most 4)");
    const uint64_t rescue_budget = std::clamp<uint64_t>(c.hbm_budget / 6, 4ull << 30, 24ull << 30);
    if (rescue_budget >= c.hbm_budget) return fail(GI_ERR_ARG, "HBM budget too small for the rescues' allowance");
    if (cudaSetDevice(c.device) != cudaSuccess || cudaFree(nullptr) != cudaSuccess) {
        cudaGetLastError();
        return fail(GI_ERR_GPU, "no usable GPU");
    }
    uint32_t pass_mb = c.pass_out_mb;
    if (!pass_mb) {
        double fit = 0.6 * (double)(c.hbm_budget - rescue_budget) / (c.workers * CTX_BYTES_PER_PASS_BYTE) / (1 << 20);
        pass_mb = (uint32_t)std::min<double>(DEFAULT_PASS_MB, fit);
    }
    if (pass_mb < MIN_PASS_MB) return fail(GI_ERR_ARG, "HBM budget too small for the workers' pass buffers");

    gi_server* s = new gi_server;
    s->cfg = c;
    s->done = done;
    s->user = user;
    s->t0 = clk::now();
    size_t free0 = 0, free1 = 0, total = 0;
    gr_release_cached();  // device blocks kept by rescues before the server: its budget is its own
    cudaMemGetInfo(&free0, &total);
    for (uint32_t w = 0; w < c.workers; w++) {
        gi_config gc{sizeof(gi_config), c.device, pass_mb, 0};
        gi_ctx* g = nullptr;
        char e[512] = {0};
        int r = gi_create(&gc, &g, e, sizeof e);
        if (r != GI_OK) {
            teardown(s);
            return fail(r, std::string("decode context: ") + e);
        }
        s->ctx.push_back(g);
    }
    cudaMemGetInfo(&free1, &total);
    const uint64_t ctx_bytes = free0 > free1 ? free0 - free1 : 0;
    uint64_t arena = c.arena_bytes;
    const uint64_t room = c.hbm_budget - rescue_budget;  // the passes' buffers and the arena
    if (!arena) arena = room > ctx_bytes ? std::min(room - ctx_bytes, ARENA_MAX) : 0;
    if (arena < ARENA_MIN || ctx_bytes + arena > room) {
        teardown(s);
        return fail(GI_ERR_ARG, "HBM budget too small: the pass buffers take " + std::to_string(ctx_bytes >> 20) +
                                    " MiB and the arena needs at least 64 MiB");
    }
    s->pass_out = gi_pass_capacity(s->ctx[0], &s->pass_in);
    s->out_buf = s->pass_out + (uint64_t)c.max_batch * 16 + (1 << 20);
    bool ok = cudaMalloc(&s->d_arena, arena) == cudaSuccess &&
              cudaStreamCreateWithFlags(&s->copy_st, cudaStreamNonBlocking) == cudaSuccess;
    for (uint32_t w = 0; ok && w < c.workers; w++) {
        void* p = nullptr;
        ok = cudaMallocHost(&p, s->out_buf) == cudaSuccess;
        if (ok) s->h_out.push_back((uint8_t*)p);
    }
    if (!ok) {
        cudaGetLastError();
        teardown(s);
        return fail(GI_ERR_GPU, "out of memory for the arena or the output buffers");
    }
    s->arena.reset(arena, 4096);
    s->st.size = sizeof(gi_server_stats);
    s->st.workers = c.workers;
    s->st.device_bytes = ctx_bytes + arena;
    s->st.arena_bytes = arena;
    s->rescue_budget = rescue_budget;
    s->admitter = std::thread(admit_loop, s);
    for (uint32_t w = 0; w < c.rescue_workers; w++) s->rescuers.emplace_back(rescue_loop, s);
    for (uint32_t w = 0; w < c.workers; w++) s->workers.emplace_back(work_loop, s, (int)w);
    *out = s;
    return GI_OK;
}

GI_API int gi_server_submit(gi_server* s, const uint8_t* in, uint64_t in_size, uint32_t flags, uint32_t expected_crc,
                            uint64_t tag) {
    if (!s || !in || !in_size) return GI_ERR_ARG;
    Request* r = new Request{tag, in, in_size, flags, expected_crc, guess_out(in, in_size, flags), false, GI_OK,
                             gz::Arena::NONE, 0, 0, 0};
    std::lock_guard<std::mutex> l(s->m);
    if (s->stop) {
        delete r;
        return GI_ERR_ARG;
    }
    r->alone = r->out_guess + 16 > s->pass_out || in_size + PASS_GAP > s->pass_in || in_size > s->arena.capacity();
    r->t_submit = s->now();
    if (flags & GI_REQ_RESCUE) s->rescue.push_back(r);
    else s->waiting.push_back(r);
    s->outstanding++;
    s->st.submitted++;
    s->st.in_bytes += in_size;
    s->cv.notify_all();
    return GI_OK;
}

GI_API int gi_server_drain(gi_server* s) {
    if (!s) return GI_ERR_ARG;
    std::unique_lock<std::mutex> l(s->m);
    s->cv.wait(l, [&] { return s->outstanding == 0; });
    return GI_OK;
}

GI_API double gi_server_clock(const gi_server* s) { return s ? s->now() : 0.0; }

GI_API int gi_server_read_stats(const gi_server* cs, gi_server_stats* out) {
    if (!cs || !out || out->size < sizeof(gi_server_stats)) return GI_ERR_ARG;
    gi_server* s = const_cast<gi_server*>(cs);
    std::lock_guard<std::mutex> l(s->m);
    *out = s->st;
    out->arena_peak = std::max(out->arena_peak, s->arena.used());
    if (s->running) out->busy_s += s->now() - s->busy_from;
    return GI_OK;
}

GI_API void gi_server_destroy(gi_server* s) {
    if (!s) return;
    gi_server_drain(s);
    teardown(s);
}

}  // extern "C"
