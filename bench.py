"""Benchmark of the Deflate decode path on GB300: decompressed GB/s of one 4 GiB gzip member.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--nseg S]

Workload (seeded, synthetic): one gzip member of 4096 segments of 1 MiB (4 GiB of output, the
trailer's ISIZE wraps to 0), each segment log text / random bytes / repeated patterns with 1%
flips / uint32 counters (p = 0.5/0.2/0.15/0.15), each at a zlib level drawn from {1, 6, 9}, all
in ONE Deflate stream written by zlib's deflate with the level changed by deflateParams (no sync
flush, no empty stored blocks; gpuzip_gb300/workloads.py:mixed_member).

One step = one full decode of the stream. `value`: the compressed stream already in GPU memory,
the output written to GPU memory (gi_inflate_device), timed with CUDA events around each call
(the calls are synchronous). `e2e`: the same stream through the public gzip entry point from
pinned host memory (gi_inflate_gzip: header parse, H2D, decode, CRC-32/ISIZE checked on the GPU,
D2H of every output byte into the library's pinned buffers); the output goes to no sink, as in
the reference's own timing (gpuinflate/gi_test.cpp:182-190). Every step's CRC-32 and size are
checked against the generator's.

`--impl reference`: the reference's CPU decoders for this path on the host's cores, on a bounded
prefix of the same stream: the oracle port of its sequential gi::Decoder (oracle/gi_oracle.c, one
thread), the port of its multi-threaded speculative decoder (oracle/gi_oracle_parallel.c, every
host thread), and system zlib standing in for the Rust host's CPU inflate; the fastest is timed.
Under torchrun (N > 1) every rank decodes its own copy (replicas; the path has no exchange).
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time
import zlib

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "decompressed GB/s, one 4 GiB gzip member (mixed content), 1 GB300"
METRIC_TEXT = "decompressed GB/s, one 64 MiB gzip member (log text), 1 GB300"


def metric_of(args):
    return METRIC_TEXT if args.workload == "text" else METRIC
CACHE = os.environ.get("GI_BENCH_CACHE", "/tmp/gpuzip_gb300_bench")


def workload(seed, nseg):
    """(member bytes, info) of the mixed workload, cached on local disk between runs."""
    from gpuzip_gb300 import workloads as W

    os.makedirs(CACHE, exist_ok=True)
    path = os.path.join(CACHE, f"mixed_params_s{seed}_n{nseg}.gz")
    meta = path + ".json"
    if os.path.exists(path) and os.path.exists(meta):
        with open(meta) as f:
            info = json.load(f)
        with open(path, "rb") as f:
            return f.read(), info
    t = time.time()
    member, info = W.mixed_member(seed=seed, nseg=nseg)
    info = {"crc": info["crc"], "size": info["size"], "deflate_size": info["deflate_size"],
            "gen_seconds": time.time() - t}
    with open(path + ".tmp", "wb") as f:
        f.write(member)
    os.replace(path + ".tmp", path)
    with open(meta, "w") as f:
        json.dump(info, f)
    return member, info


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, uuid=None):
        self.rows = []
        self.proc = None
        self.uuid = uuid

    def __enter__(self):
        cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200"]
        if self.uuid:
            cmd.insert(1, f"--id={self.uuid}")
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.reader = threading.Thread(target=self._read, daemon=True)
            self.reader.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=5)
            self.reader.join(timeout=5)

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for name, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def traffic_per_launch(kernel):
    """dram bytes per launch of `kernel` from the committed ncu summary (scaled to one full
    launch of this workload), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            t = json.load(f)
        return t.get(kernel, {}).get("bytes_per_launch")
    except (OSError, ValueError):
        return None


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def cpu_candidates(body, sample, ratio, threads):
    """Seconds each CPU path takes for the first `sample` bytes of output of the raw stream `body`
    (one run each, after one untimed run): the oracle port of the reference's sequential decoder
    (one thread); the port of the reference's multi-threaded speculative decoder on `threads`
    threads (256 KiB chunks, the reference's chunk-size argument; block starts searched in the
    input the sample needs); and the system's zlib (one thread: a single stream is sequential for
    it), standing in for the Rust host's CPU inflate."""
    import zlib

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    lib = oracle.lib()
    out = ctypes.create_string_buffer(sample + 1)
    n, used = ctypes.c_uint64(0), ctypes.c_uint64(0)
    scan = min(len(body), int(sample / max(ratio, 1.0) * 1.25) + (1 << 20))

    def sequential():
        rc = lib.oracle_inflate(body, len(body), out, sample, ctypes.byref(n), ctypes.byref(used))
        if rc not in (0, 7):
            raise RuntimeError(f"oracle failed on the workload: {rc}")

    def parallel():
        secs = (ctypes.c_double * 3)()
        rc = lib.oracle_inflate_parallel(body, len(body), scan, 256 << 10, out, sample, ctypes.byref(n), threads, secs)
        if rc != 0 or n.value != sample:
            raise RuntimeError(f"parallel CPU inflate failed on the workload: {rc}, {n.value} bytes")

    def system_zlib():
        d = zlib.decompressobj(-15)
        if len(d.decompress(body, sample)) != sample:
            raise RuntimeError("zlib did not produce the sample")

    res = {}
    for name, fn, cores in (("sequential port", sequential, 1), ("speculative port", parallel, threads),
                            ("system zlib", system_zlib, 1)):
        fn()
        t = time.perf_counter()
        fn()
        res[name] = {"seconds": time.perf_counter() - t, "cores": cores, "fn": fn}
    return res


def cpu_sample(args, info):
    """Output bytes the CPU baselines decode: the first cpu_sample_mb MiB, or the whole stream."""
    return min(args.cpu_sample_mb << 20, info["size"])


def cpu_line(res, sample, extra=""):
    """The cpu_baseline object: the fastest of the candidates, with all of them listed."""
    best = min(res, key=lambda k: res[k]["seconds"])
    gbs = {k: round(sample / v["seconds"] / 1e9, 4) for k, v in res.items()}
    what = f"first {sample >> 20} MiB of output" if sample % (1 << 20) == 0 else f"all {sample} bytes of output"
    return {"value": gbs[best], "unit": "GB/s", "cores": res[best]["cores"], "kind": "port",
            "sample": f"{what} of the same stream{extra}; the fastest of: the oracle port of the "
                      "reference's sequential gi::Decoder (1 thread), the port of its multi-threaded speculative CPU "
                      f"decoder (cpu_speculative, {os.cpu_count()} threads), system zlib (1 thread); this one: {best}",
            "candidates_gbs": gbs, "best": best}


def run_reference(args, member, info, ws, rank):
    if rank != 0:
        return
    body = member[10:10 + info["deflate_size"]]
    sample = cpu_sample(args, info)
    threads = os.cpu_count() or 1
    res = cpu_candidates(body, sample, info["size"] / info["deflate_size"], threads)
    best = min(res, key=lambda k: res[k]["seconds"])
    fn = res[best]["fn"]
    for _ in range(args.warmup):
        fn()
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        fn()
        times.append(time.perf_counter() - t)
    tot = sum(times)
    value = args.steps * sample / tot / 1e9
    cpu = cpu_line(res, sample)
    cpu["value"] = round(value, 4)
    line = {
        "impl": "reference", "metric": metric_of(args), "value": round(value, 4), "unit": "GB/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(tot / args.steps * 1e3, 2),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": config_of(args, info), "cpu_baseline": cpu,
        "e2e": {"value": round(value, 4), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def many_workload(seed, n, total):
    """The many-streams workload (cached on local disk between runs)."""
    import pickle

    from gpuzip_gb300 import workloads as W

    os.makedirs(CACHE, exist_ok=True)
    path = os.path.join(CACHE, f"many_s{seed}_n{n}_t{int(total)}.pkl")
    if os.path.exists(path):
        with open(path, "rb") as f:
            return pickle.load(f)
    streams = W.many_streams(seed=seed, n=n, total=total)
    with open(path + ".tmp", "wb") as f:
        pickle.dump(streams, f, protocol=pickle.HIGHEST_PROTOCOL)
    os.replace(path + ".tmp", path)
    return streams


def run_batch(args, ws, rank, local):
    """Many streams of uneven sizes: one library call per stream (the reference's launch model)
    against one gi_inflate_batch call for all of them."""
    import torch

    from gpuzip_gb300 import gpuinflate, shard

    torch.cuda.set_device(local)
    streams = many_workload(args.seed if args.seed != 2 else 3, args.nstreams, args.batch_total)
    job_out = sum(x["size"] for x in streams)  # the whole job, all ranks
    n_all = len(streams)
    if ws > 1:  # replicas sharing nothing: each rank decodes its share of the streams
        import torch.distributed as dist

        dist.init_process_group("nccl")
        streams = [streams[i] for i in shard.shard_streams([x["size"] for x in streams], ws)[rank]]
    total_out = sum(x["size"] for x in streams)
    total_in = sum(len(x["data"]) for x in streams)
    g = gpuinflate.Gpu(local, segment_out_mb=args.seg_out_mb)
    lib = g.lib
    n = len(streams)
    # every stream in one pinned host buffer (pageable inputs are staged by CUDA at host
    # memcpy speed, which would time the host's memory, not the decode)
    import numpy as np

    offs, pos = [], 0
    for x in streams:
        offs.append(pos)
        pos += (len(x["data"]) + 15) // 16 * 16
    host = torch.empty(max(pos, 1), dtype=torch.uint8).pin_memory()
    hv = host.numpy()
    for x, o in zip(streams, offs):
        hv[o:o + len(x["data"])] = np.frombuffer(x["data"], dtype=np.uint8)
    base = host.data_ptr()
    arr = (gpuinflate.Stream * n)()
    for i, x in enumerate(streams):
        arr[i].in_ = ctypes.c_void_p(base + offs[i])
        arr[i].in_size = len(x["data"])
        arr[i].flags = (gpuinflate.GI_STREAM_GZIP if x["gzip"] else gpuinflate.GI_STREAM_CRC) | gpuinflate.GI_STREAM_MAPPED
        arr[i].expected_crc = x["crc"]
    out_cap = total_out + 16 * n + (64 << 20)
    out = torch.empty(out_cap, dtype=torch.uint8).pin_memory()
    stats = gpuinflate.Stats()
    # the gzip members as one batch; the raw entries as one ZIP archive (both in pinned memory)
    from gpuzip_gb300 import workloads as W

    mem = [i for i, x in enumerate(streams) if x["gzip"]]
    ent = [i for i, x in enumerate(streams) if not x["gzip"]]
    marr = (gpuinflate.Stream * max(1, len(mem)))()
    for k, i in enumerate(mem):
        ctypes.memmove(ctypes.addressof(marr[k]), ctypes.addressof(arr[i]), ctypes.sizeof(gpuinflate.Stream))
    zblob = W.zip_archive([(f"entry{i:05d}.bin".encode(), streams[i]["data"], streams[i]["crc"], streams[i]["size"])
                           for i in ent])
    zpin = torch.empty(max(1, len(zblob)), dtype=torch.uint8).pin_memory()
    zpin.numpy()[:len(zblob)] = np.frombuffer(zblob, dtype=np.uint8)
    zptr = ctypes.cast(zpin.data_ptr(), ctypes.c_char_p)
    ent_out = sum(streams[i]["size"] for i in ent)
    zstats = gpuinflate.Stats()

    def batched():
        rc = lib.gi_inflate_batch(g.ctx, marr, len(mem), ctypes.c_void_p(out.data_ptr()), out_cap, ctypes.byref(stats))
        bad = [k for k, i in enumerate(mem) if marr[k].status != 0 or marr[k].out_size != streams[i]["size"]]
        if rc != 0 or bad:
            raise RuntimeError(f"batched decode failed: rc {rc}, {len(bad)} members wrong, e.g. {bad[:3]}")
        rc = lib.gi_inflate_zip(g.ctx, zptr, len(zblob), gpuinflate.ENTRY_SINK(), None, ctypes.byref(zstats))
        if rc != 0 or zstats.out_size != ent_out:  # every entry decoded and checked against its CRC-32
            raise RuntimeError(f"ZIP decode failed: rc {rc}, {zstats.out_size} of {ent_out} bytes")

    msize = ctypes.c_uint64(0)

    def plain():
        times = []
        for i, x in enumerate(streams):
            t = time.perf_counter()
            ptr = ctypes.cast(base + offs[i], ctypes.c_char_p)
            if x["gzip"]:
                rc = lib.gi_inflate_gzip(g.ctx, ptr, len(x["data"]), gpuinflate.SINK(), None, ctypes.byref(msize),
                                         ctypes.byref(stats))
            else:
                rc = lib.gi_inflate(g.ctx, ptr, len(x["data"]), 0, gpuinflate.SINK(), None, ctypes.byref(stats))
                if rc == 0 and lib.gi_last_crc32(g.ctx) != x["crc"]:
                    rc = -1
            times.append(time.perf_counter() - t)
            if rc != 0:
                raise RuntimeError(f"plain decode of stream {i} failed: {rc}")
        return times

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        batched()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        batched()
    barrier()
    tb = shard.max_over_ranks((time.perf_counter() - t0) / args.steps, device="cuda")
    prof = g.last_profile().as_dict()
    passes = stats.segments + zstats.segments
    plain()  # warm
    barrier()
    t0 = time.perf_counter()
    ptimes = plain()
    barrier()
    tp = shard.max_over_ranks(time.perf_counter() - t0, device="cuda")
    q = sorted(ptimes)
    pct = lambda p: q[min(len(q) - 1, int(p * len(q)))] * 1e3
    if rank != 0:
        g.close()
        return
    cpu = None
    if not args.no_cpu:  # system zlib over the same streams, one stream per thread on every host thread
        import concurrent.futures
        import zlib

        def cpu_one(x):
            return len(zlib.decompressobj(31 if x["gzip"] else -15).decompress(x["data"]))

        nth = os.cpu_count() or 1
        with concurrent.futures.ThreadPoolExecutor(nth) as ex:
            list(ex.map(cpu_one, streams[-64:]))  # warm
            t0 = time.perf_counter()
            cpu_out = sum(ex.map(cpu_one, sorted(streams, key=lambda x: -x["size"])))
            tc = time.perf_counter() - t0
        cpu = {"value": round(cpu_out / tc / 1e9, 3), "unit": "GB/s", "cores": nth, "kind": "port",
               "sample": f"every stream of this rank's workload ({cpu_out} bytes) through system zlib, one stream per "
                         f"thread on {nth} threads, largest first (standing in for the Rust host's CPU inflate of "
                         "members and ZIP entries)"}
    line = {
        "metric": f"decompressed GB/s, {n_all} streams of uneven sizes (gzip members and the entries of a ZIP archive), "
                  "batched form",
        "value": round(job_out / tb / 1e9, 3), "unit": "GB/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(tb * 1e3, 2), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": f"{n_all} streams, sizes log-uniform over [1 KiB, 64 MiB] scaled to {job_out} bytes "
                               "in total, one content kind and level (1/6/9) each; half standalone gzip members (one "
                               "gi_inflate_batch call), half deflate entries of one ZIP archive (one gi_inflate_zip call: "
                               "central directory read, entries checked against its CRC-32s) (seed 3)"
                               + (f"; shared over {ws} ranks largest first, no exchange" if ws > 1
                                  else f"; {total_in} bytes compressed"),
                   "io": "pinned host memory in (members and the archive), pinned host buffers out, every CRC-32 "
                         "computed on the GPU",
                   "members": len(mem), "zip_entries": len(ent), "zip_bytes": len(zblob)},
        "plain": {"value": round(job_out / tp / 1e9, 3), "unit": "GB/s", "calls": n_all,
                  "call_ms_p50": round(pct(0.50), 3), "call_ms_p99": round(pct(0.99), 3),
                  "call_ms_p999": round(pct(0.999), 3)},
        "batched_over_plain": round(tp / tb, 2), "cpu_baseline": cpu,
        "batched_passes": passes, "gpu_launches": prof["launches"],
        "stages_ms": {k: round(v, 2) for k, v in prof["kernel_ms"].items()},
    }
    print(json.dumps(line), flush=True)
    g.close()


def serve_pool(seed, npool):
    """The serving workload's request pool: npool gzip members, sizes log-uniform over
    [4 KiB, 256 MiB], content and level as the mixed workload (cached on local disk)."""
    import pickle

    from gpuzip_gb300 import workloads as W

    os.makedirs(CACHE, exist_ok=True)
    path = os.path.join(CACHE, f"serve_s{seed}_n{npool}.pkl")
    if os.path.exists(path):
        with open(path, "rb") as f:
            return pickle.load(f)
    pool = W.many_streams(seed=seed, n=npool, lo=4 << 10, hi=256 << 20, all_gzip=True)
    for j, x in enumerate(pool):
        x["damaged"] = W.zero_sector(x["data"], seed, j)
    with open(path + ".tmp", "wb") as f:
        pickle.dump(pool, f, protocol=pickle.HIGHEST_PROTOCOL)
    os.replace(path + ".tmp", path)
    return pool


def run_serve(args, ws, rank, local):
    """The serving loop: requests arriving as a Poisson process, each one gzip member of the pool
    (a tenth of them rescue requests, whose member has one zeroed 4 KiB sector), served by the
    request server (gi_server_*: HBM-budget admission into a resident device arena, passes of the
    batched form on `--workers` concurrent decode loops) and, on the same arrivals, by the plain
    form (one gi_inflate_gzip call per request, in arrival order, one at a time). Each form is also
    run saturated (every request queued at once) for its capacity."""
    import queue

    import torch

    from gpuzip_gb300 import gpuinflate, gzrescue
    from gpuzip_gb300 import workloads as W

    torch.cuda.set_device(local)
    os.environ["GPUZIP_RESCUE_DEVICE"] = str(local)
    seed = args.seed if args.seed != 2 else 5
    pool = serve_pool(seed, args.pool)
    arrivals, member, rescue = W.serve_trace(seed=seed, rate=args.rate, seconds=args.serve_seconds, npool=len(pool))
    n = len(arrivals)
    # every pool member and its damaged copy in one pinned host buffer
    blobs = []
    for x in pool:
        blobs += [x["data"], x["damaged"]]
    offs, pos = [], 0
    for b in blobs:
        offs.append(pos)
        pos += (len(b) + 4095) // 4096 * 4096
    host = torch.empty(pos, dtype=torch.uint8).pin_memory()
    hv = host.numpy()
    import numpy as np

    for b, o in zip(blobs, offs):
        hv[o:o + len(b)] = np.frombuffer(b, dtype=np.uint8)
    base_ptr = host.data_ptr()
    req_ptr = [base_ptr + offs[2 * int(member[k]) + int(rescue[k])] for k in range(n)]
    req_size = [len(blobs[2 * int(member[k]) + int(rescue[k])]) for k in range(n)]
    want_size = [pool[int(member[k])]["size"] for k in range(n)]
    want_crc = [pool[int(member[k])]["crc"] for k in range(n)]
    good_out = sum(want_size[k] for k in range(n) if not rescue[k])
    offered = sum(want_size) / args.serve_seconds
    req_flags = [gpuinflate.GI_STREAM_GZIP | (gpuinflate.GI_REQ_RESCUE if rescue[k] else 0) for k in range(n)]

    def check(status, crc, size, k):
        if rescue[k]:  # counted apart: a small member may have no block header left after its sector
            return True
        return status == 0 and crc == want_crc[k] and size == want_size[k]

    def pct(v, p):
        q = sorted(v)
        return round(q[min(len(q) - 1, int(p * len(q)))] * 1e3, 3)

    def lat_summary(lat):
        return {"p50": pct(lat, 0.50), "p99": pct(lat, 0.99), "p999": pct(lat, 0.999), "max": round(max(lat) * 1e3, 3)}

    def served(saturate):
        srv = gpuinflate.Server(local, workers=args.workers, hbm_budget=args.hbm_budget,
                                rescue_workers=args.rescue_workers)
        for k in range(min(8, n)):  # warm-up: first launches, first touch of the output buffers
            srv.submit((req_ptr[k], req_size[k]), flags=req_flags[k], tag=1 << 40 | k)
        srv.drain()
        srv.results.clear()
        st0 = srv.stats()
        base = srv.clock() + 0.02
        for k in range(n):
            if not saturate:
                d = base + arrivals[k] - srv.clock()
                if d > 0:
                    time.sleep(d)
            srv.submit((req_ptr[k], req_size[k]), flags=req_flags[k], tag=k)
        srv.drain()
        st = srv.stats()
        res = srv.results
        bad = [k for k in range(n) if not check(res[k]["status"], res[k]["crc32"], res[k]["out_size"], k)]
        t_arr = [base + (0.0 if saturate else arrivals[k]) for k in range(n)]
        lat = [res[k]["t_done"] - t_arr[k] for k in range(n)]
        span = max(res[k]["t_done"] for k in range(n)) - base
        rescued_out = sum(res[k]["out_size"] for k in range(n) if rescue[k])
        same_len = sum(1 for k in range(n) if rescue[k] and res[k]["out_size"] == want_size[k])
        nothing = sum(1 for k in range(n) if rescue[k] and res[k]["status"] != 0)
        batch = [res[k]["pass_requests"] for k in range(n)]
        srv.close()
        for key in ("submitted", "completed", "failed", "passes", "alone", "overlapped", "in_bytes", "out_bytes"):
            st[key] -= st0[key]
        st["busy_s"] = round(st["busy_s"] - st0["busy_s"], 3)
        # where the slowest thousandth of the requests spent their time
        slow = sorted(range(n), key=lambda k: -lat[k])[:max(1, n // 1000)]
        ms = lambda v: round(v * 1e3, 2)
        tail = [{"out_mb": round(want_size[k] / 2**20, 1), "latency_ms": ms(lat[k]),
                 "admit_ms": ms(res[k]["t_admit"] - t_arr[k]), "queue_ms": ms(res[k]["t_start"] - res[k]["t_admit"]),
                 "pass_ms": ms(res[k]["t_done"] - res[k]["t_start"]), "pass_requests": res[k]["pass_requests"]}
                for k in slow[:5]]
        return {"gbs": round(good_out / span / 1e9, 3), "seconds": round(span, 3), "latency_ms": lat_summary(lat),
                "wrong": len(bad), "mean_requests_per_pass": round(statistics.mean(batch), 2), "server": st,
                "slowest": tail,
                "rescue": {"requests": int(rescue.sum()), "latency_ms": lat_summary([lat[k] for k in range(n) if rescue[k]]),
                           "decode_latency_ms": lat_summary([lat[k] for k in range(n) if not rescue[k]]),
                           "output_gb": round(rescued_out / 1e9, 3), "original_length": same_len,
                           "nothing_to_rescue": nothing}}

    def plain(saturate):
        g = gpuinflate.Gpu(local)
        lib = g.lib
        stats = gpuinflate.Stats()
        msize = ctypes.c_uint64(0)
        q = queue.Queue()
        done = [None] * n
        status = [None] * n

        rlib = gzrescue.bind(gpuinflate.LIB_PATH)
        ropt = gzrescue.Options(ctypes.sizeof(gzrescue.Options), 0, 0, 0, 0, 0, 0)  # the default options
        got = [0]

        def count(_u, _d, _m, nb):  # the rescue's output reaches the host; only its size is kept
            got[0] += nb
            return 0

        rsink = gzrescue.SINK(count)

        def one(k):
            if rescue[k]:
                got[0] = 0
                res = ctypes.c_void_p()
                rc = rlib.gr_rescue(ctypes.cast(req_ptr[k], ctypes.c_char_p), req_size[k], ctypes.byref(ropt), rsink, None,
                                    ctypes.byref(res))
                if res.value:
                    rlib.gr_free(res)
                return rc, 0, got[0]
            rc = lib.gi_inflate_gzip(g.ctx, ctypes.cast(req_ptr[k], ctypes.c_char_p), req_size[k], gpuinflate.SINK(),
                                     None, ctypes.byref(msize), ctypes.byref(stats))
            return rc, lib.gi_last_crc32(g.ctx), stats.out_size

        for k in range(min(8, n)):
            one(k)

        def consumer():
            while True:
                k = q.get()
                if k is None:
                    return
                rc, crc, size = one(k)
                done[k] = time.perf_counter()
                status[k] = (rc, crc, size)

        th = threading.Thread(target=consumer)
        th.start()
        base = time.perf_counter() + 0.02
        for k in range(n):
            if not saturate:
                d = base + arrivals[k] - time.perf_counter()
                if d > 0:
                    time.sleep(d)
            q.put(k)
        q.put(None)
        th.join()
        g.close()
        bad = [k for k in range(n) if not check(status[k][0], status[k][1], status[k][2], k)]
        lat = [done[k] - (base + (0.0 if saturate else arrivals[k])) for k in range(n)]
        span = max(done) - base
        return {"gbs": round(good_out / span / 1e9, 3), "seconds": round(span, 3), "latency_ms": lat_summary(lat),
                "wrong": len(bad),
                "rescue": {"latency_ms": lat_summary([lat[k] for k in range(n) if rescue[k]]),
                           "decode_latency_ms": lat_summary([lat[k] for k in range(n) if not rescue[k]])}}

    with Clocks() as clocks:
        s_live = served(False)
    p_live = plain(False)
    s_sat = served(True)
    p_sat = plain(True)
    line = {
        "metric": f"served decode: decompressed GB/s and request latency, Poisson {args.rate:g} requests/s for "
                  f"{args.serve_seconds:g} s, 1 GB300",
        "value": s_live["gbs"], "unit": "GB/s", "n_gpus": ws, "steps": 1, "warmup": 1,
        "ms_per_step": round(s_live["seconds"] * 1e3, 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": f"{n} requests (seed {seed}): gzip members drawn from a pool of {len(pool)}, sizes "
                               "log-uniform over [4 KiB, 256 MiB], content and level as the mixed workload; "
                               f"{int(rescue.sum())} rescue requests carry one zeroed 4 KiB sector",
                   "offered_gbs": round(offered / 1e9, 3), "hbm_budget": args.hbm_budget, "workers": args.workers,
                   "io": "pinned host memory in, pinned host buffers out; CRC-32 and ISIZE of every decode request checked on "
                         "the GPU"},
        "latency_ms": s_live["latency_ms"],
        "served": s_live,
        "plain": p_live,
        "saturated": {"served_gbs": s_sat["gbs"], "plain_gbs": p_sat["gbs"],
                      "served_over_plain": round(s_sat["gbs"] / p_sat["gbs"], 2), "served": s_sat, "plain": p_sat},
        "rescue": "rescue requests are recovered (gr_rescue with inference off) by the server's rescue loop beside the "
                  "passes, and by one gr_rescue call each in the plain form; `value` counts only the undamaged requests' bytes",
        "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)


def run_bgzf(args, ws, rank, local):
    """A BGZF file (bgzip's 64 KiB members) of log text: every member in one gi_inflate_members
    call (members decoded together) against one gi_inflate_gzip call per member (how gpuzip's host
    decodes a gzip file, member by member)."""
    import torch

    from gpuzip_gb300 import gpuinflate
    from gpuzip_gb300 import workloads as W

    torch.cuda.set_device(local)
    os.makedirs(CACHE, exist_ok=True)
    path = os.path.join(CACHE, f"bgzf_s1_{args.bgzf_mb}.gz")
    if not os.path.exists(path):
        data = W.log_text(1, args.bgzf_mb << 20, exact=True)
        with open(path + ".tmp", "wb") as f:
            f.write(W.bgzf(data))
        os.replace(path + ".tmp", path)
    with open(path, "rb") as f:
        blob = f.read()
    out_size = args.bgzf_mb << 20
    pinned = torch.empty(len(blob), dtype=torch.uint8).pin_memory()
    pinned.numpy()[:] = torch.frombuffer(bytearray(blob), dtype=torch.uint8).numpy()
    ptr = ctypes.cast(pinned.data_ptr(), ctypes.c_char_p)
    g = gpuinflate.Gpu(local)
    lib = g.lib
    info = gpuinflate.MembersInfo()
    info.size = ctypes.sizeof(gpuinflate.MembersInfo)
    stats = gpuinflate.Stats()

    def batched():
        rc = lib.gi_inflate_members(g.ctx, ptr, len(blob), gpuinflate.SINK(), None, ctypes.byref(info), ctypes.byref(stats))
        if rc != 0 or stats.out_size != out_size:
            raise RuntimeError(f"member decode failed: {rc} {lib.gi_last_error(g.ctx)}")

    # member boundaries from the BGZF headers, for the one-call-per-member form
    starts, pos = [], 0
    while pos < len(blob):
        starts.append(pos)
        pos += int.from_bytes(blob[pos + 16:pos + 18], "little") + 1
    msize = ctypes.c_uint64(0)

    ends = starts[1:] + [len(blob)]

    def plain():  # each call given exactly its member (gpuzip's host passes the rest of the file)
        total = 0
        for a, e in zip(starts, ends):
            rc = lib.gi_inflate_gzip(g.ctx, ctypes.cast(pinned.data_ptr() + a, ctypes.c_char_p), e - a,
                                     gpuinflate.SINK(), None, ctypes.byref(msize), ctypes.byref(stats))
            if rc != 0:
                raise RuntimeError(f"member at {a} failed: {rc}")
            total += stats.out_size
        if total != out_size:
            raise RuntimeError("plain decode: wrong size")

    for _ in range(args.warmup):
        batched()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        batched()
    tb = (time.perf_counter() - t0) / args.steps
    members = info.members
    batched_members = info.batched
    plain()
    t0 = time.perf_counter()
    plain()
    tp = time.perf_counter() - t0
    line = {
        "metric": f"decompressed GB/s, a BGZF file of {members} members (64 KiB of log text each), whole-file call",
        "value": round(out_size / tb / 1e9, 3), "unit": "GB/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(tb * 1e3, 2), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": f"{args.bgzf_mb} MiB of log text (seed 1) as bgzip writes it: members of 65,280 input "
                               f"bytes at level 6, {len(blob)} bytes compressed",
                   "io": "pinned host memory in, output to the library's pinned buffers (no sink)"},
        "members": members, "members_batched": batched_members,
        "plain": {"value": round(out_size / tp / 1e9, 3), "unit": "GB/s", "calls": len(starts),
                  "ms_per_call": round(tp / len(starts) * 1e3, 3)},
        "whole_file_over_plain": round(tp / tb, 1),
    }
    print(json.dumps(line), flush=True)
    g.close()


def rescue_workload(nfiles):
    """(damaged .tar.gz bytes, info) of the rescue workload, cached on local disk between runs."""
    from gpuzip_gb300 import workloads as W

    os.makedirs(CACHE, exist_ok=True)
    path = os.path.join(CACHE, f"rescue_tar_s4_{nfiles}.gz")
    meta = path + ".json"
    if not (os.path.exists(path) and os.path.exists(meta)):
        member, info = W.rescue_tar(seed=4, nfiles=nfiles)
        damaged, done = W.rescue_damage(member, seed=4)
        info = {"crc": info["crc"], "size": info["size"], "member_bytes": len(member), "damage": done,
                "files": len(info["files"])}
        with open(path + ".tmp", "wb") as f:
            f.write(damaged)
        os.replace(path + ".tmp", path)
        with open(meta, "w") as f:
            json.dump(info, f)
    with open(path, "rb") as f:
        data = f.read()
    with open(meta) as f:
        info = json.load(f)
    return data, info


def run_rescue(args, ws, rank, local):
    """The damaged .tar.gz (2,000 files of mixed content, three zeroed sectors, a span written
    twice, CR LF to LF in a 16 MiB region) through gr_rescue: `value` with no sink (output and
    mask left in device memory), `e2e` with a sink that copies every output byte and mask byte to
    host memory."""
    import numpy as np
    import torch

    from gpuzip_gb300 import gpuinflate, gzrescue

    if args.impl == "reference":
        if rank == 0:
            print(json.dumps({"impl": "reference", "unavailable": "gzrescue's rescue library is built from the reference's "
                              "gpuinflate/rescue.cpp, which is not present on this host"}), flush=True)
        return
    torch.cuda.set_device(local)
    os.environ["GPUZIP_RESCUE_DEVICE"] = str(local)
    data, info = rescue_workload(args.rescue_files)
    pinned = torch.empty(len(data), dtype=torch.uint8).pin_memory()
    pinned.numpy()[:] = np.frombuffer(data, dtype=np.uint8)
    ptr = ctypes.cast(pinned.data_ptr(), ctypes.c_char_p)
    lib = gzrescue.bind(gpuinflate.LIB_PATH)
    opt = gzrescue.Options(ctypes.sizeof(gzrescue.Options), 0, 0, 0, 0, 0, 0)  # the default options: inference on
    out_cap = info["size"] + (64 << 20)
    h_out = torch.empty(out_cap, dtype=torch.uint8).pin_memory()
    h_mask = torch.empty(out_cap, dtype=torch.uint8).pin_memory()
    pos = [0]
    base_out, base_mask = h_out.data_ptr(), h_mask.data_ptr()

    def take(_user, d, m, n):
        if pos[0] + n > out_cap:
            return 1
        ctypes.memmove(base_out + pos[0], d, n)
        ctypes.memmove(base_mask + pos[0], m, n)
        pos[0] += n
        return 0

    sink = gzrescue.SINK(take)

    def call(with_sink):
        pos[0] = 0
        res = ctypes.c_void_p()
        rc = lib.gr_rescue(ptr, len(data), ctypes.byref(opt), sink if with_sink else gzrescue.SINK(), None,
                           ctypes.byref(res))
        if rc != 0 or not res.value:
            raise RuntimeError(f"gr_rescue failed: {rc}")
        st = lib.gr_result_stats(res).contents
        s = {f: getattr(st, f) for f in gzrescue.STAT_FIELDS}
        lib.gr_free(res)
        if with_sink and pos[0] != s["output_size"]:
            raise RuntimeError("the sink did not receive the whole output")
        return s

    for _ in range(args.warmup):
        first = call(False)
    with Clocks() as clocks:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            s = call(False)
            if s != first:
                raise RuntimeError("rescue results differ between runs")
        t = (time.perf_counter() - t0) / args.steps
    launches = int(lib.gr_last_launches())
    call(True)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        se = call(True)
    te = (time.perf_counter() - t0) / args.steps
    if se != first:
        raise RuntimeError("rescue results differ with a sink")
    mask = h_mask.numpy()[:se["output_size"]]
    counts = np.bincount(mask, minlength=4).tolist()
    if counts[1] != se["exact_bytes"] or counts[2] != se["suspect_bytes"] or counts[0] != se["unknown_bytes"]:
        raise RuntimeError(f"mask counts {counts} disagree with the statistics {se}")
    out = s["output_size"]
    # the recovered-file list: the tar walk over the output where it lies (one call, timed apart)
    res, tarp = ctypes.c_void_p(), ctypes.c_void_p()
    t0 = time.perf_counter()
    rc = lib.gr_rescue_tar(ptr, len(data), ctypes.byref(opt), gzrescue.SINK(), None, ctypes.byref(res), ctypes.byref(tarp))
    tt = time.perf_counter() - t0
    if rc != 0 or not tarp.value:
        raise RuntimeError(f"gr_rescue_tar failed: {rc}")
    ts = lib.gr_tar_result_stats(tarp).contents
    tar = {"files": ts.files, "intact": ts.intact, "unverified": ts.unverified, "suspect": ts.suspect,
           "partial": ts.partial, "inferred": ts.inferred, "skipped_regions": ts.skipped, "repaired": ts.repaired,
           "rescue_and_walk_ms": round(tt * 1e3, 2), "walk_ms": round((tt - t) * 1e3, 2)}
    lib.gr_tar_free(tarp)
    lib.gr_free(res)
    line = {
        "metric": "rescued GB/s (output bytes), a damaged 2,000-file .tar.gz of mixed content, 1 GB300",
        "value": round(out / t / 1e9, 3), "unit": "GB/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(t * 1e3, 2), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u8", "data": "synthetic",
        "config": {"workload": f"a .tar.gz of {info['files']} files (sizes log-uniform over [4 KiB, 8 MiB], contents of the "
                               "mixed workload, seed 4), the tar stream in 1 MiB segments at levels 1/6/9 in one Deflate stream; "
                               f"{info['size']} bytes of tar, {len(data)} bytes damaged: three 4 KiB sectors zeroed, a 64 KiB "
                               f"span written twice, CR LF to LF in a 16 MiB region ({info['damage']['crlf'][1]} CRs lost)",
                   "options": "the default gr_options (the inference of lost window bytes on)",
                   "io": "value: host input (page-locked), output and mask left in device memory (no sink); e2e: every "
                         "output and mask byte delivered to a host sink"},
        "e2e": {"value": round(out / te / 1e9, 3), "unit": "GB/s", "h2d_bytes_per_step": len(data),
                "d2h_bytes_per_step": 2 * out},
        "gpu_launches": launches,
        "cpu_baseline": None,
        "cpu_baseline_unavailable": "the reference's rescue library is built from its rescue.cpp, which is not on this host",
        "result": {k: s[k] for k in ("output_size", "exact_bytes", "suspect_bytes", "unknown_bytes", "inferred_bytes", "headers",
                                     "pieces", "damaged", "crc_check", "hidden_damage")},
        "mask_counts": counts,
        "tar": tar,
        "clocks": clocks.summary(),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def config_of(args, info):
    if args.workload == "text":
        what = "one gzip member of 64 MiB of log text (seed 1), level 6"
    else:
        what = (f"one gzip member, {args.nseg} x 1 MiB segments of mixed content (seed {args.seed}), levels 1/6/9 "
                "changed by deflateParams inside one Deflate stream (no sync flush)")
    return {"workload": what, "output_bytes": info["size"], "compressed_bytes": info["deflate_size"],
            "l2": "inputs larger than L2 (no flush)", "parallelism": "replicas"}


def text_workload():
    """(member bytes, info) of the 64 MiB log-text member (seed 1), cached on local disk."""
    from gpuzip_gb300 import workloads as W

    os.makedirs(CACHE, exist_ok=True)
    path = os.path.join(CACHE, "text_s1_64m.gz")
    meta = path + ".json"
    if os.path.exists(path) and os.path.exists(meta):
        with open(meta) as f:
            info = json.load(f)
        with open(path, "rb") as f:
            return f.read(), info
    member, text = W.single_text_member(seed=1)
    info = {"crc": zlib.crc32(text), "size": len(text), "deflate_size": len(member) - 18}
    with open(path + ".tmp", "wb") as f:
        f.write(member)
    os.replace(path + ".tmp", path)
    with open(meta, "w") as f:
        json.dump(info, f)
    return member, info


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nseg", type=int, default=4096)
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--seg-out-mb", type=int, default=0)
    ap.add_argument("--cpu-sample-mb", type=int, default=768)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--profile-only", action="store_true", help="one device-resident decode, no timing (for ncu)")
    ap.add_argument("--workload", default="member", choices=["member", "text", "batch", "serve", "bgzf", "rescue"])
    ap.add_argument("--rescue-files", type=int, default=2000, help="rescue: files in the .tar.gz")
    ap.add_argument("--nstreams", type=int, default=10000)
    ap.add_argument("--batch-total", type=float, default=8e9)
    ap.add_argument("--rate", type=float, default=200.0, help="serve: requests per second")
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--pool", type=int, default=256, help="serve: distinct members requests draw from")
    ap.add_argument("--workers", type=int, default=3, help="serve: concurrent decode loops")
    ap.add_argument("--rescue-workers", type=int, default=3, help="serve: concurrent rescue loops (at most 4)")
    ap.add_argument("--hbm-budget", type=float, default=120e9)
    ap.add_argument("--bgzf-mb", type=int, default=256, help="bgzf: MiB of output")
    args = ap.parse_args()
    ws, rank, local = dist_env()
    if args.workload == "serve":
        run_serve(args, ws, rank, local)
        return
    if args.workload == "bgzf":
        run_bgzf(args, ws, rank, local)
        return
    if args.workload == "rescue":
        run_rescue(args, ws, rank, local)
        return
    if args.workload == "batch":
        run_batch(args, ws, rank, local)
        return
    member, info = text_workload() if args.workload == "text" else workload(args.seed, args.nseg)
    if args.impl == "reference":
        run_reference(args, member, info, ws, rank)
        return

    import torch

    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from gpuzip_gb300 import gpuinflate

    if not os.path.exists(gpuinflate.LIB_PATH):
        import __graft_entry__

        __graft_entry__.build()
    g = gpuinflate.Gpu(local, segment_out_mb=args.seg_out_mb)
    body = member[10:10 + info["deflate_size"]]
    d_in = torch.frombuffer(bytearray(body), dtype=torch.uint8).cuda()
    d_out = torch.empty(info["size"] + 4096, dtype=torch.uint8, device="cuda")

    def step():
        n, st = g.inflate_device(d_in.data_ptr(), d_in.numel(), d_out.data_ptr(), d_out.numel())
        if n != info["size"] or g.last_crc32() != info["crc"]:
            raise RuntimeError(f"wrong output: {n} bytes, crc {g.last_crc32():08x}, want {info['size']} {info['crc']:08x}")
        return st, g.last_profile()

    if args.profile_only:
        step()
        torch.cuda.synchronize()
        return
    # the context's autotuner tries its candidate settings on the first calls of a kind of stream:
    # those calls come before the warm-up, untimed
    for _ in range(8):
        _, prof = step()
        if prof.tuned:
            break
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier = (lambda: torch.distributed.barrier()) if ws > 1 else (lambda: None)
    uuid = None
    try:
        uuid = "GPU-" + str(torch.cuda.get_device_properties(local).uuid)
    except Exception:
        pass
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    profs = []
    barrier()
    torch.cuda.synchronize()
    with Clocks(uuid) as clocks:
        for a, b in evs:
            a.record()
            st, pr = step()
            b.record()
            profs.append(pr.as_dict())
        torch.cuda.synchronize()
    barrier()
    step_ms = [a.elapsed_time(b) for a, b in evs]
    total_s = sum(step_ms) / 1e3
    if ws > 1:
        t = torch.tensor([total_s], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_s = float(t.item())
    value = ws * args.steps * info["size"] / total_s / 1e9

    # roofline: the kernel with the largest share of GPU time
    kms = {k: sum(p["kernel_ms"][k] for p in profs) for k in profs[0]["kernel_ms"]}
    top = max(kms, key=kms.get)
    nl = sum(p["decode_launches"] for p in profs)  # every kernel kind runs once per segment
    per_launch_s = kms[top] / 1e3 / nl
    alg_bytes = sum(p["in_bytes"] + p["out_bytes"] for p in profs) / nl
    peak, peak_kind = peaks()
    achieved = alg_bytes / per_launch_s / 1e9
    roofline = {"bound": "hbm", "kernel": top, "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 5), "peak_kind": peak_kind, "traffic": traffic_per_launch(top) if args.workload == "member" else None,
                "algorithmic_bytes_per_launch": int(alg_bytes), "launch_ms": round(per_launch_s * 1e3, 3),
                "kernel_share": {k: round(v / sum(kms.values()), 4) for k, v in kms.items()}}
    gpu_launches = sum(p["launches"] for p in profs)

    e2e = None
    if not args.no_e2e:
        pinned = torch.frombuffer(bytearray(member), dtype=torch.uint8).pin_memory()
        lib = g.lib
        msize = ctypes.c_uint64(0)
        stats = gpuinflate.Stats()

        def e2e_step():
            rc = lib.gi_inflate_gzip(g.ctx, ctypes.cast(pinned.data_ptr(), ctypes.c_char_p), pinned.numel(),
                                     gpuinflate.SINK(), None, ctypes.byref(msize), ctypes.byref(stats))
            if rc != 0 or stats.out_size != info["size"]:
                raise RuntimeError(f"e2e failed: {rc} {lib.gi_last_error(g.ctx)}")

        for _ in range(8):  # the autotuner's calls for this kind of stream (a gzip member: its ISIZE known)
            e2e_step()
            if g.last_profile().tuned:
                break
        for _ in range(max(1, args.warmup)):
            e2e_step()
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        torch.cuda.synchronize()
        e2e_s = time.perf_counter() - t0
        if ws > 1:
            t = torch.tensor([e2e_s], device="cuda", dtype=torch.float64)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            e2e_s = float(t.item())
        e2e = {"value": round(ws * args.steps * info["size"] / e2e_s / 1e9, 3), "unit": "GB/s",
               "stages_s": {k: round(getattr(stats, k), 4) for k in ("upload_s", "find_s", "decode_s", "resolve_s",
                                                                      "download_s", "seconds")},
               "h2d_bytes_per_step": len(member), "d2h_bytes_per_step": info["size"],
               "path": "gi_inflate_gzip from pinned host memory, CRC-32/ISIZE checked on the GPU, output to pinned "
                       "host buffers (no sink)"}

    cpu = None
    if rank == 0 and not args.no_cpu:
        body = member[10:10 + info["deflate_size"]]
        sample = cpu_sample(args, info)
        res = cpu_candidates(body, sample, info["size"] / info["deflate_size"], os.cpu_count() or 1)
        cpu = cpu_line(res, sample)
    if rank == 0:
        line = {
            "metric": metric_of(args), "value": round(value, 3), "unit": "GB/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(total_s / args.steps * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic", "config": config_of(args, info),
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks.summary(),
            "gpu_launches": gpu_launches,
            "stages_ms_per_step": {k: round(v / args.steps, 3) for k, v in kms.items()},
            "jobs_per_step": profs[0]["jobs"], "segments_per_step": st.segments,
            "tuning": {k: profs[-1][k] for k in ("probe_spacing_bits", "probe_lead_bits", "job_share_div", "tuned")},
        }
        print(json.dumps(line), flush=True)
    g.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
