"""Python binding of libgpuinflate.so over its C interface (ctypes).

It calls the library the way gpuzip's Rust host does (src/inflate.rs:110-168): load the shared
library, check ``gi_abi_version() == 1``, create one context with ``gi_config{16, device, 0, 0}``
and a 512-byte error buffer, serialise calls on a lock (a context serves one call at a time),
pass a sink callback that returns nonzero to stop, and map the return codes 1/2/3/other to
data / truncated / aborted / GPU errors. There is no CPU fallback: without the built library or
a GPU every call raises.
"""
import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgpuinflate.so")
ABI_VERSION = 1

GI_OK, GI_ERR_DATA, GI_ERR_TRUNCATED, GI_ERR_ABORTED, GI_ERR_GPU, GI_ERR_ARG, GI_ERR_SPACE = range(7)

EXPORTED = (
    "gi_abi_version",
    "gi_create",
    "gi_inflate",
    "gi_last_error",
    "gi_device_name",
    "gi_destroy",
    "gi_last_crc32",
    "gi_last_isize",
    "gi_inflate_device",
    "gi_inflate_gzip",
    "gi_last_profile",
    "gi_crc32_device_noalloc",
    "gi_inflate_batch",
    "gi_inflate_members",
    "gi_inflate_zip",
    "gi_server_create",
    "gi_server_submit",
    "gi_server_drain",
    "gi_server_clock",
    "gi_server_read_stats",
    "gi_server_destroy",
    "gi_tar_index_device",
    "gi_tar_entries",
    "gi_tar_end",
    "gi_tar_free",
)

GI_STREAM_GZIP = 1
GI_STREAM_CRC = 2
GI_STREAM_MAPPED = 4
GI_REQ_RESCUE = 8  # server requests only: a damaged gzip member to recover (output then mask)


class Config(ctypes.Structure):
    """gi_config (gpuinflate.h)"""

    _fields_ = [("size", ctypes.c_uint32), ("device", ctypes.c_int32), ("segment_out_mb", ctypes.c_uint32),
                ("segment_in_kb", ctypes.c_uint32)]


class Stats(ctypes.Structure):
    """gi_stats (gpuinflate.h)"""

    _fields_ = [("in_used", ctypes.c_uint64), ("out_size", ctypes.c_uint64), ("segments", ctypes.c_uint32),
                ("rounds", ctypes.c_uint32), ("jobs", ctypes.c_uint64), ("seconds", ctypes.c_double),
                ("upload_s", ctypes.c_double), ("find_s", ctypes.c_double), ("decode_s", ctypes.c_double),
                ("resolve_s", ctypes.c_double), ("download_s", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Profile(ctypes.Structure):
    """gi_profile (gpuinflate.h)"""

    KINDS = ("find", "decode", "stored", "local", "windows", "next_window", "crc")
    _fields_ = [("size", ctypes.c_uint32), ("launches", ctypes.c_uint32), ("kernel_ms", ctypes.c_double * 7),
                ("decode_launches", ctypes.c_uint32), ("reserved", ctypes.c_uint32), ("in_bytes", ctypes.c_uint64),
                ("out_bytes", ctypes.c_uint64), ("jobs", ctypes.c_uint64), ("extents", ctypes.c_uint64),
                ("stored_blocks", ctypes.c_uint64), ("probes", ctypes.c_uint64),
                ("probe_spacing_bits", ctypes.c_uint32), ("probe_lead_bits", ctypes.c_uint32),
                ("job_share_div", ctypes.c_float), ("tuned", ctypes.c_uint32)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_ if k not in ("size", "kernel_ms")}
        d["kernel_ms"] = dict(zip(self.KINDS, list(self.kernel_ms)))
        return d


class Stream(ctypes.Structure):
    """gi_stream (gpuinflate.h): one stream of a batch"""

    _fields_ = [("in_", ctypes.c_void_p), ("in_size", ctypes.c_uint64), ("flags", ctypes.c_uint32),
                ("expected_crc", ctypes.c_uint32), ("out_offset", ctypes.c_uint64), ("out_size", ctypes.c_uint64),
                ("in_used", ctypes.c_uint64), ("crc32", ctypes.c_uint32), ("status", ctypes.c_int32)]


SINK = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint8), ctypes.c_size_t)


class MembersInfo(ctypes.Structure):
    """gi_members_info (gpuinflate.h)"""

    _fields_ = [("size", ctypes.c_uint32), ("members", ctypes.c_uint32), ("batched", ctypes.c_uint64),
                ("trailing", ctypes.c_uint64), ("trailing_zero", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k not in ("size", "reserved")}


class ZipEntry(ctypes.Structure):
    """gi_zip_entry (gpuinflate.h)"""

    _fields_ = [("size", ctypes.c_uint32), ("index", ctypes.c_uint32), ("method", ctypes.c_uint16),
                ("flags", ctypes.c_uint16), ("status", ctypes.c_int32), ("out_size", ctypes.c_uint64),
                ("in_size", ctypes.c_uint64), ("crc32", ctypes.c_uint32), ("name_len", ctypes.c_uint32)]


ENTRY_SINK = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ZipEntry), ctypes.c_void_p,
                              ctypes.c_void_p, ctypes.c_size_t)


class TarEntry(ctypes.Structure):
    """gi_tar_entry (gpuinflate.h): one entry of a tar archive in device memory"""

    _fields_ = [("name", ctypes.c_char_p), ("header", ctypes.c_uint64), ("offset", ctypes.c_uint64),
                ("size", ctypes.c_uint64), ("type", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class ServerConfig(ctypes.Structure):
    """gi_server_config (gpuinflate.h)"""

    _fields_ = [("size", ctypes.c_uint32), ("device", ctypes.c_int32), ("workers", ctypes.c_uint32),
                ("max_batch", ctypes.c_uint32), ("pass_out_mb", ctypes.c_uint32), ("rescue_workers", ctypes.c_uint32),
                ("hbm_budget", ctypes.c_uint64), ("arena_bytes", ctypes.c_uint64)]


class Result(ctypes.Structure):
    """gi_result (gpuinflate.h): one finished request of the server"""

    _fields_ = [("tag", ctypes.c_uint64), ("status", ctypes.c_int32), ("crc32", ctypes.c_uint32),
                ("out_size", ctypes.c_uint64), ("in_used", ctypes.c_uint64), ("t_submit", ctypes.c_double),
                ("t_admit", ctypes.c_double), ("t_start", ctypes.c_double), ("t_done", ctypes.c_double),
                ("pass_requests", ctypes.c_uint32), ("worker", ctypes.c_uint32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServerStats(ctypes.Structure):
    """gi_server_stats (gpuinflate.h)"""

    _fields_ = [("size", ctypes.c_uint32), ("workers", ctypes.c_uint32), ("submitted", ctypes.c_uint64),
                ("completed", ctypes.c_uint64), ("failed", ctypes.c_uint64), ("passes", ctypes.c_uint64),
                ("alone", ctypes.c_uint64), ("overlapped", ctypes.c_uint64), ("in_bytes", ctypes.c_uint64),
                ("out_bytes", ctypes.c_uint64), ("device_bytes", ctypes.c_uint64), ("arena_bytes", ctypes.c_uint64),
                ("arena_peak", ctypes.c_uint64), ("busy_s", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "size"}


DONE = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.POINTER(Result), ctypes.c_void_p)


class InflateError(Exception):
    def __init__(self, code, msg):
        super().__init__(f"{['ok', 'data', 'truncated', 'aborted', 'gpu', 'arg', 'space'][code] if code < 7 else code}: {msg}")
        self.code = code
        self.msg = msg


_lib = None


def load(path=None):
    """The library, loaded once; raises when it is missing or speaks another interface version."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is not built (run gpuzip_gb300/build.py)")
    lib = ctypes.CDLL(path)
    lib.gi_abi_version.restype = ctypes.c_uint32
    if lib.gi_abi_version() != ABI_VERSION:
        raise RuntimeError(f"{path} speaks interface {lib.gi_abi_version()}, expected {ABI_VERSION}")
    vp, u64 = ctypes.c_void_p, ctypes.c_uint64
    lib.gi_create.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(vp), ctypes.c_char_p, ctypes.c_size_t]
    lib.gi_create.restype = ctypes.c_int
    lib.gi_inflate.argtypes = [vp, ctypes.c_char_p, u64, u64, SINK, vp, ctypes.POINTER(Stats)]
    lib.gi_inflate.restype = ctypes.c_int
    lib.gi_last_error.argtypes = [vp]
    lib.gi_last_error.restype = ctypes.c_char_p
    lib.gi_device_name.argtypes = [vp]
    lib.gi_device_name.restype = ctypes.c_char_p
    lib.gi_destroy.argtypes = [vp]
    lib.gi_destroy.restype = None
    lib.gi_last_crc32.argtypes = [vp]
    lib.gi_last_crc32.restype = ctypes.c_uint32
    lib.gi_last_isize.argtypes = [vp]
    lib.gi_last_isize.restype = ctypes.c_uint32
    lib.gi_inflate_device.argtypes = [vp, vp, u64, vp, u64, ctypes.POINTER(u64), ctypes.POINTER(Stats)]
    lib.gi_inflate_device.restype = ctypes.c_int
    lib.gi_inflate_gzip.argtypes = [vp, ctypes.c_char_p, u64, SINK, vp, ctypes.POINTER(u64), ctypes.POINTER(Stats)]
    lib.gi_inflate_gzip.restype = ctypes.c_int
    lib.gi_last_profile.argtypes = [vp, ctypes.POINTER(Profile)]
    lib.gi_last_profile.restype = ctypes.c_int
    lib.gi_crc32_device_noalloc.argtypes = [ctypes.c_int, vp, u64, vp, vp, ctypes.c_char_p, ctypes.c_size_t]
    lib.gi_crc32_device_noalloc.restype = ctypes.c_int
    lib.gi_inflate_batch.argtypes = [vp, ctypes.POINTER(Stream), ctypes.c_uint32, vp, u64, ctypes.POINTER(Stats)]
    lib.gi_inflate_batch.restype = ctypes.c_int
    lib.gi_inflate_members.argtypes = [vp, ctypes.c_char_p, u64, SINK, vp, ctypes.POINTER(MembersInfo),
                                       ctypes.POINTER(Stats)]
    lib.gi_inflate_members.restype = ctypes.c_int
    lib.gi_inflate_zip.argtypes = [vp, ctypes.c_char_p, u64, ENTRY_SINK, vp, ctypes.POINTER(Stats)]
    lib.gi_inflate_zip.restype = ctypes.c_int
    lib.gi_server_create.argtypes = [ctypes.POINTER(ServerConfig), DONE, vp, ctypes.POINTER(vp), ctypes.c_char_p,
                                     ctypes.c_size_t]
    lib.gi_server_create.restype = ctypes.c_int
    lib.gi_server_submit.argtypes = [vp, vp, u64, ctypes.c_uint32, ctypes.c_uint32, u64]
    lib.gi_server_submit.restype = ctypes.c_int
    lib.gi_server_drain.argtypes = [vp]
    lib.gi_server_drain.restype = ctypes.c_int
    lib.gi_server_clock.argtypes = [vp]
    lib.gi_server_clock.restype = ctypes.c_double
    lib.gi_server_read_stats.argtypes = [vp, ctypes.POINTER(ServerStats)]
    lib.gi_server_read_stats.restype = ctypes.c_int
    lib.gi_server_destroy.argtypes = [vp]
    lib.gi_server_destroy.restype = None
    lib.gi_tar_index_device.argtypes = [vp, vp, u64, ctypes.POINTER(vp)]
    lib.gi_tar_index_device.restype = ctypes.c_int
    lib.gi_tar_entries.argtypes = [vp, ctypes.POINTER(ctypes.POINTER(TarEntry))]
    lib.gi_tar_entries.restype = ctypes.c_uint32
    lib.gi_tar_end.argtypes = [vp]
    lib.gi_tar_end.restype = u64
    lib.gi_tar_free.argtypes = [vp]
    lib.gi_tar_free.restype = None
    _lib = lib
    return lib


class Gpu:
    """One decoding context on one GPU (the Rust host's inflate::Gpu)."""

    def __init__(self, device=0, segment_out_mb=0, segment_in_kb=0, path=None):
        self.lib = load(path)
        cfg = Config(ctypes.sizeof(Config), device, segment_out_mb, segment_in_kb)
        ctx = ctypes.c_void_p()
        err = ctypes.create_string_buffer(512)
        rc = self.lib.gi_create(ctypes.byref(cfg), ctypes.byref(ctx), err, 512)
        if rc != GI_OK:
            raise InflateError(rc, f"GPU not usable: {err.value.decode(errors='replace')}")
        self.ctx = ctx
        self.device = self.lib.gi_device_name(ctx).decode(errors="replace")
        self._lock = threading.Lock()

    def close(self):
        if self.ctx:
            self.lib.gi_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _error(self, rc):
        return InflateError(rc, self.lib.gi_last_error(self.ctx).decode(errors="replace"))

    def inflate(self, data, hint=0, sink=None, collect=True):
        """Decodes the raw Deflate stream at the start of `data`. Returns (output bytes or None,
        Stats). sink(chunk) -> bool (False stops) receives the output when given."""
        parts = []

        def _cb(user, ptr, n):
            try:
                chunk = ctypes.string_at(ptr, n)
                if sink is not None:
                    return 0 if sink(chunk) else 1
                parts.append(chunk)
                return 0
            except Exception:
                return 1

        cb = SINK(_cb) if (sink is not None or collect) else SINK()
        st = Stats()
        buf = bytes(data)
        with self._lock:
            rc = self.lib.gi_inflate(self.ctx, buf, len(buf), hint, cb, None, ctypes.byref(st))
            if rc != GI_OK:
                raise self._error(rc)
        return (b"".join(parts) if collect and sink is None else None), st

    def inflate_status(self, data, hint=0):
        """(return code, output, in_used) without raising on data errors (for parity tests)."""
        parts = []

        def _cb(user, ptr, n):
            parts.append(ctypes.string_at(ptr, n))
            return 0

        st = Stats()
        buf = bytes(data)
        with self._lock:
            rc = self.lib.gi_inflate(self.ctx, buf, len(buf), hint, SINK(_cb), None, ctypes.byref(st))
        return rc, (b"".join(parts) if rc == GI_OK else b""), st.in_used

    def inflate_gzip(self, member):
        """Decodes one gzip member with the CRC-32/ISIZE check done on the GPU. Returns (output,
        member size, Stats)."""
        parts = []

        def _cb(user, ptr, n):
            parts.append(ctypes.string_at(ptr, n))
            return 0

        st = Stats()
        msize = ctypes.c_uint64(0)
        buf = bytes(member)
        with self._lock:
            rc = self.lib.gi_inflate_gzip(self.ctx, buf, len(buf), SINK(_cb), None, ctypes.byref(msize), ctypes.byref(st))
            if rc != GI_OK:
                raise self._error(rc)
        return b"".join(parts), msize.value, st

    def inflate_members(self, data, sink=None):
        """Every gzip member of `data` (gi_inflate_members). Returns (output bytes or None when a
        sink is given, info dict, Stats); raises InflateError on a failure."""
        parts = []

        def _cb(user, ptr, n):
            try:
                chunk = ctypes.string_at(ptr, n)
                if sink is not None:
                    return 0 if sink(chunk) else 1
                parts.append(chunk)
                return 0
            except Exception:
                return 1

        info = MembersInfo()
        info.size = ctypes.sizeof(MembersInfo)
        st = Stats()
        buf = bytes(data)
        with self._lock:
            rc = self.lib.gi_inflate_members(self.ctx, buf, len(buf), SINK(_cb), None, ctypes.byref(info),
                                             ctypes.byref(st))
            if rc != GI_OK:
                raise self._error(rc)
        return (b"".join(parts) if sink is None else None), info.as_dict(), st

    def inflate_zip(self, data, stop_after=None):
        """Every entry of the ZIP archive `data` (gi_inflate_zip). Returns (list of dicts in
        directory order: index, name, method, flags, status, out_size, crc32, output (bytes, or
        None when not decoded), Stats). stop_after: the sink stops after this many calls."""
        entries = {}
        calls = [0]

        def _cb(user, ep, name, data_ptr, n):
            e = ep.contents
            d = entries.setdefault(e.index, {"index": e.index, "name": ctypes.string_at(name, e.name_len).decode("utf-8", "replace"),
                                             "method": e.method, "flags": e.flags, "out_size": e.out_size,
                                             "crc32": e.crc32, "output": None})
            d["status"] = e.status
            if data_ptr and n:
                d["output"] = (d["output"] or b"") + ctypes.string_at(data_ptr, n)
            elif e.status == GI_OK and d["output"] is None:
                d["output"] = b""
            calls[0] += 1
            return 1 if stop_after is not None and calls[0] >= stop_after else 0

        st = Stats()
        buf = bytes(data)
        with self._lock:
            rc = self.lib.gi_inflate_zip(self.ctx, buf, len(buf), ENTRY_SINK(_cb), None, ctypes.byref(st))
            if rc != GI_OK:
                raise self._error(rc)
        return [entries[k] for k in sorted(entries)], st

    def inflate_device(self, d_in, in_size, d_out, out_cap):
        """Device-resident form: pointers (ints) to GPU memory. Returns (out_size, Stats)."""
        st = Stats()
        n = ctypes.c_uint64(0)
        with self._lock:
            rc = self.lib.gi_inflate_device(self.ctx, ctypes.c_void_p(d_in), in_size, ctypes.c_void_p(d_out), out_cap,
                                            ctypes.byref(n), ctypes.byref(st))
            if rc != GI_OK:
                raise self._error(rc)
        return n.value, st

    def inflate_batch(self, streams, out_cap=None, out=None):
        """Decodes many streams together (gi_inflate_batch). streams: list of bytes (raw Deflate), or
        of (bytes, flags[, expected_crc]). Returns (list of dicts with output/status/crc32/in_used,
        Stats). `out` may be a preallocated writable buffer (e.g. pinned); else one is made."""
        n = len(streams)
        arr = (Stream * max(1, n))()
        keep = []
        total_in = 0
        guess = 0  # output room: a gzip member's ISIZE, else 8 bytes per input byte
        for i, sdesc in enumerate(streams):
            data, flags, crc = (sdesc, 0, 0) if isinstance(sdesc, (bytes, bytearray, memoryview)) else (
                tuple(sdesc) + (0,) * (3 - len(sdesc)))
            b = ctypes.create_string_buffer(bytes(data), len(data)) if len(data) else ctypes.create_string_buffer(1)
            keep.append(b)
            arr[i].in_ = ctypes.cast(b, ctypes.c_void_p)
            arr[i].in_size = len(data)
            arr[i].flags = flags
            arr[i].expected_crc = crc & 0xFFFFFFFF
            total_in += len(data)
            isize = int.from_bytes(bytes(data[-4:]), "little") if (flags & GI_STREAM_GZIP) and len(data) >= 18 else -1
            guess += isize if 0 <= isize <= 1032 * len(data) and isize > 8 * len(data) else 8 * len(data)
        if out is None:
            out_cap = out_cap if out_cap is not None else max(1 << 20, guess + 64 * n + (16 << 20))
            outbuf = ctypes.create_string_buffer(out_cap)
            out_ptr = ctypes.cast(outbuf, ctypes.c_void_p)
        else:
            outbuf = out
            out_cap = len(out) if out_cap is None else out_cap
            out_ptr = ctypes.c_void_p(ctypes.addressof(ctypes.c_char.from_buffer(out)))
        st = Stats()
        with self._lock:
            rc = self.lib.gi_inflate_batch(self.ctx, arr, n, out_ptr, out_cap, ctypes.byref(st))
            if rc != GI_OK:
                raise self._error(rc)
        res = []
        view = memoryview(outbuf) if out is not None else None
        for i in range(n):
            a = arr[i]
            d = {"status": a.status, "out_size": a.out_size, "in_used": a.in_used, "crc32": a.crc32,
                 "out_offset": a.out_offset}
            if a.status == GI_OK:
                if view is not None:
                    d["output"] = bytes(view[a.out_offset:a.out_offset + a.out_size])
                else:
                    d["output"] = ctypes.string_at(ctypes.addressof(outbuf) + a.out_offset, a.out_size)
            res.append(d)
        return res, st

    def last_profile(self):
        p = Profile()
        p.size = ctypes.sizeof(Profile)
        rc = self.lib.gi_last_profile(self.ctx, ctypes.byref(p))
        if rc != GI_OK:
            raise InflateError(rc, "profile")
        return p

    def tar_index_device(self, d_tar, size):
        """gi_tar_index_device: the entries of the tar archive at device pointer d_tar (size
        bytes), as dicts (name, header, offset, size, type), and the bytes the archive took."""
        t = ctypes.c_void_p()
        rc = self.lib.gi_tar_index_device(self.ctx, ctypes.c_void_p(d_tar), size, ctypes.byref(t))
        if rc != GI_OK:
            raise InflateError(rc, self.lib.gi_last_error(self.ctx).decode(errors="replace"))
        try:
            ep = ctypes.POINTER(TarEntry)()
            n = self.lib.gi_tar_entries(t, ctypes.byref(ep))
            out = [{"name": ep[i].name.decode("utf-8", "surrogateescape"), "header": ep[i].header,
                    "offset": ep[i].offset, "size": ep[i].size, "type": ep[i].type} for i in range(n)]
            return out, self.lib.gi_tar_end(t)
        finally:
            self.lib.gi_tar_free(t)

    def last_crc32(self):
        return self.lib.gi_last_crc32(self.ctx)

    def last_isize(self):
        return self.lib.gi_last_isize(self.ctx)


def crc32_device_noalloc(d_data, size, d_crc, device=0, stream=None):
    """CRC-32 of `size` bytes at device pointer d_data into the uint32 at device pointer d_crc,
    through the entry point that allocates nothing (gi_crc32_device_noalloc). Asynchronous on
    `stream` (a raw cudaStream_t value, or None for the default stream)."""
    lib = load()
    err = ctypes.create_string_buffer(256)
    rc = lib.gi_crc32_device_noalloc(device, ctypes.c_void_p(d_data), size, ctypes.c_void_p(d_crc),
                                     ctypes.c_void_p(stream) if stream else None, err, 256)
    if rc != GI_OK:
        raise InflateError(rc, err.value.decode(errors="replace"))


class Server:
    """The request server (gi_server_*): requests are admitted into a device arena against an HBM
    budget and decoded in passes of the batched form by `workers` loops whose passes overlap on
    the GPU. Every finished request lands in ``results[tag]`` (a dict of gi_result's fields, plus
    ``output`` when keep_output); on_done(result, data_ptr) is also called, from a server thread,
    with the output valid only during that call."""

    def __init__(self, device=0, workers=0, max_batch=0, pass_out_mb=0, hbm_budget=0, arena_bytes=0,
                 keep_output=False, on_done=None, path=None, rescue_workers=0):
        self.lib = load(path)
        self.results = {}
        self._inputs = {}
        self._flags = {}
        self._lock = threading.Lock()
        self._next = 0

        def _cb(user, rp, data):
            r = rp.contents
            d = r.as_dict()
            with self._lock:
                rescued = self._flags.pop(r.tag, 0) & GI_REQ_RESCUE
            if keep_output and data and r.status == GI_OK:
                d["output"] = ctypes.string_at(data, r.out_size)
                if rescued:  # the mask follows the output
                    d["mask"] = ctypes.string_at(data + r.out_size, r.out_size)
            if on_done is not None:
                try:
                    on_done(d, data)
                except Exception:
                    pass
            with self._lock:
                self._inputs.pop(r.tag, None)
                self.results[r.tag] = d

        self._cb = DONE(_cb)
        cfg = ServerConfig(ctypes.sizeof(ServerConfig), device, workers, max_batch, pass_out_mb, rescue_workers,
                           int(hbm_budget), int(arena_bytes))
        srv = ctypes.c_void_p()
        err = ctypes.create_string_buffer(512)
        rc = self.lib.gi_server_create(ctypes.byref(cfg), self._cb, None, ctypes.byref(srv), err, 512)
        if rc != GI_OK:
            raise InflateError(rc, f"server: {err.value.decode(errors='replace')}")
        self.srv = srv

    def submit(self, data, flags=GI_STREAM_GZIP, expected_crc=0, tag=None):
        """Queues one request: bytes, or (host pointer, size) of memory the caller keeps alive until
        its result arrives. Returns its tag."""
        if isinstance(data, tuple):
            ptr, size = data
            keep = None
        else:
            keep = data if isinstance(data, bytes) else bytes(data)
            ptr = ctypes.cast(ctypes.c_char_p(keep), ctypes.c_void_p).value
            size = len(keep)
        with self._lock:
            if tag is None:
                tag = self._next
            self._next = max(self._next, tag) + 1
            self._inputs[tag] = keep
            self._flags[tag] = flags
        rc = self.lib.gi_server_submit(self.srv, ctypes.c_void_p(ptr), size, flags, expected_crc & 0xFFFFFFFF, tag)
        if rc != GI_OK:
            with self._lock:
                self._inputs.pop(tag, None)
            raise InflateError(rc, "submit refused")
        return tag

    def drain(self):
        self.lib.gi_server_drain(self.srv)

    def clock(self):
        """Seconds on the server's clock (the clock of every result's t_* fields)."""
        return self.lib.gi_server_clock(self.srv)

    def stats(self):
        st = ServerStats()
        st.size = ctypes.sizeof(ServerStats)
        rc = self.lib.gi_server_read_stats(self.srv, ctypes.byref(st))
        if rc != GI_OK:
            raise InflateError(rc, "stats")
        return st.as_dict()

    def close(self):
        if self.srv:
            self.lib.gi_server_destroy(self.srv)
            self.srv = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
