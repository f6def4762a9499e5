"""ctypes binding of the gr_* rescue interface (include/gzrescue_gb300.h).

The same interface is gzrescue's libgzrescue (gpuinflate/rescue.h, interface version 4), so
`rescue()` calls either library: libgpuinflate.so here, or a build of the reference's rescue.cpp
where a test compares the two."""
import ctypes
import os

from . import gpuinflate

GR_ABI_VERSION = 4
GR_OK, GR_ERR_NO_DEFLATE, GR_ERR_ABORTED, GR_ERR_ARG, GR_ERR_MEMORY, GR_ERR_TOO_BIG, GR_ERR_INTERNAL = range(7)
GR_UNKNOWN, GR_EXACT, GR_SUSPECT, GR_INFERRED = range(4)

EXPORTED = ("gr_abi_version", "gr_rescue", "gr_rescue_raw", "gr_result_stats", "gr_result_pieces", "gr_result_notes",
            "gr_free", "gr_last_launches", "gr_rescue_tar", "gr_tar_result_stats", "gr_tar_result_files",
            "gr_tar_result_skipped", "gr_tar_free", "gr_release_cached")
TAR_INTACT, TAR_SUSPECT, TAR_PARTIAL, TAR_INFERRED, TAR_UNVERIFIED = range(5)


class Options(ctypes.Structure):  # gpuinflate/rescue.h:45-56
    _fields_ = [("size", ctypes.c_uint32), ("fill", ctypes.c_uint8), ("no_infer", ctypes.c_uint8),
                ("cr_lost", ctypes.c_uint8), ("crs_expected", ctypes.c_uint8), ("max_output", ctypes.c_uint64),
                ("cr_budget", ctypes.c_uint64)]


class Piece(ctypes.Structure):  # gpuinflate/rescue.h:58-66
    _fields_ = [("out_offset", ctypes.c_uint64), ("length", ctypes.c_uint64), ("decoded", ctypes.c_uint64),
                ("known", ctypes.c_uint64), ("in_byte_start", ctypes.c_uint64), ("in_byte_end", ctypes.c_uint64),
                ("suspect", ctypes.c_int32), ("status", ctypes.c_int32), ("blocks", ctypes.c_uint32),
                ("symbols", ctypes.c_uint32), ("why", ctypes.c_char_p)]


class Stats(ctypes.Structure):  # gpuinflate/rescue.h:68-86
    _fields_ = [("input_size", ctypes.c_uint64), ("output_size", ctypes.c_uint64), ("exact_bytes", ctypes.c_uint64),
                ("suspect_bytes", ctypes.c_uint64), ("unknown_bytes", ctypes.c_uint64), ("headers", ctypes.c_uint32),
                ("pieces", ctypes.c_uint32), ("damaged", ctypes.c_uint32), ("members", ctypes.c_uint32),
                ("crc_check", ctypes.c_int32), ("length_off", ctypes.c_int64), ("truncated", ctypes.c_int32),
                ("header_damaged", ctypes.c_int32), ("input_end", ctypes.c_uint64), ("inferred_bytes", ctypes.c_uint64),
                ("ascii_undone", ctypes.c_int32), ("cr_restored", ctypes.c_uint32), ("cr_decoded", ctypes.c_uint64),
                ("hidden_damage", ctypes.c_int32)]


class TarStats(ctypes.Structure):  # gzrescue_gb300.h
    _fields_ = [("intact", ctypes.c_uint64), ("unverified", ctypes.c_uint64), ("repaired", ctypes.c_uint64),
                ("bytes", ctypes.c_uint64), ("files", ctypes.c_uint32), ("suspect", ctypes.c_uint32),
                ("inferred", ctypes.c_uint32), ("partial", ctypes.c_uint32), ("skipped", ctypes.c_uint32),
                ("pad", ctypes.c_uint32)]


class TarFile(ctypes.Structure):  # gzrescue_gb300.h
    _fields_ = [("name", ctypes.c_char_p), ("offset", ctypes.c_uint64), ("size", ctypes.c_uint64),
                ("status", ctypes.c_int32), ("pad", ctypes.c_int32)]


SINK = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint8), ctypes.POINTER(ctypes.c_uint8),
                        ctypes.c_size_t)

STAT_FIELDS = [f for f, _ in Stats._fields_]
PIECE_FIELDS = [f for f, _ in Piece._fields_ if f != "why"]

_libs = {}


def bind(path):
    """The gr_* functions of the library at `path`, typed."""
    if path in _libs:
        return _libs[path]
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is not built")
    lib = ctypes.CDLL(path)
    vp, u64 = ctypes.c_void_p, ctypes.c_uint64
    lib.gr_abi_version.restype = ctypes.c_uint32
    if lib.gr_abi_version() != GR_ABI_VERSION:
        raise RuntimeError(f"{path} speaks rescue interface {lib.gr_abi_version()}, expected {GR_ABI_VERSION}")
    lib.gr_rescue.argtypes = [ctypes.c_char_p, u64, ctypes.POINTER(Options), SINK, vp, ctypes.POINTER(vp)]
    lib.gr_rescue.restype = ctypes.c_int
    lib.gr_rescue_raw.argtypes = [ctypes.c_char_p, u64, u64, ctypes.c_int, ctypes.c_uint32, ctypes.POINTER(Options), SINK,
                                  vp, ctypes.POINTER(vp)]
    lib.gr_rescue_raw.restype = ctypes.c_int
    lib.gr_result_stats.argtypes = [vp]
    lib.gr_result_stats.restype = ctypes.POINTER(Stats)
    lib.gr_result_pieces.argtypes = [vp, ctypes.POINTER(ctypes.POINTER(Piece))]
    lib.gr_result_pieces.restype = ctypes.c_uint32
    lib.gr_result_notes.argtypes = [vp, ctypes.POINTER(ctypes.POINTER(ctypes.c_char_p))]
    lib.gr_result_notes.restype = ctypes.c_uint32
    lib.gr_free.argtypes = [vp]
    lib.gr_free.restype = None
    if hasattr(lib, "gr_last_launches"):
        lib.gr_last_launches.restype = ctypes.c_uint64
    if hasattr(lib, "gr_release_cached"):
        lib.gr_release_cached.argtypes = []
        lib.gr_release_cached.restype = None
    if hasattr(lib, "gr_rescue_tar"):
        lib.gr_rescue_tar.argtypes = [ctypes.c_char_p, u64, ctypes.POINTER(Options), SINK, vp, ctypes.POINTER(vp),
                                      ctypes.POINTER(vp)]
        lib.gr_rescue_tar.restype = ctypes.c_int
        lib.gr_tar_result_stats.argtypes = [vp]
        lib.gr_tar_result_stats.restype = ctypes.POINTER(TarStats)
        lib.gr_tar_result_files.argtypes = [vp, ctypes.POINTER(ctypes.POINTER(TarFile))]
        lib.gr_tar_result_files.restype = ctypes.c_uint32
        lib.gr_tar_result_skipped.argtypes = [vp, ctypes.POINTER(ctypes.POINTER(u64))]
        lib.gr_tar_result_skipped.restype = ctypes.c_uint32
        lib.gr_tar_free.argtypes = [vp]
        lib.gr_tar_free.restype = None
    _libs[path] = lib
    return lib


def rescue(data, raw=False, expected_size=None, expected_crc=None, fill=0, no_infer=False, cr_lost=0, max_output=0,
           lib_path=None, keep_output=True, crs_expected=0, cr_budget=0):
    """Rescues gzip (or, raw=True, raw Deflate) bytes; returns a dict with rc, data, mask, stats,
    pieces and notes (data and mask empty when keep_output is False). cr_lost, crs_expected and
    cr_budget are gr_options' fields of those names (the search for CRs a raw stream lost)."""
    lib = bind(lib_path or gpuinflate.LIB_PATH)
    out, mask = bytearray(), bytearray()
    calls = [0, 0]

    def sink(_user, d, m, n):
        calls[0] += 1
        calls[1] = max(calls[1], n)
        if keep_output:
            out.extend(ctypes.string_at(d, n))
            mask.extend(ctypes.string_at(m, n))
        return 0

    cb = SINK(sink)
    opt = Options(ctypes.sizeof(Options), fill, 1 if no_infer else 0, cr_lost, crs_expected, max_output, cr_budget)
    res = ctypes.c_void_p()
    if raw:
        size = 0xFFFFFFFFFFFFFFFF if expected_size is None else expected_size
        rc = lib.gr_rescue_raw(bytes(data), len(data), size, 0 if expected_crc is None else 1, expected_crc or 0,
                               ctypes.byref(opt), cb, None, ctypes.byref(res))
    else:
        rc = lib.gr_rescue(bytes(data), len(data), ctypes.byref(opt), cb, None, ctypes.byref(res))
    r = {"rc": rc, "data": bytes(out), "mask": bytes(mask), "stats": None, "pieces": [], "notes": [],
         "sink_calls": calls[0], "largest_chunk": calls[1]}
    if res.value:
        st = lib.gr_result_stats(res).contents
        r["stats"] = {f: getattr(st, f) for f in STAT_FIELDS}
        pp = ctypes.POINTER(Piece)()
        n = lib.gr_result_pieces(res, ctypes.byref(pp))
        for i in range(n):
            p = pp[i]
            d = {f: getattr(p, f) for f in PIECE_FIELDS}
            d["why"] = (p.why or b"").decode("utf-8", "replace")
            r["pieces"].append(d)
        nn = ctypes.POINTER(ctypes.c_char_p)()
        k = lib.gr_result_notes(res, ctypes.byref(nn))
        r["notes"] = [nn[i].decode("utf-8", "replace") for i in range(k)]
        lib.gr_free(res)
    return r


def rescue_tar(data, fill=0, no_infer=False, lib_path=None):
    """gr_rescue_tar: the rescue (no sink) and the tar walk on the GPU. Returns rc, the rescue's
    stats, and the file list as the oracle of the reader gives it: intact (count), unverified
    (count), suspect / inferred / partial (names in archive order), skipped [(offset, bytes)],
    repaired and bytes, plus every file with its status."""
    lib = bind(lib_path or gpuinflate.LIB_PATH)
    opt = Options(ctypes.sizeof(Options), fill, 1 if no_infer else 0, 0, 0, 0, 0)
    res, tar = ctypes.c_void_p(), ctypes.c_void_p()
    rc = lib.gr_rescue_tar(bytes(data), len(data), ctypes.byref(opt), SINK(), None, ctypes.byref(res), ctypes.byref(tar))
    out = {"rc": rc, "stats": None, "tar": None}
    if res.value:
        st = lib.gr_result_stats(res).contents
        out["stats"] = {f: getattr(st, f) for f in STAT_FIELDS}
        lib.gr_free(res)
    if tar.value:
        ts = lib.gr_tar_result_stats(tar).contents
        fp = ctypes.POINTER(TarFile)()
        n = lib.gr_tar_result_files(tar, ctypes.byref(fp))
        files = [(fp[i].name.decode("utf-8", "replace"), fp[i].offset, fp[i].size, fp[i].status) for i in range(n)]
        sp = ctypes.POINTER(ctypes.c_uint64)()
        k = lib.gr_tar_result_skipped(tar, ctypes.byref(sp))
        skipped = [[sp[2 * i], sp[2 * i + 1]] for i in range(k)]
        out["tar"] = {
            "intact": ts.intact, "unverified": ts.unverified,
            "suspect": [f[0] for f in files if f[3] == TAR_SUSPECT],
            "inferred": [f[0] for f in files if f[3] == TAR_INFERRED],
            "partial": [f[0] for f in files if f[3] == TAR_PARTIAL],
            "skipped": skipped, "repaired": ts.repaired, "bytes": ts.bytes, "files": files,
        }
        lib.gr_tar_free(tar)
    return out
