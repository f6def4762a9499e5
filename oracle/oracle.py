"""ctypes bindings for the CPU oracle (liboracle.so) and, where it was built, the reference's own
host decoder (_ref/libgi_ref.so). TEST INFRASTRUCTURE ONLY: imported by tests/, by
__graft_entry__.smoke() as the checker, and by bench.py's CPU-baseline leg. The product
(gpuzip_gb300) never imports this module.
"""
import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OK, DATA, TRUNCATED, TOO_BIG = 0, 1, 2, 7

_lib = None
_ref = None


TREE_NOTE = os.path.join(HERE, "_ref", "TREE")  # where build() last found the reference tree


def reference_tree():
    """The reference source tree: GI_REFERENCE_DIR, else the tree build() last built _ref/ from,
    else None. Only where that tree exists are the reference's own files compared or built."""
    env = os.environ.get("GI_REFERENCE_DIR")
    if env:
        return env
    try:
        with open(TREE_NOTE) as f:
            return f.read().strip() or None
    except OSError:
        return None


def build(reference_dir=None):
    """Builds liboracle.so (always) and, when `reference_dir` (or GI_REFERENCE_DIR) names a
    reference tree that exists, _ref/ from it."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    ref = reference_dir or os.environ.get("GI_REFERENCE_DIR")
    if ref and os.path.isdir(os.path.join(ref, "gpuinflate")):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref}"], check=True)
        with open(TREE_NOTE, "w") as f:
            f.write(ref)


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        _lib = ctypes.CDLL(path)
        u8p, u64, u64p = ctypes.c_char_p, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)
        _lib.oracle_inflate.argtypes = [u8p, u64, ctypes.c_void_p, u64, u64p, u64p]
        _lib.oracle_inflate.restype = ctypes.c_int
        _lib.oracle_crc32.argtypes = [ctypes.c_uint32, u8p, u64]
        _lib.oracle_crc32.restype = ctypes.c_uint32
        _lib.oracle_prefilter128.argtypes = [u64, u64]
        _lib.oracle_prefilter128.restype = ctypes.c_int
        _lib.oracle_plausible_dynamic_header.argtypes = [u8p, u64, u64]
        _lib.oracle_plausible_dynamic_header.restype = ctypes.c_int
        _lib.oracle_first_headers.argtypes = [u8p, u64, u64, u64, u64, ctypes.c_void_p, u64]
        _lib.oracle_first_headers.restype = None
        _lib.oracle_inflate_parallel.argtypes = [u8p, u64, u64, u64, ctypes.c_void_p, u64, u64p, ctypes.c_int,
                                                 ctypes.POINTER(ctypes.c_double)]
        _lib.oracle_inflate_parallel.restype = ctypes.c_int
    return _lib


def ref_lib():
    """The reference's own decoder, or None when it was not built (no reference tree)."""
    global _ref
    if _ref is None:
        path = os.path.join(HERE, "_ref", "libgi_ref.so")
        if not os.path.exists(path):
            return None
        _ref = ctypes.CDLL(path)
        u8p, u64, u64p = ctypes.c_char_p, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)
        _ref.ref_inflate.argtypes = [u8p, u64, ctypes.c_void_p, u64, u64p, u64p]
        _ref.ref_inflate.restype = ctypes.c_int
        _ref.ref_prefilter128.argtypes = [u64, u64]
        _ref.ref_prefilter128.restype = ctypes.c_int
        _ref.ref_plausible_dynamic_header.argtypes = [u8p, u64, u64]
        _ref.ref_plausible_dynamic_header.restype = ctypes.c_int
    return _ref


def _run(fn, data, max_out):
    out = ctypes.create_string_buffer(max(1, max_out))
    n = ctypes.c_uint64(0)
    used = ctypes.c_uint64(0)
    rc = fn(bytes(data), len(data), out, max_out, ctypes.byref(n), ctypes.byref(used))
    if rc == OK:
        return rc, out.raw[: n.value], used.value
    return rc, b"", 0


def inflate(data, max_out=None):
    """(status, output bytes, in_used) of the oracle's sequential decode."""
    if max_out is None:
        max_out = max(64 << 20, len(data) * 16)
    return _run(lib().oracle_inflate, data, max_out)


def ref_inflate(data, max_out=None):
    """(status, output bytes, in_used) of the reference's own host decoder."""
    r = ref_lib()
    if r is None:
        raise RuntimeError("reference decoder not built")
    if max_out is None:
        max_out = max(64 << 20, len(data) * 16)
    return _run(r.ref_inflate, data, max_out)


def inflate_parallel(data, out_cap, threads, scan_bytes=None, chunk_bytes=4096):
    """(status, output bytes, phase seconds) of the multi-threaded CPU inflate (the reference's
    speculative CPU decoder restated): the first up to out_cap bytes of output, one block start
    searched per chunk_bytes of the first scan_bytes of input (all of it by default)."""
    out = ctypes.create_string_buffer(max(1, out_cap))
    n = ctypes.c_uint64(0)
    secs = (ctypes.c_double * 3)()
    rc = lib().oracle_inflate_parallel(bytes(data), len(data), len(data) if scan_bytes is None else scan_bytes, chunk_bytes,
                                       out, out_cap, ctypes.byref(n), threads, secs)
    return rc, (out.raw[:n.value] if rc == OK else b""), list(secs)


def crc32(data, crc=0):
    return lib().oracle_crc32(crc, bytes(data), len(data))


def first_headers(data, bit_lo, bit_hi, chunk_bits):
    nchunks = max(1, (bit_hi - bit_lo + chunk_bits - 1) // chunk_bits)
    arr = (ctypes.c_uint64 * nchunks)()
    lib().oracle_first_headers(bytes(data), len(data), bit_lo, bit_hi, chunk_bits, arr, nchunks)
    return list(arr)
