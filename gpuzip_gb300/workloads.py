"""Seeded synthetic Deflate workloads (the inputs the decoder is tested and measured on).

None of the reference's datasets are reproduced: every stream here is generated from a seed.

* ``log_text`` - log lines ``YYYY-MM-DD HH:MM:SS LEVEL w1 w2 ... wn\\n`` with 5-25 words drawn
  Zipf(s=1.1) (rank r has weight r**-1.1) from a 10,000-word vocabulary of 3-12 random lowercase
  letters; LEVEL uniform over INFO/WARN/ERROR/DEBUG; the timestamp advances 0-3 s per line.
* ``single_text_member`` - 64 MiB of that text (cut at the end of the line that crosses 64 MiB)
  as one gzip member, zlib level 6, 32 KiB window.
* ``mixed_member`` - one gzip member of ``nseg`` segments of 1 MiB each, every segment one of:
  log text (p=0.50), uniform random bytes (0.20), a 4-64-byte pattern repeated with 1% of its
  bytes replaced at random (0.15), little-endian uint32 counters with small random deltas
  (0.15); each segment compressed at a level drawn from {1, 6, 9}, all inside ONE Deflate
  stream by zlib's own deflate with the level changed by deflateParams between segments (which
  ends the current block, not byte-aligned, when the match finder changes, and adds no empty
  stored block). Runs of at least 64 segments are compressed in parallel processes, each with
  the 32 KiB before it as its preset dictionary; a run ends after a segment of random bytes, whose
  last 64 KiB go through deflateParams(0) into stored blocks (what zlib writes for random bytes
  at any level), then a Z_BLOCK flush, so the run ends on a byte boundary and the next run's
  blocks follow it in place. The stream has no empty stored block or other sync marker. 4096
  segments = 4 GiB, whose gzip ISIZE wraps to 0.
* ``fuzz_streams`` - eight small raw streams of every block kind (levels 1/6/9, fixed only,
  stored only, Huffman only, mixed random/text/runs, tiny), the kinds the reference fuzzes
  (gpuinflate/make_fuzz_inputs.py); made from this module's own text.
"""
import ctypes
import ctypes.util
import multiprocessing as mp
import struct
import zlib

import numpy as np

MIB = 1 << 20
LEVELS = (b"INFO", b"WARN", b"ERROR", b"DEBUG")
T0 = 1704067200  # 2024-01-01 00:00:00 UTC

# ---------------------------------------------------------------- CRC-32 arithmetic

POLY = 0xEDB88320


def _mulmod(a, b):
    """a(x) * b(x) mod the CRC polynomial, in the reflected bit order CRC-32 uses (bit 31 = x^0)."""
    p = 0
    m = 1 << 31
    while m:
        if a & m:
            p ^= b
        b = (b >> 1) ^ POLY if b & 1 else b >> 1
        m >>= 1
    return p


_X2N = []
_p = 1 << 30  # x^1
for _ in range(64):
    _X2N.append(_p)
    _p = _mulmod(_p, _p)


def _x8n(n):
    """x^(8n) mod P"""
    p = 1 << 31
    k = 3
    while n:
        if n & 1:
            p = _mulmod(_X2N[k % 64], p)
        n >>= 1
        k += 1
    return p


def crc32_combine(crc1, crc2, len2):
    """CRC-32 of A+B from crc(A), crc(B) and len(B)."""
    return _mulmod(_x8n(len2), crc1) ^ crc2


# ---------------------------------------------------------------- log text


class _Vocab:
    def __init__(self, seed):
        rng = np.random.default_rng([seed, 7_000_001])
        self.lens = rng.integers(3, 13, size=10000)
        self.chars = rng.integers(97, 123, size=int(self.lens.sum()), dtype=np.uint8)
        self.offs = np.concatenate([[0], np.cumsum(self.lens)[:-1]])
        w = np.arange(1, 10001, dtype=np.float64) ** -1.1
        c = np.cumsum(w)
        self.cdf = c / c[-1]


_VOCABS = {}


def _vocab(seed):
    if seed not in _VOCABS:
        _VOCABS[seed] = _Vocab(seed)
    return _VOCABS[seed]


def _lines(rng, voc, nlines, t_start):
    """nlines log lines as one uint8 array, and the next timestamp."""
    nw = rng.integers(5, 26, size=nlines)
    dt = rng.integers(0, 4, size=nlines)
    t = t_start + np.cumsum(dt) - dt[0]
    lev = rng.integers(0, 4, size=nlines)
    ids = np.searchsorted(voc.cdf, rng.random(int(nw.sum())), side="right")
    ids = np.minimum(ids, 9999)
    wl = voc.lens[ids]
    lev_len = np.array([len(x) for x in LEVELS])[lev]
    hdr = 20 + lev_len + 1  # "YYYY-MM-DD HH:MM:SS " + LEVEL + " "
    body = np.add.reduceat(wl + 1, np.concatenate([[0], np.cumsum(nw)[:-1]]))
    line_len = hdr + body
    ls = np.concatenate([[0], np.cumsum(line_len)[:-1]])
    total = int(line_len.sum())
    out = np.empty(total, dtype=np.uint8)
    ts = np.datetime_as_string(t.astype("datetime64[s]")).astype("S19")
    tsb = np.frombuffer(ts.tobytes(), dtype=np.uint8).reshape(nlines, 19).copy()
    tsb[:, 10] = ord(" ")
    out[ls[:, None] + np.arange(19)] = tsb
    out[ls + 19] = ord(" ")
    for k, name in enumerate(LEVELS):
        sel = ls[lev == k]
        if len(sel):
            out[sel[:, None] + 20 + np.arange(len(name))] = np.frombuffer(name, dtype=np.uint8)
            out[sel + 20 + len(name)] = ord(" ")
    # words: position of each word in its line's body
    line_of_word = np.repeat(np.arange(nlines), nw)
    cw = np.concatenate([[0], np.cumsum(wl + 1)[:-1]])
    first_word = np.concatenate([[0], np.cumsum(nw)[:-1]])
    wpos = ls[line_of_word] + hdr[line_of_word] + (cw - cw[first_word][line_of_word])
    nchar = int(wl.sum())
    within = np.arange(nchar) - np.repeat(np.concatenate([[0], np.cumsum(wl)[:-1]]), wl)
    out[np.repeat(wpos, wl) + within] = voc.chars[np.repeat(voc.offs[ids], wl) + within]
    sep = np.full(len(ids), ord(" "), dtype=np.uint8)
    sep[np.cumsum(nw) - 1] = ord("\n")
    out[wpos + wl] = sep
    return out, int(t[-1]) + int(rng.integers(0, 4))


def log_text(seed, nbytes, exact=False, t_start=T0, vocab_seed=None):
    """At least nbytes of log text, cut at the end of the line that crosses nbytes (or exactly
    nbytes when exact)."""
    voc = _vocab(seed if vocab_seed is None else vocab_seed)
    rng = np.random.default_rng(seed)
    parts, have, t = [], 0, t_start
    while have < nbytes:
        need = nbytes - have
        n = max(64, min(200_000, need // 100 + 16))
        arr, t = _lines(rng, voc, n, t)
        parts.append(arr)
        have += len(arr)
    text = np.concatenate(parts)
    if exact:
        return text[:nbytes].tobytes()
    end = int(np.argmax(text[nbytes - 1 :] == ord("\n"))) + nbytes if have > nbytes else have
    return text[:end].tobytes()


# ---------------------------------------------------------------- containers


def gzip_wrap(deflated, crc, isize, mtime=0):
    return b"\x1f\x8b\x08\x00" + struct.pack("<I", mtime) + b"\x00\xff" + deflated + struct.pack("<II", crc, isize & 0xFFFFFFFF)


def raw_deflate(data, level=6, strategy=zlib.Z_DEFAULT_STRATEGY, zdict=None, final=True):
    kw = {"zdict": zdict} if zdict else {}
    c = zlib.compressobj(level, zlib.DEFLATED, -15, 9, strategy, **kw)
    return c.compress(data) + c.flush(zlib.Z_FINISH if final else zlib.Z_SYNC_FLUSH)


def single_text_member(seed=1, nbytes=64 * MIB):
    """(gzip member, text): the single-member log-text workload."""
    text = log_text(seed, nbytes)
    body = raw_deflate(text, 6)
    return gzip_wrap(body, zlib.crc32(text), len(text)), text


# ---------------------------------------------------------------- mixed content

KIND_TEXT, KIND_RANDOM, KIND_PATTERN, KIND_COUNTER = 0, 1, 2, 3


def mixed_plan(seed, nseg):
    """(kinds, levels) of every segment."""
    rng = np.random.default_rng([seed, 1])
    kinds = rng.choice(4, size=nseg, p=[0.5, 0.2, 0.15, 0.15])
    levels = rng.choice(np.array([1, 6, 9]), size=nseg)
    return kinds, levels


def mixed_segment(seed, index, kind, seg_bytes=MIB):
    """The content of segment `index` of the mixed workload (exactly seg_bytes)."""
    rng = np.random.default_rng([seed, 2, index])
    if kind == KIND_TEXT:
        return log_text(int(rng.integers(1 << 62)), seg_bytes, exact=True, t_start=T0 + 3600 * index, vocab_seed=seed)
    if kind == KIND_RANDOM:
        return rng.integers(0, 256, size=seg_bytes, dtype=np.uint8).tobytes()
    if kind == KIND_PATTERN:
        p = int(rng.integers(4, 65))
        pat = rng.integers(0, 256, size=p, dtype=np.uint8)
        a = np.tile(pat, seg_bytes // p + 1)[:seg_bytes]
        nflip = seg_bytes // 100
        a[rng.integers(0, seg_bytes, size=nflip)] = rng.integers(0, 256, size=nflip, dtype=np.uint8)
        return a.tobytes()
    start = int(rng.integers(0, 1 << 32))
    deltas = rng.integers(0, 16, size=seg_bytes // 4, dtype=np.uint64)
    vals = (start + np.cumsum(deltas)) & 0xFFFFFFFF
    return vals.astype("<u4").tobytes()


class _ZStream(ctypes.Structure):
    """zlib's z_stream as its shared library lays it out (LP64: uLong is 64 bits)."""

    _fields_ = [("next_in", ctypes.c_void_p), ("avail_in", ctypes.c_uint), ("total_in", ctypes.c_ulong),
                ("next_out", ctypes.c_void_p), ("avail_out", ctypes.c_uint), ("total_out", ctypes.c_ulong),
                ("msg", ctypes.c_char_p), ("state", ctypes.c_void_p), ("zalloc", ctypes.c_void_p),
                ("zfree", ctypes.c_void_p), ("opaque", ctypes.c_void_p), ("data_type", ctypes.c_int),
                ("adler", ctypes.c_ulong), ("reserved", ctypes.c_ulong)]


_Z = None
Z_NO_FLUSH, Z_BLOCK_FLUSH, Z_FINISH_FLUSH = 0, 5, 4


def _libz():
    global _Z
    if _Z is None:
        z = ctypes.CDLL(ctypes.util.find_library("z") or "libz.so.1")
        p = ctypes.POINTER(_ZStream)
        z.zlibVersion.restype = ctypes.c_char_p
        z.deflateInit2_.argtypes = [p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_char_p, ctypes.c_int]
        z.deflate.argtypes = [p, ctypes.c_int]
        z.deflateParams.argtypes = [p, ctypes.c_int, ctypes.c_int]
        z.deflateSetDictionary.argtypes = [p, ctypes.c_char_p, ctypes.c_uint]
        z.deflatePending.argtypes = [p, ctypes.POINTER(ctypes.c_uint), ctypes.POINTER(ctypes.c_int)]
        z.deflateEnd.argtypes = [p]
        _Z = z
    return _Z


class Deflater:
    """One raw Deflate stream written by zlib's deflate through its C interface, for the calls
    Python's zlib module does not offer: deflateParams (a level change inside the stream) and
    deflatePending (the bits of the last block still held back after a Z_BLOCK flush)."""

    def __init__(self, level, zdict=None):
        self.z = _libz()
        self.s = _ZStream()
        rc = self.z.deflateInit2_(ctypes.byref(self.s), int(level), 8, -15, 9, 0, self.z.zlibVersion(),
                                  ctypes.sizeof(_ZStream))
        if rc != 0:
            raise RuntimeError(f"deflateInit2 failed: {rc}")
        self.level = int(level)
        if zdict:
            rc = self.z.deflateSetDictionary(ctypes.byref(self.s), zdict, len(zdict))
            if rc != 0:
                raise RuntimeError(f"deflateSetDictionary failed: {rc}")

    def _run(self, data, flush):
        out = []
        src = ctypes.create_string_buffer(bytes(data), max(1, len(data)))
        self.s.next_in = ctypes.cast(src, ctypes.c_void_p)
        self.s.avail_in = len(data)
        cap = len(data) + (len(data) >> 3) + (64 << 10)
        while True:
            buf = ctypes.create_string_buffer(cap)
            self.s.next_out = ctypes.cast(buf, ctypes.c_void_p)
            self.s.avail_out = cap
            rc = self.z.deflate(ctypes.byref(self.s), flush)
            if rc not in (0, 1, -5):  # Z_OK, Z_STREAM_END, Z_BUF_ERROR (no progress possible)
                raise RuntimeError(f"deflate failed: {rc}")
            out.append(buf.raw[:cap - self.s.avail_out])
            if self.s.avail_out and self.s.avail_in == 0:
                return b"".join(out)

    def write(self, data):
        return self._run(data, Z_NO_FLUSH)

    def params(self, level):
        """A level change, as deflateParams makes it (any output it flushes is returned)."""
        out = []
        while True:
            cap = 1 << 20
            buf = ctypes.create_string_buffer(cap)
            self.s.next_in, self.s.avail_in = None, 0
            self.s.next_out = ctypes.cast(buf, ctypes.c_void_p)
            self.s.avail_out = cap
            rc = self.z.deflateParams(ctypes.byref(self.s), int(level), 0)
            out.append(buf.raw[:cap - self.s.avail_out])
            if rc == 0:
                self.level = int(level)
                return b"".join(out)
            if rc != -5:
                raise RuntimeError(f"deflateParams failed: {rc}")

    def end_block(self):
        """(bytes, bits): the stream so far ended by a Z_BLOCK flush, with the 0-7 bits of its last
        byte that zlib still holds (the byte is padded with zeros)."""
        body = self._run(b"", Z_BLOCK_FLUSH)
        pend, bits = ctypes.c_uint(0), ctypes.c_int(0)
        self.z.deflatePending(ctypes.byref(self.s), ctypes.byref(pend), ctypes.byref(bits))
        if pend.value:
            raise RuntimeError("zlib holds whole bytes after a Z_BLOCK flush")
        nbits = 8 * len(body) + bits.value
        if bits.value:
            # the held bits lead the first byte the final flush writes
            tail = self._run(b"", Z_FINISH_FLUSH)
            body += bytes([tail[0] & ((1 << bits.value) - 1)])
        return body, nbits

    def finish(self):
        return self._run(b"", Z_FINISH_FLUSH)

    def close(self):
        self.z.deflateEnd(ctypes.byref(self.s))


RUN_SEGMENTS = 64  # segments per compressor process of the mixed workload (at least)


def run_bounds(kinds, nseg, every=RUN_SEGMENTS):
    """Where the mixed workload's compressor runs start: each run ends after a segment of uniform
    random bytes (whose end is written as stored blocks, so the run ends on a byte boundary and
    the next run's bits follow it in place), the first such segment once the run has at least
    `every` segments."""
    bounds, i = [0], every
    while i < nseg:
        j = i - 1
        while j < nseg - 1 and kinds[j] != KIND_RANDOM:
            j += 1
        if j >= nseg - 1:
            break
        bounds.append(j + 1)
        i = j + 1 + every
    return bounds + [nseg]


def _mixed_run(args):
    """Segments [first, last) compressed as one run of the stream: the preset dictionary is the
    32 KiB before the run, the level changes by deflateParams, and the run ends with a Z_BLOCK
    flush right after stored blocks (so on a byte boundary), or with the final block for the last
    run. (first, bytes, crc, size)."""
    seed, first, last, nseg, kinds, levels, seg_bytes = args
    zdict = mixed_segment(seed, first - 1, kinds[first - 1], seg_bytes)[-32768:] if first > 0 else None
    d = Deflater(levels[first], zdict=zdict)
    out, crc, size = [], 0, 0
    for i in range(first, last):
        if levels[i] != d.level:
            out.append(d.params(levels[i]))
        data = mixed_segment(seed, i, kinds[i], seg_bytes)
        if i == last - 1 and last < nseg:
            # the run's closing random segment: its last 64 KiB as stored blocks (level 0), as
            # zlib writes random bytes at any level, so the run ends on a byte boundary
            cut = max(0, len(data) - (64 << 10))
            out.append(d.write(data[:cut]))
            out.append(d.params(0))
            out.append(d.write(data[cut:]))
        else:
            out.append(d.write(data))
        crc = crc32_combine(crc, zlib.crc32(data), len(data))
        size += len(data)
    if last == nseg:
        out.append(d.finish())
    else:
        tail, bits = d.end_block()
        if bits % 8:
            raise RuntimeError(f"segments {first}-{last}: the run does not end on a byte boundary")
        out.append(tail)
    d.close()
    return first, b"".join(out), crc, size


def mixed_member(seed=2, nseg=4096, seg_bytes=MIB, workers=None, want_raw=False):
    """(gzip member, info) of the mixed workload. info: crc, size, kinds, levels, deflate offset,
    and the raw output when want_raw (only for small nseg)."""
    kinds, levels = mixed_plan(seed, nseg)
    kl, ll = [int(k) for k in kinds], [int(v) for v in levels]
    bounds = run_bounds(kl, nseg)
    jobs = [(seed, a, b, nseg, kl, ll, seg_bytes) for a, b in zip(bounds[:-1], bounds[1:])]
    workers = workers or min(mp.cpu_count(), 32)
    if len(jobs) > 1 and workers > 1:
        ctx = mp.get_context("spawn")
        with ctx.Pool(min(workers, len(jobs))) as pool:
            res = pool.map(_mixed_run, sorted(jobs, key=lambda j: j[1] - j[2]), chunksize=1)
    else:
        res = [_mixed_run(j) for j in jobs]
    res.sort(key=lambda r: r[0])
    crc, size = 0, 0
    for _, _, c, n in res:
        crc = crc32_combine(crc, c, n)
        size += n
    body = b"".join(r[1] for r in res)
    member = gzip_wrap(body, crc, size)
    info = {"crc": crc, "size": size, "kinds": kinds, "levels": levels, "deflate_offset": 10, "deflate_size": len(body),
            "runs": len(jobs)}
    if want_raw:
        info["raw"] = b"".join(mixed_segment(seed, i, int(kinds[i]), seg_bytes) for i in range(nseg))
    return member, info


def fuzz_streams(seed=7):
    """name -> raw Deflate stream, every block kind (small: for fuzzing and parity)."""
    text = log_text(seed, 2 * MIB)
    rng = np.random.default_rng(seed)
    mixed = bytearray()
    while len(mixed) < MIB:
        k = int(rng.integers(3))
        n = int(rng.integers(1, 40000))
        if k == 0:
            mixed += rng.integers(0, 256, size=n, dtype=np.uint8).tobytes()
        elif k == 1:
            a = int(rng.integers(len(text) - n))
            mixed += text[a : a + n]
        else:
            mixed += bytes([int(rng.integers(256))]) * n
    return {
        "f-l1": raw_deflate(text[:MIB], 1),
        "f-l6": raw_deflate(text, 6),
        "f-l9": raw_deflate(text[:MIB], 9),
        "f-fixed": raw_deflate(text[:MIB], 6, zlib.Z_FIXED),
        "f-stored": raw_deflate(text[: 512 << 10], 0),
        "f-mixed": raw_deflate(bytes(mixed), 6),
        "f-huffman": raw_deflate(text[:MIB], 6, zlib.Z_HUFFMAN_ONLY),
        "f-tiny": raw_deflate(b"hello, hello, hello world\n" * 3, 6),
    }


class SplitMix64:
    """The mutation RNG of the reference's fuzzer (gpuinflate/gi_test.cpp:99-108)."""

    def __init__(self, seed):
        self.s = seed & 0xFFFFFFFFFFFFFFFF

    def next(self):
        M = 0xFFFFFFFFFFFFFFFF
        self.s = (self.s + 0x9E3779B97F4A7C15) & M
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
        return z ^ (z >> 31)

    def below(self, n):
        return self.next() % n if n else 0


def mutate(data, rng):
    """One damaged copy of data: 1-4 of the reference fuzzer's six mutation kinds
    (gpuinflate/gi_test.cpp:197-218): bit flip (twice as likely), byte overwrite, span of
    1-64 random bytes, truncation, a copied span of up to 4096 bytes."""
    m = bytearray(data)
    for _ in range(1 + rng.below(4)):
        if not m:
            break
        k = rng.below(6)
        if k in (0, 1):
            m[rng.below(len(m))] ^= 1 << rng.below(8)
        elif k == 2:
            m[rng.below(len(m))] = rng.next() & 0xFF
        elif k == 3:
            a = rng.below(len(m))
            n = min(1 + rng.below(64), len(m) - a)
            for i in range(n):
                m[a + i] = rng.next() & 0xFF
        elif k == 4:
            del m[rng.below(len(m)) + 1 :]
        else:
            a, b = rng.below(len(m)), rng.below(len(m))
            n = min(1 + rng.below(4096), len(m) - a, len(m) - b)
            m[b : b + n] = m[a : a + n]
    return bytes(m)


# ---------------------------------------------------------------- many streams (batched, served)


def stream_content(seed, index, size, kind):
    """`size` bytes of one content kind (the mixed workload's four), seeded by (seed, index)."""
    rng = np.random.default_rng([seed, 3, index])
    if kind == KIND_TEXT:
        return log_text(int(rng.integers(1 << 62)), size, exact=True, vocab_seed=seed) if size else b""
    if kind == KIND_RANDOM:
        return rng.integers(0, 256, size=size, dtype=np.uint8).tobytes()
    if kind == KIND_PATTERN:
        p = int(rng.integers(4, 65))
        pat = rng.integers(0, 256, size=p, dtype=np.uint8)
        a = np.tile(pat, size // p + 1)[:size]
        nflip = size // 100
        if nflip:
            a[rng.integers(0, size, size=nflip)] = rng.integers(0, 256, size=nflip, dtype=np.uint8)
        return a.tobytes()
    start = int(rng.integers(0, 1 << 32))
    vals = (start + np.cumsum(rng.integers(0, 16, size=(size + 3) // 4, dtype=np.uint64))) & 0xFFFFFFFF
    return vals.astype("<u4").tobytes()[:size]


def _stream_job(args):
    seed, index, size, kind, level, gz = args
    data = stream_content(seed, index, size, kind)
    body = raw_deflate(data, int(level))
    crc = zlib.crc32(data)
    return index, (gzip_wrap(body, crc, len(data)) if gz else body), crc, len(data)


def many_streams(seed=3, n=10000, lo=1 << 10, hi=64 << 20, total=None, workers=None, all_gzip=False):
    """n independent streams: sizes log-uniform over [lo, hi] (then scaled so their sum is `total`
    bytes when given), content of one kind each (p = 0.5/0.2/0.15/0.15 as the mixed workload),
    level from {1, 6, 9}; even indices are gzip members, odd ones raw Deflate entries whose CRC-32
    is known (as a ZIP entry's), or all gzip members with all_gzip. Returns a list of dicts: data,
    gzip, crc, size."""
    rng = np.random.default_rng([seed, 4])
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), size=n))
    if total:
        sizes *= total / sizes.sum()
    sizes = np.maximum(sizes.astype(np.int64), 1)
    kinds = rng.choice(4, size=n, p=[0.5, 0.2, 0.15, 0.15])
    levels = rng.choice(np.array([1, 6, 9]), size=n)
    jobs = [(seed, i, int(sizes[i]), int(kinds[i]), int(levels[i]), all_gzip or i % 2 == 0) for i in range(n)]
    # largest first, so the pool's workers end together
    jobs.sort(key=lambda j: -j[2])
    workers = workers or min(mp.cpu_count(), 32)
    if n >= 16 and workers > 1:
        with mp.get_context("spawn").Pool(workers) as pool:
            res = pool.map(_stream_job, jobs, chunksize=1)
    else:
        res = [_stream_job(j) for j in jobs]
    res.sort(key=lambda r: r[0])
    return [{"data": d, "gzip": all_gzip or i % 2 == 0, "crc": c, "size": s} for i, d, c, s in res]


def serve_trace(seed=5, rate=200.0, seconds=60.0, npool=256, rescue_frac=0.10):
    """Arrivals of the serving workload: a Poisson process of `rate` requests per second for
    `seconds`, each request drawing one member of a pool of `npool` (uniformly), a fraction
    `rescue_frac` of them marked as rescue requests (their member arrives with one 4 KiB sector
    zeroed). Returns (arrival times in seconds, pool index per request, rescue flag per request)."""
    rng = np.random.default_rng([seed, 5])
    n_guess = int(rate * seconds * 1.5) + 64
    t = np.cumsum(rng.exponential(1.0 / rate, size=n_guess))
    while t[-1] < seconds:  # (practically never) more arrivals than the guess
        t = np.concatenate([t, t[-1] + np.cumsum(rng.exponential(1.0 / rate, size=n_guess))])
    t = t[t < seconds]
    member = rng.integers(0, npool, size=len(t))
    rescue = rng.random(len(t)) < rescue_frac
    return t, member, rescue


def zero_sector(member, seed, index):
    """A copy of gzip member `member` with one 4 KiB sector (4 KiB-aligned in the file) zeroed
    inside its compressed body (all of the body when it is shorter)."""
    b = bytearray(member)
    lo, hi = 10, max(11, len(b) - 8)
    rng = np.random.default_rng([seed, 6, index])
    first, last = lo // 4096, (hi - 1) // 4096
    sec = int(rng.integers(first, last + 1))
    a, e = max(lo, sec * 4096), min(hi, sec * 4096 + 4096)
    b[a:e] = bytes(e - a)
    return bytes(b)


def bgzf(data, block=0xFF00, level=6):
    """`data` as a BGZF file (bgzip's format): gzip members of at most `block` input bytes, each
    header carrying the "BC" extra subfield with the member's size less one, then the empty
    end-of-file member."""
    out = bytearray()
    for a in range(0, len(data) + 1, block):
        chunk = data[a:a + block]
        if not chunk and a:
            break
        body = raw_deflate(chunk, level)
        bsize = 12 + 6 + len(body) + 8  # header with XLEN, the subfield, body, trailer
        out += bytes([0x1F, 0x8B, 8, 4, 0, 0, 0, 0, 0, 0xFF, 6, 0, ord("B"), ord("C"), 2, 0])
        out += (bsize - 1).to_bytes(2, "little") + body
        out += zlib.crc32(chunk).to_bytes(4, "little") + len(chunk).to_bytes(4, "little")
    # the end-of-file marker: an empty member
    empty = raw_deflate(b"", level)
    out += bytes([0x1F, 0x8B, 8, 4, 0, 0, 0, 0, 0, 0xFF, 6, 0, ord("B"), ord("C"), 2, 0])
    out += (12 + 6 + len(empty) + 8 - 1).to_bytes(2, "little") + empty + bytes(8)
    return bytes(out)


def zip_archive(entries):
    """A ZIP archive (stored as written by a plain archiver: local headers, data, the central
    directory, the end record) of already-compressed entries: (name bytes, raw Deflate body,
    CRC-32, uncompressed size), method 8 each. Offsets and sizes must stay below 4 GiB."""
    out = bytearray()
    cd = bytearray()
    for name, body, crc, size in entries:
        off = len(out)
        out += struct.pack("<IHHHHHIIIHH", 0x04034B50, 20, 0, 8, 0, 0x21, crc, len(body), size, len(name), 0)
        out += name + body
        cd += struct.pack("<IHHHHHHIIIHHHHHII", 0x02014B50, 20, 20, 0, 8, 0, 0x21, crc, len(body), size, len(name),
                          0, 0, 0, 0, 0, off)
        cd += name
    cd_off = len(out)
    out += cd
    out += struct.pack("<IHHHHIIH", 0x06054B50, 0, 0, len(entries), len(entries), len(cd), cd_off, 0)
    return bytes(out)


# ---------------------------------------------------------------- rescue: a damaged .tar.gz


def ustar_header(name, size, mtime=T0, typeflag=b"0"):
    """A POSIX ustar header block (512 bytes): a regular file, or another type."""
    h = bytearray(512)
    nb = name.encode()[:100]
    h[0:len(nb)] = nb
    h[100:108] = b"0000644\0"
    h[108:116] = b"0001750\0"
    h[116:124] = b"0001750\0"
    h[124:136] = b"%011o\0" % size
    h[136:148] = b"%011o\0" % mtime
    h[148:156] = b" " * 8
    h[156:157] = typeflag
    h[257:263] = b"ustar\0"
    h[263:265] = b"00"
    h[148:156] = b"%06o\0 " % sum(h)
    return bytes(h)


def tar_archive(files):
    """A tar archive (ustar) of (name, bytes) or (name, bytes, "pax") entries, ended by two zero
    blocks. A name longer than 100 bytes goes in a GNU long-name entry ('L') before its header, or
    with "pax" in a pax extended header ('x') with a path record."""
    parts = []

    def add(name, data, typeflag=b"0"):
        parts.append(ustar_header(name, len(data), typeflag=typeflag))
        parts.append(data)
        parts.append(bytes(-len(data) % 512))

    for entry in files:
        name, data = entry[0], entry[1]
        if len(entry) > 2 and entry[2] == "pax":
            rec = b" path=" + name.encode() + b"\n"
            n = len(rec) + 1
            while len(str(n)) + len(rec) != n:
                n = len(str(n)) + len(rec)
            add("PaxHeaders/" + name[-80:], str(n).encode() + rec, b"x")
        elif len(name.encode()) > 100:
            add("././@LongLink", name.encode() + b"\0", b"L")
        add(name, data)
    parts.append(bytes(1024))
    return b"".join(parts)


def _file_job(args):
    seed, index, size, kind = args
    return stream_content(seed, 1_000_000 + index, size, kind)


def _seg_job(args):
    index, seg, zdict, level, final = args
    return index, raw_deflate(seg, int(level), zdict=zdict, final=final)


def rescue_tar(seed=4, nfiles=2000, lo=4 << 10, hi=8 << 20, workers=None):
    """(gzip member, info): a .tar.gz of `nfiles` files whose sizes are log-uniform over [lo, hi],
    each one content kind of the mixed workload (log text 0.50, random 0.20, pattern 0.15,
    counters 0.15), the tar stream compressed in 1 MiB segments at levels drawn from {1, 6, 9},
    all in one Deflate stream (as ``mixed_member``). info: crc, size, files [(name, offset in
    the tar, size)]."""
    rng = np.random.default_rng([seed, 11])
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), size=nfiles)).astype(np.int64)
    kinds = rng.choice(4, size=nfiles, p=[0.5, 0.2, 0.15, 0.15])
    jobs = [(seed, i, int(sizes[i]), int(kinds[i])) for i in range(nfiles)]
    workers = workers or min(mp.cpu_count(), 32)
    ctx = mp.get_context("spawn")
    with ctx.Pool(workers) as pool:
        contents = pool.map(_file_job, jobs, chunksize=8)
    names = [f"data/part{i // 100:02d}/file{i:05d}.bin" for i in range(nfiles)]
    tar = tar_archive(list(zip(names, contents)))
    files, off = [], 0
    for name, data in zip(names, contents):
        files.append((name, off + 512, len(data)))
        off += 512 + len(data) + (-len(data) % 512)
    del contents
    nseg = (len(tar) + MIB - 1) // MIB
    levels = rng.choice(np.array([1, 6, 9]), size=nseg)
    segjobs = [(i, tar[i * MIB:(i + 1) * MIB], tar[max(0, i * MIB - 32768):i * MIB] if i else None, int(levels[i]),
                i == nseg - 1) for i in range(nseg)]
    with ctx.Pool(workers) as pool:
        bodies = pool.map(_seg_job, segjobs, chunksize=4)
    bodies.sort(key=lambda r: r[0])
    crc = zlib.crc32(tar)
    member = gzip_wrap(b"".join(b for _, b in bodies), crc, len(tar))
    return member, {"crc": crc, "size": len(tar), "files": files}


def rescue_damage(member, seed=4, sectors=3, dup=64 << 10, crlf_region=16 << 20):
    """(damaged copy, what was done): `sectors` 4 KiB sectors zeroed at random 4 KiB-aligned places
    of the compressed body, one `dup`-byte span written twice (a download resumed at the wrong
    place), and every CR LF turned into LF inside one `crlf_region`-byte region."""
    rng = np.random.default_rng([seed, 12])
    b = bytearray(member)
    lo, hi = 10, len(b) - 8
    done = {"sectors": [], "dup": None, "crlf": None}
    for _ in range(sectors):
        s = int(rng.integers(lo // 4096 + 1, hi // 4096 - 1)) * 4096
        b[s:s + 4096] = bytes(4096)
        done["sectors"].append(s)
    d = int(rng.integers(lo, hi - dup))
    b[d + dup:d + dup] = b[d:d + dup]
    done["dup"] = d
    r = int(rng.integers(lo, max(lo + 1, len(b) - 8 - crlf_region)))
    region = bytes(b[r:r + crlf_region])
    fixed = region.replace(b"\r\n", b"\n")
    b[r:r + crlf_region] = fixed
    done["crlf"] = [r, len(region) - len(fixed)]
    return bytes(b), done
