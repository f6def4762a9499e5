"""CPU: the seeded workload generators."""
import zlib

from gpuzip_gb300 import workloads as W


def test_log_text_shape_and_determinism():
    a = W.log_text(1, 200_000)
    assert a == W.log_text(1, 200_000)
    assert a.endswith(b"\n") and len(a) >= 200_000
    line = a.split(b"\n")[0].split(b" ")
    assert len(line[0]) == 10 and line[0][4:5] == b"-" and len(line[1]) == 8
    assert line[2] in (b"INFO", b"WARN", b"ERROR", b"DEBUG")
    assert 5 <= len(line) - 3 <= 25
    assert all(3 <= len(w) <= 12 and w.isalpha() and w.islower() for w in line[3:])


def test_mixed_member_is_one_valid_gzip_member():
    member, info = W.mixed_member(seed=2, nseg=6, seg_bytes=1 << 16, workers=1, want_raw=True)
    d = zlib.decompressobj(31)
    out = d.decompress(member)
    assert d.eof and not d.unused_data
    assert out == info["raw"] and len(out) == 6 << 16
    assert zlib.crc32(out) == info["crc"]


def test_crc32_combine_matches_zlib():
    a, b = b"x" * 1000 + bytes(range(256)), b"hello" * 333
    assert W.crc32_combine(zlib.crc32(a), zlib.crc32(b), len(b)) == zlib.crc32(a + b)
    assert W.crc32_combine(zlib.crc32(a), 0, 0) == zlib.crc32(a)


def test_mutations_are_deterministic():
    s = W.raw_deflate(W.log_text(2, 50_000), 6)
    r1, r2 = W.SplitMix64(5), W.SplitMix64(5)
    assert [W.mutate(s, r1) for _ in range(5)] == [W.mutate(s, r2) for _ in range(5)]
