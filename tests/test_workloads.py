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


def test_tar_archive_reads_with_tarfile():
    import io
    import tarfile

    files = [("a.txt", b"hello"), ("n" * 150 + "/long.txt", b"long name"), ("p/" + "q" * 120 + ".bin", b"pax", "pax"),
             ("empty", b"")]
    t = W.tar_archive(files)
    assert len(t) % 512 == 0 and t[-1024:] == bytes(1024)
    with tarfile.open(fileobj=io.BytesIO(t)) as tf:
        got = [(m.name, tf.extractfile(m).read()) for m in tf.getmembers()]
    assert got == [(f[0], f[1]) for f in files]


def test_rescue_tar_and_damage():
    import io
    import tarfile

    member, info = W.rescue_tar(seed=4, nfiles=24, lo=1 << 10, hi=64 << 10, workers=2)
    raw = zlib.decompress(member, 31)
    assert len(raw) == info["size"] and zlib.crc32(raw) == info["crc"]
    with tarfile.open(fileobj=io.BytesIO(raw)) as tf:
        ms = tf.getmembers()
    assert [(m.name, m.offset_data, m.size) for m in ms] == [tuple(f) for f in info["files"]]
    again, _ = W.rescue_tar(seed=4, nfiles=24, lo=1 << 10, hi=64 << 10, workers=1)
    assert again == member  # the same bytes whatever the workers
    damaged, done = W.rescue_damage(member, seed=4, crlf_region=1 << 16)
    assert len(damaged) == len(member) + (64 << 10) - done["crlf"][1]
    for s in done["sectors"]:
        assert s % 4096 == 0
    d2, done2 = W.rescue_damage(member, seed=4, crlf_region=1 << 16)
    assert d2 == damaged and done2 == done
