"""GPU: the batched form (gi_inflate_batch) against zlib and the oracle: many streams of every
kind and size in one call, each with its own bytes, in_used, GPU CRC-32 and error class."""
import zlib

import pytest

import oracle
from gpuzip_gb300 import gpuinflate
from gpuzip_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _streams():
    fz = W.fuzz_streams()
    out = []
    for k, s in fz.items():
        out.append(s)
    text = W.log_text(31, 3 << 20)
    out.append(W.raw_deflate(text, 6))
    member, info = W.mixed_member(seed=5, nseg=6, seg_bytes=1 << 20, want_raw=False)
    out.append(member[10:])
    for n in (1, 100, 5000, 70000, 300000):
        out.append(W.raw_deflate(W.log_text(40 + n, n)[:n], [1, 6, 9][n % 3]))
    return out


def test_batch_matches_zlib(gpu):
    streams = _streams()
    res, st = gpu.inflate_batch(streams)
    for s, r in zip(streams, res):
        d = zlib.decompressobj(-15)
        want = d.decompress(s)
        assert r["status"] == 0
        assert r["output"] == want
        assert r["in_used"] == len(s) - len(d.unused_data)
        assert r["crc32"] == zlib.crc32(want)
        assert r["out_offset"] % 16 == 0


def test_batch_gzip_members_and_zip_entries(gpu):
    items, wants = [], []
    for i, n in enumerate((10, 4096, 200_000, 2_500_000)):
        text = W.log_text(50 + i, n)
        wants.append(text)
        if i % 2:
            items.append((W.gzip_wrap(W.raw_deflate(text, 6), zlib.crc32(text), len(text)) + b"tail",
                          gpuinflate.GI_STREAM_GZIP))
        else:
            items.append((W.raw_deflate(text, 9), gpuinflate.GI_STREAM_CRC, zlib.crc32(text)))
    bad_crc = (W.raw_deflate(wants[0], 6), gpuinflate.GI_STREAM_CRC, zlib.crc32(wants[0]) ^ 1)
    bad_member = W.gzip_wrap(W.raw_deflate(wants[1], 6), zlib.crc32(wants[1]) ^ 4, len(wants[1]))
    res, _ = gpu.inflate_batch(items + [bad_crc, (bad_member, gpuinflate.GI_STREAM_GZIP)])
    for i, (r, want) in enumerate(zip(res, wants)):
        assert r["status"] == 0, i
        assert r["output"] == want
        if i % 2:
            assert r["in_used"] == len(items[i][0]) - 4
    assert res[4]["status"] == gpuinflate.GI_ERR_DATA
    assert res[5]["status"] == gpuinflate.GI_ERR_DATA


def test_batch_error_classes_match_the_oracle(gpu):
    rng = W.SplitMix64(77)
    base = list(W.fuzz_streams().values())
    streams = [W.mutate(base[i % len(base)], rng) for i in range(120)]
    res, _ = gpu.inflate_batch(streams)
    bad = []
    for i, (s, r) in enumerate(zip(streams, res)):
        rc, out, used = oracle.inflate(s, 64 << 20)
        if rc == oracle.TOO_BIG:
            continue
        if rc != 0:
            ok = r["status"] == rc
        else:
            ok = r["status"] == 0 and r["output"] == out and r["in_used"] == used
        if not ok:
            bad.append((i, rc, r["status"], len(out), r["out_size"]))
    assert not bad, bad[:8]


def test_batch_many_small_streams(gpu):
    streams = [W.raw_deflate(W.log_text(1000 + i, 200 + 37 * i), 6) for i in range(3000)]
    res, st = gpu.inflate_batch(streams)
    assert all(r["status"] == 0 for r in res)
    for i in range(0, 3000, 97):
        assert res[i]["output"] == zlib.decompressobj(-15).decompress(streams[i])
    assert st.segments <= 2  # one pass of the GPU pipeline for all of them


def test_batch_output_space(gpu):
    s = W.raw_deflate(W.log_text(9, 100_000), 6)
    res, _ = gpu.inflate_batch([s, s], out_cap=120_000)
    assert res[0]["status"] == 0
    assert res[1]["status"] == gpuinflate.GI_ERR_SPACE
