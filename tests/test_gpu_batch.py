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


def test_batch_long_streams_scan_their_windows_in_groups(gpu):
    # streams of 16 spans (8 MiB) and more take the grouped window scan; shorter ones the walk
    items, wants = [], []
    for i, n in enumerate((8 << 20, (8 << 20) + 12345, 21 << 20, 300_000, 35 << 20, 5000)):
        text = W.log_text(70 + i, n, exact=True)
        wants.append(text)
        items.append((W.gzip_wrap(W.raw_deflate(text, [1, 6, 9][i % 3]), zlib.crc32(text), len(text)),
                      gpuinflate.GI_STREAM_GZIP))
    member, info = W.mixed_member(seed=8, nseg=24, seg_bytes=1 << 20, want_raw=False)
    items.append((member, gpuinflate.GI_STREAM_GZIP))
    wants.append(zlib.decompress(member, 31))
    res, st = gpu.inflate_batch(items)
    for i, (r, want) in enumerate(zip(res, wants)):
        assert r["status"] == 0, i
        assert r["out_size"] == len(want), i
        assert r["output"] == want, i
        assert r["crc32"] == zlib.crc32(want)


def test_batch_high_ratio_members_in_one_pass(gpu):
    # outputs hundreds of times their input: decoders sized from each member's ISIZE
    items, wants = [], []
    for i in range(6):
        pat = bytes((i * 37 + k) & 255 for k in range(8 + 8 * i))
        data = pat * ((24 << 20) // len(pat))
        wants.append(data)
        items.append((W.gzip_wrap(W.raw_deflate(data, 9), zlib.crc32(data), len(data)), gpuinflate.GI_STREAM_GZIP))
    res, st = gpu.inflate_batch(items)
    for i, (r, want) in enumerate(zip(res, wants)):
        assert r["status"] == 0 and r["output"] == want, i
    assert st.segments == 1


def test_batch_mapped_inputs_are_gathered(gpu):
    # streams in page-locked host memory (GI_STREAM_MAPPED): read by the gather kernel, at offsets of
    # every alignment, mixed with ordinary host streams
    import ctypes

    import torch

    texts = [W.log_text(90 + i, n, exact=True) for i, n in enumerate((1, 777, 70_000, 300_001, 1_000_003))]
    members = [W.gzip_wrap(W.raw_deflate(t, 6), zlib.crc32(t), len(t)) for t in texts]
    pinned = torch.empty(sum(len(m) + 64 for m in members), dtype=torch.uint8).pin_memory()
    view = pinned.numpy()
    arr = (gpuinflate.Stream * (2 * len(members)))()
    import numpy as np

    pos, keep = 16, []  # the first at a 16-byte boundary, the others at odd offsets
    for i, m in enumerate(members):
        view[pos:pos + len(m)] = np.frombuffer(m, dtype=np.uint8)
        arr[i].in_ = ctypes.c_void_p(pinned.data_ptr() + pos)
        arr[i].in_size = len(m)
        arr[i].flags = gpuinflate.GI_STREAM_GZIP | gpuinflate.GI_STREAM_MAPPED
        pos += len(m) + 1 + i  # every alignment case
        b = ctypes.create_string_buffer(m, len(m))
        keep.append(b)
        j = len(members) + i
        arr[j].in_ = ctypes.cast(b, ctypes.c_void_p)
        arr[j].in_size = len(m)
        arr[j].flags = gpuinflate.GI_STREAM_GZIP
    total = 2 * sum(len(t) for t in texts) + 16 * 64 + (1 << 20)
    out = ctypes.create_string_buffer(total)
    st = gpuinflate.Stats()
    rc = gpu.lib.gi_inflate_batch(gpu.ctx, arr, len(arr), ctypes.cast(out, ctypes.c_void_p), total, ctypes.byref(st))
    assert rc == 0
    for k in range(len(arr)):
        want = texts[k % len(texts)]
        a = arr[k]
        assert a.status == 0, k
        assert ctypes.string_at(ctypes.addressof(out) + a.out_offset, a.out_size) == want, k
        assert a.crc32 == zlib.crc32(want)
