"""GPU: whole gzip files through gi_inflate_members, against Python's own multi-member gzip reader:
BGZF files (members decoded together), plain concatenations (member by member), a mix of both,
trailing zeros and garbage, header CRCs, corrupt members, a sink that stops, and no member."""
import gzip
import struct
import zlib

import pytest

from gpuzip_gb300 import gpuinflate
from gpuzip_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def member(data, level=6, fhcrc=False, bad_hcrc=False):
    if not fhcrc:
        return W.gzip_wrap(W.raw_deflate(data, level), zlib.crc32(data), len(data))
    head = bytes([0x1F, 0x8B, 8, 2, 0, 0, 0, 0, 0, 0xFF])
    hcrc = zlib.crc32(head) & 0xFFFF
    if bad_hcrc:
        hcrc ^= 1
    return head + struct.pack("<H", hcrc) + W.raw_deflate(data, level) + struct.pack("<II", zlib.crc32(data), len(data))


def test_bgzf_members_decoded_together(gpu):
    data = W.log_text(5, 6 << 20, exact=True)
    f = W.bgzf(data)
    out, info, st = gpu.inflate_members(f)
    assert out == data == gzip.decompress(f)
    assert info["members"] == info["batched"] == (len(data) + 0xFEFF) // 0xFF00 + 1
    assert info["trailing"] == 0 and st.in_used == len(f)


def test_plain_concatenation_and_trailing_bytes(gpu):
    parts = [W.log_text(10 + i, n, exact=True) for i, n in enumerate((1000, 250_000, 1, 3_000_000))]
    f = b"".join(member(p, [1, 6, 9][i % 3]) for i, p in enumerate(parts))
    for tail, zero in ((b"", 0), (bytes(100), 1), (b"not gzip" * 3, 0)):
        out, info, st = gpu.inflate_members(f + tail)
        assert out == b"".join(parts)
        assert info["members"] == len(parts) and info["batched"] == 0
        assert info["trailing"] == len(tail) and (info["trailing_zero"] == zero or not tail)
        assert st.in_used == len(f)


def test_bgzf_and_plain_members_mixed(gpu):
    a, b, c = (W.log_text(20 + i, n, exact=True) for i, n in enumerate((200_000, 70_000, 150_000)))
    f = W.bgzf(a) + member(b, fhcrc=True) + W.bgzf(c)
    out, info, _ = gpu.inflate_members(f)
    assert out == a + b + c == gzip.decompress(f)
    assert info["members"] == info["batched"] + 1


def test_errors(gpu):
    data = W.log_text(30, 500_000, exact=True)
    f = bytearray(W.bgzf(data))
    f[-28 - 8] ^= 1  # the last data member's CRC (the end-of-file member is 28 bytes)
    with pytest.raises(gpuinflate.InflateError) as e:
        gpu.inflate_members(bytes(f))
    assert e.value.code == gpuinflate.GI_ERR_DATA
    f[-28 - 8] ^= 1
    f[100] ^= 0x55  # damaged Deflate data in the first member: invalid, or running past its end
    with pytest.raises(gpuinflate.InflateError) as e:
        gpu.inflate_members(bytes(f))
    assert e.value.code in (gpuinflate.GI_ERR_DATA, gpuinflate.GI_ERR_TRUNCATED)
    bad = member(data)
    bad = bad[:-8] + struct.pack("<II", zlib.crc32(data) ^ 1, len(data))
    with pytest.raises(gpuinflate.InflateError) as e:
        gpu.inflate_members(member(b"first") + bad)
    assert e.value.code == gpuinflate.GI_ERR_DATA and "CRC" in e.value.msg
    with pytest.raises(gpuinflate.InflateError) as e:
        gpu.inflate_members(member(data, fhcrc=True, bad_hcrc=True))
    assert e.value.code == gpuinflate.GI_ERR_DATA and "header CRC" in e.value.msg
    with pytest.raises(gpuinflate.InflateError) as e:
        gpu.inflate_members(member(data)[:-5])
    assert e.value.code == gpuinflate.GI_ERR_TRUNCATED
    for nothing in (b"", b"plain text, not gzip"):
        with pytest.raises(gpuinflate.InflateError) as e:
            gpu.inflate_members(nothing)
        assert e.value.code == gpuinflate.GI_ERR_DATA


def test_sink_stops(gpu):
    f = W.bgzf(W.log_text(40, 1 << 20, exact=True))
    seen = []

    def sink(chunk):
        seen.append(len(chunk))
        return len(seen) < 3

    with pytest.raises(gpuinflate.InflateError) as e:
        gpu.inflate_members(f, sink=sink)
    assert e.value.code == gpuinflate.GI_ERR_ABORTED and len(seen) == 3
    out, info, _ = gpu.inflate_members(f)  # the context is usable again
    assert info["members"] > 3
