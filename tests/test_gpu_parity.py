"""GPU: the CUDA path through the C interface against the oracle and the reference's golden
results - bytes, error class and in_used must be identical (integer work: bit-exact)."""
import hashlib
import zlib

import pytest

import golden_cases
import oracle
from gpuzip_gb300 import gpuinflate
from gpuzip_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fuzz_streams():
    return W.fuzz_streams()


def test_every_block_kind(gpu, fuzz_streams):
    for name, s in fuzz_streams.items():
        out, st = gpu.inflate(s)
        want = zlib.decompressobj(-15).decompress(s)
        assert out == want, name
        assert st.in_used == len(s), name
        assert gpu.last_crc32() == zlib.crc32(want), name
        assert gpu.last_isize() == len(want) & 0xFFFFFFFF, name


def test_every_block_kind_small_segments(gpu_small_segments, fuzz_streams):
    for name, s in fuzz_streams.items():
        out, st = gpu_small_segments.inflate(s)
        want = zlib.decompressobj(-15).decompress(s)
        assert out == want, name
        assert st.in_used == len(s), name
        assert gpu_small_segments.last_crc32() == zlib.crc32(want), name
        if len(s) > 64 << 10:
            assert st.segments > 1, name


def test_trailing_bytes_not_read(gpu):
    s = W.raw_deflate(W.log_text(4, 300_000), 6)
    out, st = gpu.inflate(s + b"\x1f\x8b" + b"garbage" * 100)
    assert st.in_used == len(s)
    assert out == zlib.decompressobj(-15).decompress(s)


def test_golden_fixtures(gpu):
    bad = []
    for c, data in golden_cases.cases():
        rc, out, used = gpu.inflate_status(data)
        if c["status"] == 0:
            ok = rc == 0 and hashlib.sha256(out).hexdigest() == c["sha256"] and used == c["in_used"]
        else:
            ok = rc == c["status"]
        if not ok:
            bad.append((c["stream"], c["variant"], rc, c["status"], len(out), c["out_len"], used, c["in_used"]))
    assert not bad, bad[:8]


def test_golden_fixtures_small_segments(gpu_small_segments):
    bad = []
    for c, data in golden_cases.cases()[::3]:
        rc, out, used = gpu_small_segments.inflate_status(data)
        if c["status"] == 0:
            ok = rc == 0 and hashlib.sha256(out).hexdigest() == c["sha256"] and used == c["in_used"]
        else:
            ok = rc == c["status"]
        if not ok:
            bad.append((c["stream"], c["variant"], rc, c["status"], len(out), c["out_len"], used, c["in_used"]))
    assert not bad, bad[:8]


def test_fuzz_against_oracle(gpu, fuzz_streams):
    rng = W.SplitMix64(4242)
    bad = []
    for name, s in fuzz_streams.items():
        for it in range(25):
            m = W.mutate(s, rng)
            want = oracle.inflate(m, 64 << 20)
            if want[0] == oracle.TOO_BIG:
                continue
            got = gpu.inflate_status(m)
            if want[0] != 0:
                ok = got[0] == want[0]
            else:
                ok = got == want
            if not ok:
                bad.append((name, it, got[0], want[0], len(got[1]), len(want[1]), got[2], want[2]))
    assert not bad, bad[:8]


def test_edge_inputs(gpu):
    assert gpu.inflate_status(b"")[0] == gpuinflate.GI_ERR_TRUNCATED
    assert gpu.inflate_status(b"\x03\x00")[0] == 0  # one empty final fixed block
    assert gpu.inflate_status(b"\x03\x00")[2] == 2
    assert gpu.inflate_status(b"\x01\x00\x00\xff\xff")[:2] == (0, b"")  # empty final stored block
    assert gpu.inflate_status(b"\x07")[0] == gpuinflate.GI_ERR_DATA  # BTYPE 3
    tiny = W.raw_deflate(b"a", 9)
    assert gpu.inflate_status(tiny)[:2] == (0, b"a")


def test_sink_abort(gpu):
    s = W.raw_deflate(W.log_text(6, 3 << 20), 6)
    with pytest.raises(gpuinflate.InflateError) as e:
        gpu.inflate(s, sink=lambda chunk: False)
    assert e.value.code == gpuinflate.GI_ERR_ABORTED
    out, _ = gpu.inflate(s)  # the context stays usable
    assert out == zlib.decompressobj(-15).decompress(s)


def test_gzip_member_crc_checked_on_gpu(gpu):
    text = W.log_text(9, 2 << 20)
    member = W.gzip_wrap(W.raw_deflate(text, 6), zlib.crc32(text), len(text))
    out, msize, st = gpu.inflate_gzip(member + b"next member")
    assert out == text and msize == len(member)
    broken = member[:-8] + (zlib.crc32(text) ^ 1).to_bytes(4, "little") + member[-4:]
    with pytest.raises(gpuinflate.InflateError) as e:
        gpu.inflate_gzip(broken)
    assert e.value.code == gpuinflate.GI_ERR_DATA and "CRC" in e.value.msg


def test_mixed_content_stream(gpu):
    member, info = W.mixed_member(seed=2, nseg=24, seg_bytes=1 << 20, want_raw=True)
    out, msize, st = gpu.inflate_gzip(member)
    assert out == info["raw"]
    assert gpu.last_crc32() == info["crc"]


def test_device_resident_form(gpu):
    torch = pytest.importorskip("torch")
    text = W.log_text(12, 5 << 20)
    s = W.raw_deflate(text, 6)
    d_in = torch.frombuffer(bytearray(s), dtype=torch.uint8).cuda()
    d_out = torch.empty(len(text) + 100, dtype=torch.uint8, device="cuda")
    n, st = gpu.inflate_device(d_in.data_ptr(), len(s), d_out.data_ptr(), d_out.numel())
    torch.cuda.synchronize()
    assert n == len(text) and st.in_used == len(s)
    assert bytes(d_out[:n].cpu().numpy()) == text
    small = torch.empty(1000, dtype=torch.uint8, device="cuda")
    with pytest.raises(gpuinflate.InflateError) as e:
        gpu.inflate_device(d_in.data_ptr(), len(s), small.data_ptr(), small.numel())
    assert e.value.code == gpuinflate.GI_ERR_SPACE
