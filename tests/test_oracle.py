"""CPU: the oracle against the reference's golden results, zlib, and the reference decoder."""
import hashlib
import zlib

import pytest

import golden_cases
import oracle
from gpuzip_gb300 import workloads as W


@pytest.fixture(scope="module")
def golden():
    return golden_cases.cases()


def test_oracle_matches_reference_golden(golden):
    bad = []
    for c, data in golden:
        rc, out, used = oracle.inflate(data, 8 << 20)
        got = {"status": rc, "out_len": len(out), "sha256": hashlib.sha256(out).hexdigest(), "in_used": used}
        want = {k: c[k] for k in got}
        if got != want:
            bad.append((c["stream"], c["variant"], got, want))
    assert not bad, bad[:5]


def test_golden_covers_every_class(golden):
    statuses = {c["status"] for c, _ in golden}
    assert statuses == {0, 1, 2}


def test_oracle_matches_zlib_on_every_block_kind():
    for name, s in W.fuzz_streams().items():
        rc, out, used = oracle.inflate(s, 8 << 20)
        assert rc == 0, name
        assert out == zlib.decompressobj(-15).decompress(s), name
        assert used == len(s), name


def test_in_used_stops_at_final_block():
    s = W.raw_deflate(b"abc" * 1000, 6)
    rc, out, used = oracle.inflate(s + b"trailing bytes", 1 << 20)
    assert rc == 0 and out == b"abc" * 1000 and used == len(s)


def test_reference_before_start_is_data_error():
    # a fixed block whose first symbol is a match (distance 1 before anything was written)
    # BFINAL=1, BTYPE=01, then length code 257 (0000001, 7 bits) and distance code 0 (00000)
    bits = [1, 1, 0] + [0, 0, 0, 0, 0, 0, 1] + [0, 0, 0, 0, 0] + [0] * 7
    v = 0
    for i, b in enumerate(bits):
        v |= b << i
    data = v.to_bytes((len(bits) + 7) // 8 + 2, "little")
    assert oracle.inflate(data, 1 << 20)[0] == oracle.DATA


def test_empty_and_truncated():
    assert oracle.inflate(b"", 1 << 20)[0] == oracle.TRUNCATED
    s = W.raw_deflate(W.log_text(3, 100_000), 6)
    assert oracle.inflate(s[: len(s) // 2], 1 << 20)[0] in (oracle.TRUNCATED, oracle.DATA)
    assert oracle.inflate(s[:-1], 1 << 20)[0] == oracle.TRUNCATED


def test_crc32():
    data = W.log_text(5, 300_000)
    assert oracle.crc32(data) == zlib.crc32(data)
    a, b = data[:123_457], data[123_457:]
    assert W.crc32_combine(zlib.crc32(a), zlib.crc32(b), len(b)) == zlib.crc32(data)


def test_oracle_matches_reference_decoder_directly():
    if oracle.ref_lib() is None:
        pytest.skip("reference decoder not built here (no reference tree)")
    rng = W.SplitMix64(99)
    for name, s in W.fuzz_streams().items():
        if name == "f-l6":
            continue
        for _ in range(12):
            m = W.mutate(s, rng)
            assert oracle.inflate(m, 8 << 20) == oracle.ref_inflate(m, 8 << 20), name


def test_first_headers_are_real_block_starts():
    # every block start the finder's rules accept in a stream of dynamic blocks at known places
    # must include the true block starts of a level-6 stream (one per chunk at most)
    text = W.log_text(8, 600_000)
    s = W.raw_deflate(text, 6)
    first = oracle.first_headers(s, 0, len(s) * 8, 4096 * 8)
    assert any(f != 2**64 - 1 for f in first)
    if oracle.ref_lib() is not None:
        r = oracle.ref_lib()
        for f in first:
            if f != 2**64 - 1:
                assert r.ref_plausible_dynamic_header(s, len(s), f) == 1


def test_parallel_cpu_inflate_matches_zlib():
    """The multi-threaded CPU baseline (the reference's speculative CPU decoder restated) gives
    zlib's bytes for every block kind, for a mixed member with several chunk sizes and thread
    counts, and for a prefix of it."""
    import zlib

    for name, s in W.fuzz_streams().items():
        want = zlib.decompressobj(-15).decompress(s)
        rc, out, _ = oracle.inflate_parallel(s, len(want) + 16, 4)
        assert rc == oracle.OK and out == want, name
    member, info = W.mixed_member(seed=2, nseg=24, want_raw=True)
    body = member[10:10 + info["deflate_size"]]
    for threads, chunk in ((1, 4096), (3, 16 << 10), (8, 256 << 10)):
        rc, out, secs = oracle.inflate_parallel(body, info["size"], threads, chunk_bytes=chunk)
        assert rc == oracle.OK and out == info["raw"], (threads, chunk)
        assert len(secs) == 3
    rc, out, _ = oracle.inflate_parallel(body, 5 << 20, 4, scan_bytes=len(body) // 2)
    assert rc == oracle.OK and out == info["raw"][:5 << 20]
