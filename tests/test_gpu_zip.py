"""GPU: ZIP archives through gi_inflate_zip, against Python's zipfile: deflated entries at every
level, stored entries, directories, empty entries, an entry with a wrong CRC, data prepended to the
archive, two directory records sharing one entry's bytes, encrypted entries, Zip64 (more than
65,535 entries), a sink that stops, and a file that is not a ZIP."""
import io
import struct
import zipfile

import pytest

from gpuzip_gb300 import gpuinflate
from gpuzip_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def archive(files):
    b = io.BytesIO()
    with zipfile.ZipFile(b, "w") as z:
        for name, data, method, level in files:
            if name.endswith("/"):
                z.writestr(zipfile.ZipInfo(name), b"")
            else:
                z.writestr(name, data, compress_type=method, compresslevel=level)
    return b.getvalue()


def sample_files():
    files = []
    for i, n in enumerate((1, 1000, 70_000, 400_000, 3_000_000)):
        files.append((f"text{i}.log", W.log_text(60 + i, n, exact=True), zipfile.ZIP_DEFLATED, [1, 6, 9][i % 3]))
    files.append(("dir/", b"", zipfile.ZIP_STORED, None))
    files.append(("dir/stored.bin", bytes(range(256)) * 40, zipfile.ZIP_STORED, None))
    files.append(("empty.txt", b"", zipfile.ZIP_DEFLATED, 6))
    files.append(("random.bin", W.stream_content(7, 1, 200_000, W.KIND_RANDOM), zipfile.ZIP_DEFLATED, 6))
    return files


def test_entries_equal_zipfile(gpu):
    files = sample_files()
    z = archive(files)
    entries, st = gpu.inflate_zip(z)
    ref = zipfile.ZipFile(io.BytesIO(z))
    assert [e["name"] for e in entries] == ref.namelist()
    for e, (name, data, method, _) in zip(entries, files):
        if name.endswith("/"):
            assert e["status"] == gpuinflate.GI_ERR_ARG and e["output"] is None
            continue
        assert e["status"] == gpuinflate.GI_OK, name
        assert e["output"] == data == ref.read(name), name
        assert e["method"] == method


def test_wrong_crc_fails_one_entry(gpu):
    files = sample_files()
    z = bytearray(archive(files))
    ref = zipfile.ZipFile(io.BytesIO(bytes(z)))
    bad = ref.getinfo("text3.log")
    # the central directory record of text3.log: its CRC field
    pos = 0
    while True:
        pos = bytes(z).index(b"PK\x01\x02", pos)
        nlen = struct.unpack_from("<H", z, pos + 28)[0]
        if bytes(z[pos + 46:pos + 46 + nlen]) == b"text3.log":
            break
        pos += 4
    struct.pack_into("<I", z, pos + 16, bad.CRC ^ 1)
    entries, _ = gpu.inflate_zip(bytes(z))
    for e in entries:
        if e["name"] == "text3.log":
            assert e["status"] == gpuinflate.GI_ERR_DATA and e["output"] is None
        elif not e["name"].endswith("/"):
            assert e["status"] == gpuinflate.GI_OK


def test_prepended_data_and_not_a_zip(gpu):
    files = sample_files()[:3]
    z = b"#!self-extractor stub\n" * 100 + archive(files)
    entries, _ = gpu.inflate_zip(z)
    assert [e["output"] for e in entries] == [f[1] for f in files]
    for junk in (b"", b"PK\x03\x04 not really", W.log_text(3, 10_000, exact=True)):
        with pytest.raises(gpuinflate.InflateError) as err:
            gpu.inflate_zip(junk)
        assert err.value.code == gpuinflate.GI_ERR_DATA


def test_shared_bytes_and_encrypted_entries_are_left_out(gpu):
    files = sample_files()[:3]
    z = bytearray(archive(files))
    eocd = bytes(z).rindex(b"PK\x05\x06")
    ncd, size_cd, off_cd = struct.unpack_from("<HII", z, eocd + 10)
    first = bytes(z[off_cd:off_cd + 46 + struct.unpack_from("<H", z, off_cd + 28)[0]])
    # a second directory record for the first entry (a zip bomb names one stream twice), renamed
    dup = bytearray(first)
    dup[46:46 + 5] = b"DUPLI"
    # the second entry encrypted (flag bit 0 in its directory record)
    p2 = off_cd + len(first)
    struct.pack_into("<H", z, p2 + 8, struct.unpack_from("<H", z, p2 + 8)[0] | 1)
    z = z[:eocd] + dup + z[eocd:]
    eocd += len(dup)
    struct.pack_into("<HHI", z, eocd + 8, ncd + 1, ncd + 1, size_cd + len(dup))
    entries, _ = gpu.inflate_zip(bytes(z))
    st = [e["status"] for e in entries]
    assert st[0] == gpuinflate.GI_ERR_ARG and st[-1] == gpuinflate.GI_ERR_ARG  # the pair sharing bytes
    assert st[1] == gpuinflate.GI_ERR_ARG  # encrypted
    assert st[2] == gpuinflate.GI_OK and entries[2]["output"] == files[2][1]


def test_zip64_directory(gpu):
    b = io.BytesIO()
    with zipfile.ZipFile(b, "w") as zf:
        for i in range(65_600):
            zf.writestr(f"f{i}", bytes([i & 255]))
    z = b.getvalue()
    assert b"PK\x06\x06" in z  # Zip64 end record
    entries, _ = gpu.inflate_zip(z)
    assert len(entries) == 65_600
    assert all(e["status"] == 0 and e["output"] == bytes([e["index"] & 255]) for e in entries)


def test_sink_stops(gpu):
    z = archive(sample_files())
    with pytest.raises(gpuinflate.InflateError) as err:
        gpu.inflate_zip(z, stop_after=2)
    assert err.value.code == gpuinflate.GI_ERR_ABORTED
    entries, _ = gpu.inflate_zip(z)  # the context is usable again
    assert len(entries) == len(sample_files())
