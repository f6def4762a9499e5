"""CPU: the oracle of the recovered-file list (oracle/tar_oracle.py) against the reference's own
test of its tar reader (src/rescue.rs:853-898), restated: a tar of 40 files and one with a long
name, damaged with a stretch of unknown bytes over a header and file data, suspect bytes in one
file, inferred bytes in another, garbage that shifts nothing and a cut at the end, reads with
partial, suspect, inferred and skipped entries; undamaged, every file reads intact. Also the two
rules after the reader (src/main.rs:546-558) and the header checksum's signed form."""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
import tar_oracle as T  # noqa: E402

from gpuzip_gb300 import workloads as W  # noqa: E402


def reference_test_tar():
    files = []
    for i in range(40):
        n = (i * 997) % 5000 + i
        files.append((f"dir/f{i}.txt", bytes(((k * 31 + i) & 0xFF) for k in range(n))))
    files.append(("n" * 150 + "/long.txt", b"long name"))
    return W.tar_archive(files), len(files)


def test_damaged_tar_reads_with_every_kind_of_entry():
    tar, nfiles = reference_test_tar()
    data = bytearray(tar)
    mask = bytearray([T.EXACT]) * len(data)
    for i in range(9000, 15000):
        mask[i] = T.UNKNOWN
        data[i] = 0
    for i in range(30000, 30100):
        mask[i] = T.SUSPECT
    for i in range(50000, 50010):
        mask[i] = T.INFERRED
    for i in range(70001, 70600):
        data[i] ^= 0x5A
    cut = len(data) - 3000
    o = T.untar(bytes(data[:cut]), bytes(mask[:cut]))
    assert o["partial"] and o["suspect"] and o["inferred"] and o["skipped"], o
    o = T.untar(tar, bytes([T.EXACT]) * len(tar))
    assert o["intact"] == nfiles and not o["skipped"] and not o["partial"] and not o["suspect"]
    assert o["bytes"] == sum(((i * 997) % 5000 + i) for i in range(40)) + len(b"long name")


def test_unverified_rules():
    tar, nfiles = reference_test_tar()
    exact = bytes([T.EXACT]) * len(tar)
    o = T.untar(tar, exact, crc_check=0, damaged=0)
    assert o["intact"] == 0 and o["unverified"] == nfiles
    o = T.untar(tar, exact, crc_check=0, damaged=1)
    assert o["intact"] == nfiles and o["unverified"] == 0
    o = T.untar(tar, exact, crc_check=-1, damaged=1, hidden_damage=1)
    assert o["intact"] == 0 and o["unverified"] == nfiles


def test_header_checksum_forms():
    h = bytearray(W.ustar_header("a", 5))
    assert T.header_valid(h)
    h[0:1] = b"\xe9"  # a byte above 127: the unsigned sum differs from the signed one
    s_unsigned = sum(h[:148]) + 8 * 32 + sum(h[156:])
    s_signed = sum(b - 256 if b > 127 else b for b in h[:148]) + 8 * 32 + sum(b - 256 if b > 127 else b for b in h[156:])
    h[148:156] = b"%06o\0 " % s_unsigned
    assert T.header_valid(h)
    h[148:156] = b"%06o\0 " % (s_signed & 0o777777)
    assert T.header_valid(h) == (s_signed >= 0)
    # digits stop at a NUL or a space (none: 0); what is left is trimmed and must be octal
    assert T.octal(b"   ") == 0 and T.octal(b"\0\0") == 0 and T.octal(b"0000644\0") == 0o644
    assert T.octal(b"\t\t") is None and T.octal(b"8") is None and T.octal(b"+17") == 0o17


def plus_pax_tar(name, length_prefix="+"):
    """A tar whose one file gets its path from a pax record written with a leading '+' on its
    length ("+NN path=...\\n"), which Rust's parse::<usize> accepts."""
    rec = b" path=" + name.encode() + b"\n"
    n = len(rec) + 2
    while len(length_prefix + str(n)) + len(rec) != n:
        n = len(length_prefix + str(n)) + len(rec)
    pax = (length_prefix + str(n)).encode() + rec
    data = b"the file's bytes\n" * 40
    parts = [W.ustar_header("PaxHeaders/plus", len(pax), typeflag=b"x"), pax, bytes(-len(pax) % 512),
             W.ustar_header(name[-90:], len(data)), data, bytes(-len(data) % 512), bytes(1024)]
    return b"".join(parts), len(pax) + 512 * 2  # (tar, an offset inside the file's data)


def test_pax_record_length_with_a_plus_sign():
    name = "deep/" + "p" * 120 + "/file.txt"
    tar, inside = plus_pax_tar(name)
    mask = bytearray([T.EXACT]) * len(tar)
    mask[inside + 600] = T.SUSPECT  # the file is listed by name among the suspect ones
    assert T.untar(tar, bytes(mask))["suspect"] == [name]
    assert T.rust_usize(b"+17") == 17 and T.rust_usize(b"17") == 17
    for bad in (b"", b"+", b"-3", b" 3", b"1_0", b"3 ", b"++3", str(1 << 64).encode()):
        assert T.rust_usize(bad) is None, bad
    # a length Rust does not parse ends the records: the header's own (shortened) name is used
    tar_bad, inside = plus_pax_tar(name, length_prefix="0x")
    mask = bytearray([T.EXACT]) * len(tar_bad)
    mask[inside + 600] = T.SUSPECT
    assert T.untar(tar_bad, bytes(mask))["suspect"] == [name[-90:]]
