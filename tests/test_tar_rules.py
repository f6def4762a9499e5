"""CPU: the tar header rules of the GPU tar walk (gpuzip_gb300/csrc/gi_tar.h, the source the
header-finding kernel compiles), built on the host by tests/tar_check.cpp, agree with the oracle's
restatement of gpuzip's reader (oracle/tar_oracle.py) on number fields of every form (octal with
spaces, NULs, white space and '+', GNU base-256, digits past 64 bits, bytes that are not digits)
and on headers (valid, with signed-sum checksums, with checksums off by one, with damaged bytes)."""
import os
import random
import shutil
import subprocess
import sys

import pytest

from gpuzip_gb300 import workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import tar_oracle as T  # noqa: E402


def fields(rng, n):
    out = []
    alphabet = b"01234567 \0\t\n\x0b\x0c\r\x85\xa0+89x-"
    for k in range(n):
        kind = k % 6
        if kind == 0:  # a plain octal field
            out.append(b"%011o\0" % rng.randrange(8 ** 11))
        elif kind == 1:  # GNU base-256
            out.append(bytes([0x80 | rng.randrange(128)]) + bytes(rng.randrange(256) for _ in range(11)))
        elif kind == 2:  # 12 digits: up to 36 bits; a leading base-256 marker or 22 digits would pass 64
            out.append(b"%012o" % rng.randrange(8 ** 12))
        else:  # random bytes from a troublesome alphabet
            out.append(bytes(rng.choice(alphabet) for _ in range(12)))
    return out


def headers(rng, n):
    out = []
    for k in range(n):
        h = bytearray(W.ustar_header("f%d/%s" % (k, "x" * rng.randrange(60)), rng.randrange(1 << 30)))
        kind = k % 5
        if kind == 1:  # bytes above 127: the signed and unsigned sums differ
            for _ in range(rng.randrange(1, 6)):
                h[rng.randrange(0, 100)] = rng.randrange(128, 256)
            s_signed = sum(b - 256 if b > 127 else b for i, b in enumerate(h) if not 148 <= i < 156) + 8 * 32
            if s_signed >= 0:
                h[148:156] = b"%06o\0 " % s_signed
        elif kind == 2:  # a checksum off by one
            v = int(bytes(h[148:154]), 8) + rng.choice((-1, 1))
            h[148:156] = b"%06o\0 " % max(v, 0)
        elif kind == 3:  # damaged bytes
            for _ in range(rng.randrange(1, 4)):
                h[rng.randrange(512)] = rng.randrange(256)
        elif kind == 4:  # a checksum field of another form
            h[148:156] = rng.choice([b"        ", b"\0\0\0\0\0\0\0\0", b"  1234 \0", b"+0001750", b"0001750\0"])
        out.append(bytes(h))
    return out


def test_tar_rules_match_oracle(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "tar_check")
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "gpuzip_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "tar_check.cpp"), "-o", exe], check=True)
    rng = random.Random(12)
    fs, hs = fields(rng, 6000), headers(rng, 3000)
    (tmp_path / "f.bin").write_bytes(b"".join(fs))
    (tmp_path / "h.bin").write_bytes(b"".join(hs))
    out = subprocess.run([exe, str(tmp_path / "f.bin"), str(tmp_path / "h.bin")], capture_output=True, text=True,
                         check=True).stdout.split("\n")
    for i, f in enumerate(fs):
        ok, v = out[i].split()
        want = T.octal(f)
        assert (ok == "1") == (want is not None), f
        if want is not None:
            assert int(v) == want, f
    valid = 0
    for j, h in enumerate(hs):
        got = out[len(fs) + j] == "1"
        assert got == T.header_valid(h), j
        valid += got
    assert 1000 < valid < 3000  # both outcomes exercised
