"""CPU: the finder's code-length-code test in its table form (gpuzip_gb300/csrc/gi_find_cl.h, the
source the finder kernel compiles) agrees with the field-by-field definition, and with the
oracle's restatement of the reference's prefilter (oracle_prefilter128) on the same bits."""
import os
import random
import shutil
import subprocess

import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_table_form_equals_definition(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "cl_check")
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "gpuzip_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "cl_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe, "2000000"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout
    cases, complete = map(int, out.stdout.split())
    assert cases > 2_500_000 and complete > 400_000  # the constructed complete codes were exercised


def cl_complete(v1, v2):
    hclen = ((v1 >> 13) & 15) + 4
    f = (v1 >> 17) | ((v2 << 47) & (2 ** 64 - 1))
    s = 0
    for i in range(hclen):
        ln = (f >> (3 * i)) & 7
        s += (128 >> ln) if ln else 0
    return s == 128


def test_definition_matches_oracle_prefilter():
    rng = random.Random(3)
    hits = 0
    for _ in range(50000):
        v1, v2 = rng.getrandbits(64), rng.getrandbits(64)
        v1 = (v1 & ~0b110) | 0b100  # BTYPE 2
        head_ok = ((v1 >> 3) & 31) <= 29 and ((v1 >> 8) & 31) <= 29
        want = oracle.lib().oracle_prefilter128(v1, v2)
        assert want == (head_ok and cl_complete(v1, v2))
        hits += want
    assert hits > 50
