"""CPU: the rescue interface (include/gzrescue_gb300.h): every gr_* symbol it declares is
exported, its structs have the layouts of gzrescue's gpuinflate/rescue.h (interface 4) as the C
compiler lays them out (and, where the reference tree is present, the same as its own header),
and bad arguments are refused before any GPU work."""
import ctypes
import os
import re
import subprocess
import tempfile

import pytest

import oracle
from gpuzip_gb300 import gpuinflate, gzrescue

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_HEADER = os.path.join(oracle.reference_tree() or "", "gpuinflate", "rescue.h")

PROBE = r"""
#include <stdio.h>
#include <stddef.h>
#include HEADER
int main(void) {
    printf("%zu %zu %zu\n", sizeof(gr_options), sizeof(gr_piece), sizeof(gr_stats));
    printf("%zu %zu %zu %zu\n", offsetof(gr_options, max_output), offsetof(gr_piece, why), offsetof(gr_stats, crc_check),
           offsetof(gr_stats, hidden_damage));
    return 0;
}
"""


def layout(header):
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "probe.c")
        with open(src, "w") as f:
            f.write(PROBE.replace("HEADER", '"' + header + '"'))
        exe = os.path.join(d, "probe")
        subprocess.run(["gcc", "-o", exe, src], check=True)
        return subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(gpuinflate.LIB_PATH):
        from gpuzip_gb300 import build

        build.build()
    return gzrescue.bind(gpuinflate.LIB_PATH)


def test_exports_every_declared_symbol(lib):
    src = open(os.path.join(ROOT, "include", "gzrescue_gb300.h")).read()
    names = set(re.findall(r"GR_API\s+[\w\s\*]+?\b(gr_\w+)\s*\(", src))
    assert {"gr_abi_version", "gr_rescue", "gr_rescue_raw", "gr_result_stats", "gr_result_pieces", "gr_result_notes",
            "gr_free"} <= names
    out = subprocess.run(["nm", "-D", "--defined-only", gpuinflate.LIB_PATH], capture_output=True, text=True).stdout
    assert set(re.findall(r" T (gr_\w+)", out)) == names
    assert set(gzrescue.EXPORTED) == names
    assert lib.gr_abi_version() == 4


def test_struct_layouts():
    mine = layout(os.path.join(ROOT, "include", "gzrescue_gb300.h"))
    assert [int(x) for x in mine[:3]] == [ctypes.sizeof(gzrescue.Options), ctypes.sizeof(gzrescue.Piece),
                                          ctypes.sizeof(gzrescue.Stats)]
    assert int(mine[3]) == gzrescue.Options.max_output.offset
    assert int(mine[4]) == gzrescue.Piece.why.offset
    assert int(mine[5]) == gzrescue.Stats.crc_check.offset
    assert int(mine[6]) == gzrescue.Stats.hidden_damage.offset
    if os.path.exists(REF_HEADER):
        assert layout(REF_HEADER) == mine


TAR_PROBE = r"""
#include <stdio.h>
#include <stddef.h>
#include HEADER
int main(void) {
    printf("%zu %zu %zu %zu %zu\n", sizeof(gr_tar_stats), sizeof(gr_tar_file), offsetof(gr_tar_stats, files),
           offsetof(gr_tar_file, offset), offsetof(gr_tar_file, status));
    return 0;
}
"""


def test_tar_struct_layouts():
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "probe.c")
        with open(src, "w") as f:
            f.write(TAR_PROBE.replace("HEADER", '"' + os.path.join(ROOT, "include", "gzrescue_gb300.h") + '"'))
        exe = os.path.join(d, "probe")
        subprocess.run(["gcc", "-o", exe, src], check=True)
        got = [int(x) for x in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    assert got == [ctypes.sizeof(gzrescue.TarStats), ctypes.sizeof(gzrescue.TarFile), gzrescue.TarStats.files.offset,
                   gzrescue.TarFile.offset.offset, gzrescue.TarFile.status.offset]


def test_bad_arguments_without_gpu(lib):
    res = ctypes.c_void_p(1)
    rc = lib.gr_rescue(None, 5, None, gzrescue.SINK(), None, ctypes.byref(res))
    assert rc == gzrescue.GR_ERR_ARG and not res.value
    rc = lib.gr_rescue_raw(None, 5, 10, 0, 0, None, gzrescue.SINK(), None, ctypes.byref(res))
    assert rc == gzrescue.GR_ERR_ARG
    assert lib.gr_result_pieces(None, None) == 0 and lib.gr_result_notes(None, None) == 0
    assert not lib.gr_result_stats(None)
    lib.gr_free(None)
    tar = ctypes.c_void_p(1)
    rc = lib.gr_rescue_tar(None, 5, None, gzrescue.SINK(), None, ctypes.byref(res), ctypes.byref(tar))
    assert rc == gzrescue.GR_ERR_ARG and not tar.value
    assert lib.gr_tar_result_files(None, None) == 0 and lib.gr_tar_result_skipped(None, None) == 0
    assert not lib.gr_tar_result_stats(None)
    lib.gr_tar_free(None)


def test_release_cached_without_gpu(lib):
    """With no rescue run, no slot keeps a block: the call returns without touching the device."""
    lib.gr_release_cached()
    lib.gr_release_cached()
