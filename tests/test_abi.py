"""CPU: the C interface library loads, exports every symbol include/gpuinflate.h declares, keeps
interface 1's struct layouts, and rejects bad arguments before touching a GPU."""
import ctypes
import os
import re
import subprocess

import pytest

from gpuzip_gb300 import gpuinflate

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    src = open(os.path.join(ROOT, "include", "gpuinflate.h")).read()
    return set(re.findall(r"GI_API\s+[\w\s\*]+?\b(gi_\w+)\s*\(", src))


def declared_rescue():
    src = open(os.path.join(ROOT, "include", "gzrescue_gb300.h")).read()
    return set(re.findall(r"GR_API\s+[\w\s\*]+?\b(gr_\w+)\s*\(", src))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(gpuinflate.LIB_PATH):
        from gpuzip_gb300 import build

        build.build()
    return gpuinflate.load()


def test_exports_every_declared_symbol(lib):
    names = declared()
    assert {"gi_abi_version", "gi_create", "gi_inflate", "gi_last_error", "gi_device_name", "gi_destroy"} <= names
    out = subprocess.run(["nm", "-D", "--defined-only", gpuinflate.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (gi_\w+)", out))
    assert names <= exported, names - exported
    assert exported == names, exported - names  # nothing else is exported (visibility hidden)
    assert set(gpuinflate.EXPORTED) == names


def test_dynamic_table_holds_only_the_interfaces(lib):
    """Every defined dynamic symbol of the library is a declared gi_* or gr_* function: no C++
    runtime instances (std::thread, std::vector of this library's types) leak into the table a
    host that also links libstdc++ could resolve against."""
    out = subprocess.run(["nm", "-D", "--defined-only", gpuinflate.LIB_PATH], capture_output=True, text=True).stdout
    rows = [ln.split() for ln in out.splitlines() if ln.strip()]
    syms = {r[-1]: r[-2] for r in rows}
    want = declared() | declared_rescue()
    assert "gr_rescue" in want and "gr_rescue_raw" in want and "gr_free" in want
    assert set(syms) == want, (set(syms) - want, want - set(syms))
    assert all(kind == "T" for kind in syms.values()), syms


def test_abi_version(lib):
    assert lib.gi_abi_version() == 1


def test_struct_layouts_match_interface_1():
    # gpuinflate.h of the reference: gi_config 16 bytes, gi_stats 80 (src/inflate.rs:16-39 mirrors them)
    assert ctypes.sizeof(gpuinflate.Config) == 16
    assert ctypes.sizeof(gpuinflate.Stats) == 80
    assert gpuinflate.Stats.seconds.offset == 32


def test_bad_arguments_without_gpu(lib):
    cfg = gpuinflate.Config(8, 0, 0, 0)  # size too small
    ctx = ctypes.c_void_p()
    err = ctypes.create_string_buffer(512)
    assert lib.gi_create(ctypes.byref(cfg), ctypes.byref(ctx), err, 512) == gpuinflate.GI_ERR_ARG
    assert ctx.value is None
    assert b"too small" in err.value
    assert lib.gi_create(ctypes.byref(cfg), None, err, 512) == gpuinflate.GI_ERR_ARG
    st = gpuinflate.Stats()
    assert lib.gi_inflate(None, b"x", 1, 0, gpuinflate.SINK(), None, ctypes.byref(st)) == gpuinflate.GI_ERR_ARG
    assert lib.gi_last_error(None) == b"no context"
    assert lib.gi_device_name(None) == b""
    lib.gi_destroy(None)


def test_server_struct_layouts():
    assert ctypes.sizeof(gpuinflate.ServerConfig) == 40
    assert ctypes.sizeof(gpuinflate.Result) == 72
    assert ctypes.sizeof(gpuinflate.ServerStats) == 104
    assert gpuinflate.Result.t_submit.offset == 32
    assert gpuinflate.ServerStats.busy_s.offset == 96


def test_server_bad_arguments_without_gpu(lib):
    srv = ctypes.c_void_p()
    err = ctypes.create_string_buffer(512)
    cb = gpuinflate.DONE(lambda user, r, data: None)
    small = gpuinflate.ServerConfig(8)
    assert lib.gi_server_create(ctypes.byref(small), cb, None, ctypes.byref(srv), err, 512) == gpuinflate.GI_ERR_ARG
    assert b"too small" in err.value and srv.value is None
    cfg = gpuinflate.ServerConfig(ctypes.sizeof(gpuinflate.ServerConfig))
    assert lib.gi_server_create(ctypes.byref(cfg), gpuinflate.DONE(), None, ctypes.byref(srv), err, 512) == \
        gpuinflate.GI_ERR_ARG
    assert b"callback" in err.value
    cfg.workers = 99
    assert lib.gi_server_create(ctypes.byref(cfg), cb, None, ctypes.byref(srv), err, 512) == gpuinflate.GI_ERR_ARG
    assert lib.gi_server_create(ctypes.byref(cfg), cb, None, None, err, 512) == gpuinflate.GI_ERR_ARG
    assert lib.gi_server_submit(None, b"x", 1, 1, 0, 0) == gpuinflate.GI_ERR_ARG
    assert lib.gi_server_drain(None) == gpuinflate.GI_ERR_ARG
    st = gpuinflate.ServerStats(ctypes.sizeof(gpuinflate.ServerStats))
    assert lib.gi_server_read_stats(None, ctypes.byref(st)) == gpuinflate.GI_ERR_ARG
    assert lib.gi_server_clock(None) == 0.0
    lib.gi_server_destroy(None)


def test_members_info_layout():
    assert ctypes.sizeof(gpuinflate.MembersInfo) == 32


def test_zip_entry_layout():
    assert ctypes.sizeof(gpuinflate.ZipEntry) == 40
    assert gpuinflate.ZipEntry.out_size.offset == 16


def test_tar_entry_layout():
    assert ctypes.sizeof(gpuinflate.TarEntry) == 40
    assert gpuinflate.TarEntry.size.offset == 24 and gpuinflate.TarEntry.type.offset == 32
