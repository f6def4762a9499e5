"""GPU: the CRC-32 entry point that allocates nothing (gi_crc32_device_noalloc).

It exists for callers that cannot call cudaMalloc (a serving process whose device memory is all
reserved by its own pool, a framework that hands out memory only through its allocator). This
file runs last so that, if it fails, a run that stops at the first failure has run every other
test; it also passes alone in a fresh process, where its first call does the per-device set-up.
"""
import zlib

import pytest

from gpuzip_gb300 import gpuinflate
from gpuzip_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_noalloc_crc_matches_the_decode_path_twice():
    torch = pytest.importorskip("torch")
    g = gpuinflate.Gpu(0, segment_out_mb=64)
    try:
        text = W.log_text(21, 3 << 20) + bytes(range(256)) * 37
        s = W.raw_deflate(text, 6)
        d_in = torch.frombuffer(bytearray(s), dtype=torch.uint8).cuda()
        d_out = torch.empty(len(text) + 64, dtype=torch.uint8, device="cuda")
        n, _ = g.inflate_device(d_in.data_ptr(), len(s), d_out.data_ptr(), d_out.numel())
        assert n == len(text)
        want = g.last_crc32()  # the existing entry point's CRC, computed on the GPU
        assert want == zlib.crc32(text)
        d_crc = torch.zeros(2, dtype=torch.int64, device="cuda")
        for _ in range(2):  # two calls in a row share the fixed scratch
            d_crc.zero_()
            gpuinflate.crc32_device_noalloc(d_out.data_ptr(), n, d_crc.data_ptr())
            torch.cuda.synchronize()
            assert int(d_crc[0].item()) & 0xFFFFFFFF == want
        # a length that is not a multiple of the 4 KiB tile, and an empty one
        gpuinflate.crc32_device_noalloc(d_out.data_ptr(), 12345, d_crc.data_ptr())
        torch.cuda.synchronize()
        assert int(d_crc[0].item()) & 0xFFFFFFFF == zlib.crc32(text[:12345])
        gpuinflate.crc32_device_noalloc(d_out.data_ptr(), 0, d_crc.data_ptr())
        torch.cuda.synchronize()
        assert int(d_crc[0].item()) & 0xFFFFFFFF == 0
    finally:
        g.close()


def test_noalloc_rejects_what_does_not_fit():
    torch = pytest.importorskip("torch")
    d = torch.zeros(64, dtype=torch.uint8, device="cuda")
    d_crc = torch.zeros(1, dtype=torch.int64, device="cuda")
    with pytest.raises(gpuinflate.InflateError) as e:
        gpuinflate.crc32_device_noalloc(d.data_ptr(), (1 << 30) + 1, d_crc.data_ptr())
    assert e.value.code == gpuinflate.GI_ERR_ARG and "1 GiB" in e.value.msg
    with pytest.raises(gpuinflate.InflateError) as e:
        gpuinflate.crc32_device_noalloc(d.data_ptr() + 1, 16, d_crc.data_ptr())
    assert e.value.code == gpuinflate.GI_ERR_ARG and "aligned" in e.value.msg


SET_UP_THEN_FULL = r"""
import sys, zlib
import torch
sys.path.insert(0, sys.argv[1])
from gpuzip_gb300 import gpuinflate
data = bytes(range(256)) * 40000 + b"tail"
d = torch.frombuffer(bytearray(data), dtype=torch.uint8).cuda()
d_crc = torch.zeros(1, dtype=torch.int64, device="cuda")
torch.cuda.synchronize()
gpuinflate.crc32_device_noalloc(d.data_ptr(), 0, d_crc.data_ptr())  # the set-up call, before the pool
torch.cuda.synchronize()
free, _ = torch.cuda.mem_get_info()
filler = torch.empty(free - (256 << 20), dtype=torch.uint8, device="cuda")  # the caller's pool
torch.cuda.synchronize()
before, _ = torch.cuda.mem_get_info()
for _ in range(2):
    d_crc.zero_()
    gpuinflate.crc32_device_noalloc(d.data_ptr(), len(data), d_crc.data_ptr())
    torch.cuda.synchronize()
    assert int(d_crc[0].item()) & 0xFFFFFFFF == zlib.crc32(data)
after, _ = torch.cuda.mem_get_info()
assert after == before, (before, after)
print("ok", before >> 20, "MiB free")
"""


def test_noalloc_after_the_device_is_filled():
    """A fresh process, lazy module loading: the set-up call (size 0) comes first, then the caller
    takes all but 256 MiB of the device for its own pool; the entry point then computes the CRC-32
    twice with no change in free device memory."""
    import os
    import subprocess
    import sys

    pytest.importorskip("torch")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, CUDA_MODULE_LOADING="LAZY")
    r = subprocess.run([sys.executable, "-c", SET_UP_THEN_FULL, root], capture_output=True, text=True, env=env,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok")
