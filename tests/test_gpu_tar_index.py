"""GPU: the entries of a tar archive decoded into device memory (gi_tar_index_device), against
Python's tarfile reading the same archive: names (GNU long names, pax paths, ustar prefixes),
data offsets, sizes and types, for archives in the GNU, pax and ustar formats; a header whose
checksum fails is refused as damaged."""
import io
import tarfile
import zlib

import numpy as np
import pytest

from gpuzip_gb300 import gpuinflate
from gpuzip_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def make_tar(fmt, seed=5, nfiles=300):
    rng = np.random.default_rng(seed)
    buf = io.BytesIO()
    with tarfile.open(fileobj=buf, mode="w", format=fmt) as tf:
        for i in range(nfiles):
            if i % 37 == 5:
                ti = tarfile.TarInfo(f"dir{i}/")
                ti.type = tarfile.DIRTYPE
                tf.addfile(ti)
                continue
            if i % 53 == 7:
                ti = tarfile.TarInfo(f"links/l{i}")
                ti.type = tarfile.SYMTYPE
                ti.linkname = f"../files/f{i - 1}"
                tf.addfile(ti)
                continue
            deep = i % 11 == 3 and fmt != tarfile.USTAR_FORMAT
            name = ("n" * 140 + f"/deep{i}.bin") if deep else (f"{'p' * 90}/{'q' * 20}/f{i}" if i % 13 == 2 else f"files/f{i}")
            n = int(rng.integers(0, 70000)) if i % 5 else int(rng.integers(1, 2_000_000))
            data = rng.integers(0, 256, size=n, dtype=np.uint8).tobytes() if i % 3 else W.log_text(i, n)[:n]
            ti = tarfile.TarInfo(name)
            ti.size = len(data)
            tf.addfile(ti, io.BytesIO(data))
    return buf.getvalue()


def on_device(torch, gpu, tar):
    s = W.raw_deflate(tar, 6)
    d_in = torch.frombuffer(bytearray(s), dtype=torch.uint8).cuda()
    d_out = torch.empty(len(tar) + 4096, dtype=torch.uint8, device="cuda")
    n, _ = gpu.inflate_device(d_in.data_ptr(), len(s), d_out.data_ptr(), d_out.numel())
    torch.cuda.synchronize()
    assert n == len(tar)
    return d_out


@pytest.mark.parametrize("fmt", [tarfile.GNU_FORMAT, tarfile.PAX_FORMAT, tarfile.USTAR_FORMAT], ids=["gnu", "pax", "ustar"])
def test_index_matches_tarfile(gpu, fmt):
    torch = pytest.importorskip("torch")
    tar = make_tar(fmt)
    d_out = on_device(torch, gpu, tar)
    entries, end = gpu.tar_index_device(d_out.data_ptr(), len(tar))
    with tarfile.open(fileobj=io.BytesIO(tar), mode="r:") as tf:
        members = tf.getmembers()
    assert len(entries) == len(members)
    for e, m in zip(entries, members):
        assert e["name"].rstrip("/") == m.name.rstrip("/")
        # tarfile's offset is where the entry's first block (a long-name or pax entry) starts;
        # the index gives the entry's own header, the block before its data
        assert e["offset"] == m.offset_data and e["header"] == m.offset_data - 512
        assert e["size"] == m.size and bytes([e["type"]]) == m.type
    assert end <= len(tar) and not any(tar[end - 512:end])
    # a file's bytes where the index says they are
    big = max(entries, key=lambda e: e["size"])
    got = bytes(d_out[big["offset"]:big["offset"] + big["size"]].cpu().numpy())
    assert got == tar[big["offset"]:big["offset"] + big["size"]]


def test_damaged_header_is_refused(gpu):
    torch = pytest.importorskip("torch")
    tar = bytearray(make_tar(tarfile.GNU_FORMAT, nfiles=20))
    with tarfile.open(fileobj=io.BytesIO(bytes(tar)), mode="r:") as tf:
        third = tf.getmembers()[3].offset
    tar[third + 10] ^= 0x40  # a name byte: the checksum fails
    d_out = on_device(torch, gpu, bytes(tar))
    with pytest.raises(gpuinflate.InflateError) as e:
        gpu.tar_index_device(d_out.data_ptr(), len(tar))
    assert e.value.code == gpuinflate.GI_ERR_DATA and str(third) in e.value.msg
