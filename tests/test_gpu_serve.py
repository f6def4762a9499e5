"""GPU: the request server (gi_server_*). Every request's result is the same in the mix as alone
(and the same as zlib's): requests arriving while passes run, a request larger than a pass, a
damaged member among good ones, admission held back by a small arena, and passes of two workers
running at the same time."""
import random
import time
import zlib

import pytest

from gpuzip_gb300 import gpuinflate
from gpuzip_gb300 import workloads as W

pytestmark = pytest.mark.gpu

GZIP, CRC = gpuinflate.GI_STREAM_GZIP, gpuinflate.GI_STREAM_CRC


def expected(x):
    if x["gzip"]:
        return zlib.decompress(x["data"], 31)
    return zlib.decompress(x["data"], -15)


def member(data, level=6):
    return W.gzip_wrap(W.raw_deflate(data, level), zlib.crc32(data), len(data))


@pytest.fixture(scope="module")
def mix():
    # 40 streams of 1 KiB .. 8 MiB: gzip members and raw entries with a known CRC-32
    return W.many_streams(seed=11, n=40, lo=1 << 10, hi=8 << 20, workers=1)


def test_mix_equals_alone_and_zlib(gpu, mix):
    srv = gpuinflate.Server(0, workers=2, hbm_budget=40e9, keep_output=True)
    rng = random.Random(5)
    for i, x in enumerate(mix):
        srv.submit(x["data"], flags=GZIP if x["gzip"] else CRC, expected_crc=x["crc"], tag=i)
        time.sleep(rng.random() * 0.004)  # arrivals spread over the passes
    srv.drain()
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(mix) and st["failed"] == 0 and st["submitted"] == len(mix)
    for i, x in enumerate(mix):
        r = srv.results[i]
        assert r["status"] == gpuinflate.GI_OK, (i, r)
        want = expected(x)
        assert r["output"] == want, i
        assert r["crc32"] == x["crc"] and r["out_size"] == x["size"]
        assert r["in_used"] == len(x["data"])
        alone = gpu.inflate_gzip(x["data"])[0] if x["gzip"] else gpu.inflate(x["data"])[0]
        assert alone == r["output"], i
        assert r["t_submit"] <= r["t_admit"] <= r["t_start"] <= r["t_done"]
    assert st["arena_peak"] <= st["arena_bytes"] and st["device_bytes"] <= 40e9


def test_large_request_decoded_alone():
    text = W.log_text(21, 96 << 20, exact=True)
    big = member(text)
    small = member(b"tiny request\n" * 100)
    srv = gpuinflate.Server(0, workers=2, pass_out_mb=64, hbm_budget=40e9, keep_output=True)
    srv.submit(small, tag=0)
    srv.submit(big, tag=1)
    srv.submit(small, tag=2)
    srv.drain()
    st = srv.stats()
    srv.close()
    assert st["alone"] >= 1
    assert srv.results[1]["status"] == 0 and srv.results[1]["output"] == text
    assert srv.results[1]["pass_requests"] == 1
    assert srv.results[0]["output"] == srv.results[2]["output"] == b"tiny request\n" * 100


def test_damaged_member_in_mix(mix):
    good = [x for x in mix if x["gzip"] and x["size"] > 64 << 10][:6]
    bad = W.zero_sector(good[0]["data"], 5, 0)
    srv = gpuinflate.Server(0, workers=2, hbm_budget=40e9, keep_output=True)
    for i, x in enumerate(good):
        srv.submit(x["data"], tag=i)
        if i == 2:
            srv.submit(bad, tag=100)
    srv.drain()
    srv.close()
    assert srv.results[100]["status"] in (gpuinflate.GI_ERR_DATA, gpuinflate.GI_ERR_TRUNCATED)
    for i, x in enumerate(good):
        assert srv.results[i]["status"] == 0 and srv.results[i]["output"] == expected(x)


def test_admission_waits_for_arena_room():
    rng = random.Random(9)
    reqs = []
    for i in range(24):  # 24 x 4 MiB of random bytes: 96 MiB of input, arena 64 MiB
        data = rng.randbytes(4 << 20)
        reqs.append((member(data, 1), data))
    srv = gpuinflate.Server(0, workers=2, pass_out_mb=64, hbm_budget=40e9, arena_bytes=64 << 20, keep_output=True)
    for i, (m, _) in enumerate(reqs):
        srv.submit(m, tag=i)
    srv.drain()
    st = srv.stats()
    srv.close()
    assert st["arena_bytes"] == 64 << 20
    assert st["arena_peak"] <= 64 << 20
    assert st["passes"] >= 2
    for i, (_, data) in enumerate(reqs):
        assert srv.results[i]["status"] == 0 and srv.results[i]["output"] == data


def test_passes_overlap_on_the_gpu():
    text = W.log_text(22, 200 << 20, exact=True)
    big = member(text, 1)
    smalls = [member(W.log_text(30 + i, 256 << 10, exact=True)) for i in range(8)]
    srv = gpuinflate.Server(0, workers=2, hbm_budget=60e9)
    srv.submit(big, tag=0)
    t_end = time.time() + 20
    while srv.stats()["passes"] < 1 and time.time() < t_end:
        time.sleep(0.0002)
    for i, m in enumerate(smalls):
        srv.submit(m, tag=1 + i)
    srv.drain()
    st = srv.stats()
    srv.close()
    r = srv.results
    assert all(r[k]["status"] == 0 for k in r)
    # the small requests ran on the other worker while the big pass was still running
    assert st["overlapped"] >= 1
    assert any(r[k]["worker"] != r[0]["worker"] and r[k]["t_start"] < r[0]["t_done"] for k in range(1, 9))
    assert min(r[k]["t_done"] for k in range(1, 9)) < r[0]["t_done"]


def test_rescue_requests_beside_passes(mix):
    """A damaged member submitted for rescue (GI_REQ_RESCUE) comes back with the output and mask
    that gr_rescue gives for it alone, while the other requests decode as usual."""
    from gpuzip_gb300 import gzrescue

    good = [x for x in mix if x["gzip"] and x["size"] > 256 << 10][:4]
    bad = W.zero_sector(good[1]["data"], 7, 0)
    srv = gpuinflate.Server(0, workers=2, hbm_budget=40e9, keep_output=True)
    for i, x in enumerate(good):
        srv.submit(x["data"], tag=i)
    srv.submit(bad, flags=GZIP | gpuinflate.GI_REQ_RESCUE, tag=100)
    srv.submit(good[0]["data"], flags=GZIP | gpuinflate.GI_REQ_RESCUE, tag=101)  # undamaged: all exact
    srv.drain()
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(good) + 2 and st["failed"] == 0
    for i, x in enumerate(good):
        assert srv.results[i]["output"] == expected(x)
    alone = gzrescue.rescue(bad)  # the default options, as the server's
    r = srv.results[100]
    assert r["status"] == 0 and r["output"] == alone["data"] and r["mask"] == alone["mask"]
    assert r["out_size"] == alone["stats"]["output_size"] and r["crc32"] == 0
    r = srv.results[101]
    assert r["output"] == expected(good[0]) and r["mask"] == bytes([gzrescue.GR_EXACT]) * len(r["output"])


def test_rescues_run_together(mix):
    """Several rescue requests at once: the server's rescue loops (three) and gr_rescue calls from
    several host threads run them together, on the rescue slots, and each comes back exactly as
    when it ran alone."""
    import concurrent.futures

    from gpuzip_gb300 import gzrescue

    members = [x for x in mix if x["gzip"] and x["size"] > 128 << 10][:6]
    damaged = [W.zero_sector(x["data"], 11, i) for i, x in enumerate(members)]
    alone = [gzrescue.rescue(d) for d in damaged]
    srv = gpuinflate.Server(0, workers=2, hbm_budget=60e9, keep_output=True, rescue_workers=3)
    for i, d in enumerate(damaged):
        srv.submit(d, flags=GZIP | gpuinflate.GI_REQ_RESCUE, tag=i)
    srv.drain()
    srv.close()
    for i, a in enumerate(alone):
        r = srv.results[i]
        assert r["status"] == 0 and r["output"] == a["data"] and r["mask"] == a["mask"], i
    with concurrent.futures.ThreadPoolExecutor(4) as ex:
        together = list(ex.map(gzrescue.rescue, damaged))
    for a, t in zip(alone, together):
        assert t["data"] == a["data"] and t["mask"] == a["mask"] and t["stats"] == a["stats"]
