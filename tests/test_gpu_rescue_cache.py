"""GPU: the device blocks a rescue keeps for its slot's next call (gr_release_cached). A rescue of
a damaged 48 MiB member holds hundreds of megabytes for its resolve; after the call they stay
with the slot (no allocation on the next call), gr_release_cached gives them back to the device,
and a rescue after that gives the same result as before."""
import zlib

import numpy as np
import pytest

from gpuzip_gb300 import gpuinflate, gzrescue

pytestmark = pytest.mark.gpu


def damaged_member():
    rng = np.random.default_rng(31)
    words = [bytes(rng.integers(97, 123, int(n), dtype=np.uint8)) for n in rng.integers(2, 9, 4096)]
    pick = rng.integers(0, len(words), 9 << 20)
    text = b" ".join(words[i] for i in pick)[: 48 << 20]
    c = zlib.compressobj(6, zlib.DEFLATED, 31)
    member = bytearray(c.compress(text) + c.flush())
    mid = (len(member) // 2) & ~4095
    member[mid:mid + 4096] = bytes(4096)  # one zeroed sector
    return bytes(member), len(text)


def test_kept_blocks_released_and_rescue_unchanged():
    torch = pytest.importorskip("torch")
    data, size = damaged_member()
    first = gzrescue.rescue(data, keep_output=False)
    assert first["rc"] == gzrescue.GR_OK and first["stats"]["output_size"] >= size - (1 << 20)
    lib = gzrescue.bind(gpuinflate.LIB_PATH)
    torch.cuda.synchronize()
    free_kept, _ = torch.cuda.mem_get_info()
    lib.gr_release_cached()
    free_back, _ = torch.cuda.mem_get_info()
    # the resolve's entries alone are 8 bytes per output byte
    assert free_back - free_kept >= 8 * size
    lib.gr_release_cached()  # nothing kept: a second call does nothing
    again = gzrescue.rescue(data, keep_output=False)
    assert again["rc"] == first["rc"] and again["stats"] == first["stats"] and again["pieces"] == first["pieces"]
