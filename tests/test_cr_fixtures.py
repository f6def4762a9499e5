"""The fixtures of the lost-CR search hold together: every case takes out the CR of CR LF pairs of
its base's compressed bytes, the bases are the streams the fixture's sizes and CRCs describe, and
a search that found CRs restored exactly as many as were taken out."""
import os
import sys
import zlib

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_cr_golden as C  # noqa: E402


def test_cr_cases_are_consistent():
    bases, info, cases = C.load()
    assert len(cases) >= 12
    for name, i in info.items():
        out = zlib.decompress(bases[name], -15)
        assert len(out) == i["size"] and zlib.crc32(out) == i["crc"], name
    restored_two = False
    for c in cases:
        pairs = C.crlf_pairs(bases[c["base"]])
        assert set(c["strip"]) <= set(pairs), c["name"]
        data = C.strip_crs(bases[c["base"]], c["strip"])
        assert len(data) == len(bases[c["base"]]) - len(c["strip"])
        s = c["reference"]["stats"]
        if s["cr_restored"]:
            assert s["cr_restored"] == len(c["strip"]) and s["crc_check"] == 1, c["name"]
            restored_two |= s["cr_restored"] == 2
        if c["crs_expected"] == 255 or c["cr_lost"] == 2:
            assert s["cr_decoded"] == 0
    assert restored_two
