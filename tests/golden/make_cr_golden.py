"""Makes the golden fixtures of the search for the CRs a raw Deflate stream lost to an ASCII-mode
transfer, from the REFERENCE's own rescue library.

    python tests/golden/make_cr_golden.py      (needs oracle/_ref/libgzrescue_ref.so: `make -C oracle ref`)

A Windows-to-Unix ASCII transfer takes the CR out of every CR LF pair, in the compressed bytes too.
gzrescue's gr_rescue_raw, given the stream's size and CRC, puts one or two of them back
(gpuinflate/rescue.cpp:2270-2363 find_lost_crs, called from :2499-2510). Each case takes a base
raw stream, removes the CR of some of the CR LF pairs in its compressed bytes (`strip_crs`, a pure
function of the positions, which the fixture records), and calls gr_rescue_raw with the size and
CRC known and the case's cr_lost, crs_expected and cr_budget options: once with no_infer = 1 and
once with the inference on. Recorded: the return code, the output's and mask's SHA-256, the mask's
counts, every statistic (cr_restored, and cr_decoded: the input bytes the search decoded) and
every piece.

Bases: tests/golden/rescue/raw.bin (the raw stream of the other rescue fixtures, four CR LF pairs),
three of the decoder's golden streams (tests/golden/streams/g-mixed, g-fixed, g-l1: small enough
that two lost CRs are found within the default budget, and one pair 16 bytes into a fixed-Huffman
block), and tests/golden/rescue/cr_auto.bin (a raw stream of 2 MiB of log text, seed 392, level 9,
memLevel 5: two CR LF pairs, so that with both gone the input looks CR-stripped on its own).
"""
import json
import os
import sys
import zlib

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)
import make_rescue_golden as G  # noqa: E402
from gpuzip_gb300 import gzrescue  # noqa: E402
from gpuzip_gb300 import workloads as W  # noqa: E402

OUT = os.path.join(HERE, "cr_golden.json")
AUTO = os.path.join(G.BASE_DIR, "cr_auto.bin")


def crlf_pairs(data):
    """Positions j with data[j:j+2] == b'\\r\\n' (the CRs a transfer would take out)."""
    out, j = [], data.find(b"\r\n")
    while j >= 0:
        out.append(j)
        j = data.find(b"\r\n", j + 1)
    return out


def strip_crs(data, positions):
    """data without the CR at each position (each the CR of a CR LF pair)."""
    out, p = bytearray(), 0
    for j in sorted(positions):
        assert data[j:j + 2] == b"\r\n", j
        out += data[p:j]
        p = j + 1
    out += data[p:]
    return bytes(out)


def auto_base():
    text = W.log_text(392, 2 << 20, exact=True)
    c = zlib.compressobj(9, zlib.DEFLATED, -15, 5)
    return c.compress(text) + c.flush(), {"size": len(text), "crc": zlib.crc32(text)}


STREAMS = ("g-mixed", "g-fixed", "g-l1")


def small_bases():
    bases = {}
    for name in STREAMS:
        with open(os.path.join(HERE, "streams", name + ".deflate"), "rb") as f:
            bases[name] = f.read()
    return bases


def load():
    bases, _, _ = G.load_bases()
    bases.update(small_bases())
    with open(AUTO, "rb") as f:
        bases["cr_auto"] = f.read()
    with open(OUT) as f:
        g = json.load(f)
    return bases, g["info"], g["cases"]


def cases(bases):
    p = crlf_pairs(bases["raw"])
    q = crlf_pairs(bases["cr_auto"])
    m, f, l1 = (crlf_pairs(bases[n]) for n in STREAMS)
    return [
        # (name, base, CRs taken out, cr_lost, crs_expected, cr_budget)
        ("raw-cr-first", "raw", [p[0]], 1, 0, 0),
        ("raw-cr-late", "raw", [p[3]], 1, 0, 0),
        ("raw-cr-one-told", "raw", [p[1]], 1, 1, 0),
        ("raw-cr-two-near", "raw", [p[1], p[2]], 1, 0, 0),
        ("raw-cr-two-far", "raw", [p[0], p[3]], 1, 2, 0),
        ("raw-cr-two-told-one", "raw", [p[0], p[1]], 1, 1, 0),
        ("raw-cr-three", "raw", [p[0], p[1], p[3]], 1, 0, 0),
        ("raw-cr-budget", "raw", [p[1], p[3]], 1, 0, 3 << 20),
        ("raw-cr-none-lost", "raw", [], 1, 0, 0),
        ("raw-cr-told-none", "raw", [p[2]], 1, 255, 0),
        ("raw-cr-never", "raw", [p[2]], 2, 0, 0),
        ("auto-cr-two", "cr_auto", list(q), 0, 0, 0),
        ("mixed-cr-two", "g-mixed", [m[0], m[1]], 1, 0, 0),
        ("mixed-cr-two-told", "g-mixed", [m[1], m[3]], 1, 2, 0),
        ("fixed-cr-start", "g-fixed", [f[0]], 1, 0, 0),
        ("l1-cr-one-told", "g-l1", [l1[0]], 1, 1, 0),
    ]


def run_case(base, strip, cr_lost, crs_expected, cr_budget, bases, info, lib_path, no_infer):
    data = strip_crs(bases[base], strip)
    i = info[base]
    return gzrescue.rescue(data, raw=True, expected_size=i["size"], expected_crc=i["crc"], cr_lost=cr_lost,
                           crs_expected=crs_expected, cr_budget=cr_budget, lib_path=lib_path, no_infer=no_infer)


def main():
    if not os.path.exists(G.REF_LIB):
        sys.exit(f"{G.REF_LIB} is missing: run `make -C oracle ref` first")
    bases, info, _ = G.load_bases()
    auto, auto_info = auto_base()
    with open(AUTO, "wb") as f:
        f.write(auto)
    bases["cr_auto"] = auto
    info = {"raw": info["raw"], "cr_auto": auto_info}
    for name, b in small_bases().items():
        bases[name] = b
        text = zlib.decompress(b, -15)
        info[name] = {"size": len(text), "crc": zlib.crc32(text)}
    out = {"info": info, "cases": []}
    for name, base, strip, cr_lost, crs_expected, budget in cases(bases):
        d = {}
        for key, no_infer in (("reference", True), ("reference_infer", False)):
            r = run_case(base, strip, cr_lost, crs_expected, budget, bases, info, G.REF_LIB, no_infer)
            d[key] = G.describe(r)
        out["cases"].append({"name": name, "base": base, "strip": strip, "cr_lost": cr_lost,
                             "crs_expected": crs_expected, "cr_budget": budget, **d})
        s = d["reference"]["stats"] or {}
        print(f"{name:22s} rc {d['reference']['rc']} out {d['reference']['out_len']:8d} restored {s.get('cr_restored')} "
              f"decoded {s.get('cr_decoded')} pieces {len(d['reference']['pieces'])} crc {s.get('crc_check')}", flush=True)
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
