"""Makes the golden fixtures of the Deflate decode path from the REFERENCE's own decoder.

    python tests/golden/make_golden.py          (needs oracle/_ref/libgi_ref.so: `make -C oracle ref`)

For each of eight small raw Deflate streams (every block kind; written to tests/golden/streams/)
and 120 damaged copies of each (the reference fuzzer's mutation kinds, SplitMix64 seeds), it
records what the reference decoder (gpuinflate/inflate.cuh, driven as gpuinflate/gi_test.cpp:47-91
drives it) returns: the error class, the output length, its SHA-256 and CRC-32, and in_used.
The base streams are stored as bytes, and the mutations are a pure-Python function of the seed,
so the fixtures do not depend on the zlib or numpy of the machine that checks them.
"""
import hashlib
import json
import os
import sys
import zlib

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle  # noqa: E402
from gpuzip_gb300 import workloads as W  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
MUTATIONS = 120
MAX_OUT = 8 << 20


def base_streams():
    text = W.log_text(11, 160 << 10)
    import numpy as np

    rng = np.random.default_rng(11)
    mixed = bytearray()
    while len(mixed) < (192 << 10):
        k = int(rng.integers(3))
        n = int(rng.integers(1, 9000))
        if k == 0:
            mixed += rng.integers(0, 256, size=n, dtype=np.uint8).tobytes()
        elif k == 1:
            a = int(rng.integers(len(text) - n))
            mixed += text[a : a + n]
        else:
            mixed += bytes([int(rng.integers(256))]) * n
    return {
        "g-l1": W.raw_deflate(text[: 96 << 10], 1),
        "g-l6": W.raw_deflate(text, 6),
        "g-l9": W.raw_deflate(text[: 96 << 10], 9),
        "g-fixed": W.raw_deflate(text[: 64 << 10], 6, zlib.Z_FIXED),
        "g-stored": W.raw_deflate(text[: 48 << 10], 0),
        "g-mixed": W.raw_deflate(bytes(mixed), 6),
        "g-huffman": W.raw_deflate(text[: 64 << 10], 6, zlib.Z_HUFFMAN_ONLY),
        "g-tiny": W.raw_deflate(b"hello, hello, hello world\n" * 3, 6),
    }


def describe(rc, out, used):
    return {"status": rc, "out_len": len(out), "sha256": hashlib.sha256(out).hexdigest(), "crc32": zlib.crc32(out),
            "in_used": used}


def main():
    if oracle.ref_lib() is None:
        oracle.build()
    if oracle.ref_lib() is None:
        sys.exit("the reference decoder is not built (no reference tree)")
    sdir = os.path.join(HERE, "streams")
    os.makedirs(sdir, exist_ok=True)
    cases = []
    for si, (name, data) in enumerate(base_streams().items()):
        with open(os.path.join(sdir, name + ".deflate"), "wb") as f:
            f.write(data)
        rng = W.SplitMix64(1000 + si)
        variants = [("base", data)]
        for it in range(MUTATIONS):
            variants.append((f"m{it}", W.mutate(data, rng)))
        for tag, m in variants:
            rc, out, used = oracle.ref_inflate(m, MAX_OUT)
            if rc == oracle.TOO_BIG:
                continue
            cases.append({"stream": name, "seed": 1000 + si, "variant": tag, **describe(rc, out, used)})
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "decoder": "reference gi::Decoder (oracle/_ref)",
                   "mutations_per_stream": MUTATIONS, "max_out": MAX_OUT, "cases": cases}, f, indent=0)
    print(f"{len(cases)} cases")


if __name__ == "__main__":
    main()
