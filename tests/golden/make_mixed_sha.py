"""Makes tests/golden/mixed4096_sha256.json: SHA-256 of every 256 MiB of the 4 GiB mixed member's
output (seed 2, 4096 segments of 1 MiB), as the oracle decodes the member, checked here against
the generator's own plaintext; with the member's size, CRC-32 and compressed size.

    python tests/golden/make_mixed_sha.py [--nseg 4096] [--seed 2]

The GPU test (tests/test_gpu_full_size.py) regenerates the member on the GPU host (the generator
is seeded and the plaintext does not depend on the zlib build) and compares the GPU's output,
chunk by chunk, with these digests.
"""
import argparse
import ctypes
import hashlib
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

CHUNK = 256 << 20


def digests(buf, size):
    return [hashlib.sha256(memoryview(buf)[a:min(size, a + CHUNK)]).hexdigest() for a in range(0, size, CHUNK)]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--nseg", type=int, default=4096)
    ap.add_argument("--seed", type=int, default=2)
    args = ap.parse_args()
    import oracle
    from gpuzip_gb300 import workloads as W

    t = time.time()
    member, info = W.mixed_member(seed=args.seed, nseg=args.nseg)
    print(f"generated in {time.time() - t:.1f} s: {len(member)} bytes", flush=True)
    size = info["size"]
    body = member[10:10 + info["deflate_size"]]
    out = ctypes.create_string_buffer(size + 1)
    n, used = ctypes.c_uint64(0), ctypes.c_uint64(0)
    t = time.time()
    rc = oracle.lib().oracle_inflate(body, len(body), out, size + 1, ctypes.byref(n), ctypes.byref(used))
    print(f"oracle decode in {time.time() - t:.1f} s: rc {rc}, {n.value} bytes, in_used {used.value}", flush=True)
    assert rc == 0 and n.value == size and used.value == len(body), "the oracle does not decode the member"
    got = digests(out, size)
    del out
    # the generator's own plaintext, segment by segment
    kinds, _ = W.mixed_plan(args.seed, args.nseg)
    want, h, have = [], hashlib.sha256(), 0
    for i in range(args.nseg):
        seg = W.mixed_segment(args.seed, i, int(kinds[i]))
        h.update(seg)
        have += len(seg)
        if have % CHUNK == 0 or i == args.nseg - 1:
            want.append(h.hexdigest())
            h = hashlib.sha256()
    assert got == want, "the oracle's output differs from the generator's plaintext"
    fx = {"seed": args.seed, "nseg": args.nseg, "chunk_bytes": CHUNK, "size": size, "crc32": info["crc"],
          "deflate_size": info["deflate_size"], "runs": info["runs"], "sha256": got,
          "made_by": "tests/golden/make_mixed_sha.py: the oracle's decode of the member, equal to the generator's plaintext"}
    path = os.path.join(HERE, f"mixed{args.nseg}_sha256.json")
    with open(path, "w") as f:
        json.dump(fx, f, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    main()
