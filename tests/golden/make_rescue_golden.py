"""Makes the golden fixtures of the rescue path from the REFERENCE's own rescue library.

    python tests/golden/make_rescue_golden.py      (needs oracle/_ref/libgzrescue_ref.so: `make -C oracle ref`)

Four undamaged base files are written to tests/golden/rescue/ (a gzip member of log text, a
gzip member of mixed content at mixed levels, three gzip members back to back, a raw Deflate
stream). Each case applies a list of damage operations to a base - zeroed sectors, a span written
twice, a truncation, a run of 0xFF bytes, one flipped bit, a damaged header, a zero tail, CR LF
to LF in a region, LF to CR LF everywhere - with `damage()`, a pure-Python function of the
operations, so the damaged bytes do not depend on the zlib of the machine that checks them.
For every case the reference's gr_rescue (or gr_rescue_raw), called with no_infer = 1 and again
with the inference of lost window bytes on (its default), gives: its return code, the SHA-256 of
the output and of the mask, the mask's counts per state, every statistic and every piece (all
fields but the text of `why`).
"""
import hashlib
import json
import os
import sys
import zlib

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import tar_oracle  # noqa: E402
from gpuzip_gb300 import gzrescue  # noqa: E402
from gpuzip_gb300 import workloads as W  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
BASE_DIR = os.path.join(HERE, "rescue")
OUT = os.path.join(HERE, "rescue_golden.json")
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libgzrescue_ref.so")


def deflate(data, level, mem_level=8, strategy=zlib.Z_DEFAULT_STRATEGY):
    """Raw Deflate; zlib ends a block every 2^(mem_level + 6) - 1 symbols (16,383 at its default 8)."""
    c = zlib.compressobj(level, zlib.DEFLATED, -15, mem_level, strategy)
    return c.compress(data) + c.flush()


def member(data, level, mem_level=8, strategy=zlib.Z_DEFAULT_STRATEGY):
    return W.gzip_wrap(deflate(data, level, mem_level, strategy), zlib.crc32(data), len(data))


def make_bases():
    text = W.log_text(41, 1024 << 10, exact=True)
    mixed = W.mixed_member(seed=43, nseg=6, seg_bytes=256 << 10, workers=1)[0]
    members = (member(W.log_text(44, 400 << 10, exact=True), 6, 5) + member(W.log_text(45, 300 << 10, exact=True), 9, 6) +
               member(W.log_text(46, 350 << 10, exact=True), 1, 5))
    raw_text = W.log_text(47, 900 << 10, exact=True)
    return {
        "tar": member(tar_base(), 6, 5),
        "text": member(text, 6, 5),
        "text8": member(W.log_text(48, 1280 << 10, exact=True), 6),
        "fixed": member(W.log_text(50, 384 << 10, exact=True), 6, 5, zlib.Z_FIXED),
        "mixed": mixed,
        "members": members,
        "raw": deflate(raw_text, 9, 5),
    }, {"raw": {"size": len(raw_text), "crc": zlib.crc32(raw_text)}}


def tar_base():
    """A tar of 48 files of the mixed workload's contents (2-96 KiB), one with a GNU long name and
    one with a pax path."""
    import numpy as np

    rng = np.random.default_rng([49, 1])
    files = []
    for i in range(48):
        size = int(np.exp(rng.uniform(np.log(2 << 10), np.log(96 << 10))))
        kind = int(rng.choice(4, p=[0.5, 0.2, 0.15, 0.15]))
        name = f"src/mod{i // 8}/file{i:03d}.dat"
        entry = (name, W.stream_content(49, i, size, kind))
        if i == 17:
            entry = ("deep/" + "n" * 120 + f"/file{i:03d}.dat", entry[1])
        if i == 31:
            entry = ("pax/" + "p" * 110 + f"/file{i:03d}.dat", entry[1], "pax")
        files.append(entry)
    return W.tar_archive(files)


def damage(data, ops):
    """The bytes of `data` with the damage operations applied in order."""
    b = bytearray(data)
    for op in ops:
        kind = op[0]
        if kind == "zero":
            _, at, n = op
            b[at:at + n] = bytes(min(n, len(b) - at))
        elif kind == "fill":
            _, at, n, v = op
            b[at:at + n] = bytes([v]) * min(n, len(b) - at)
        elif kind == "dup":  # bytes [at, at+n) written again right after themselves
            _, at, n = op
            b[at + n:at + n] = b[at:at + n]
        elif kind == "cut":
            del b[op[1]:]
        elif kind == "flip":
            b[op[1] >> 3] ^= 1 << (op[1] & 7)
        elif kind == "append":
            b += bytes([op[2]]) * op[1]
        elif kind == "crlf_to_lf":  # every CR LF in [at, at+n) loses its CR
            _, at, n = op
            region = bytes(b[at:at + n]).replace(b"\r\n", b"\n")
            b[at:at + n] = region
        elif kind == "lf_to_crlf":  # every LF gets a CR before it
            b = bytearray(bytes(b).replace(b"\n", b"\r\n"))
        else:
            raise ValueError(kind)
    return bytes(b)


def cases(bases):
    def frac(name, f, align=4096):
        return int(len(bases[name]) * f) // align * align

    t = "text"
    return [
        ("text-clean", t, []),
        ("text-sector", t, [("zero", frac(t, 0.40), 4096)]),
        ("text-three-sectors", t, [("zero", frac(t, 0.21), 4096), ("zero", frac(t, 0.52), 4096), ("zero", frac(t, 0.83), 4096)]),
        ("text-dup-span", t, [("dup", frac(t, 0.30), 65536)]),
        ("text-truncated", t, [("cut", frac(t, 0.65, 1) + 123)]),
        ("text-ff-run", t, [("fill", frac(t, 0.55), 2048, 0xFF)]),
        ("text-bit-flip", t, [("flip", frac(t, 0.45, 1) * 8 + 5)]),
        ("text-header", t, [("zero", 0, 10)]),
        ("text-zero-tail", t, [("append", 300, 0)]),
        ("text-crlf-region", t, [("crlf_to_lf", frac(t, 0.30), frac(t, 0.30))]),
        ("text-lf-to-crlf", t, [("lf_to_crlf",)]),
        ("text-sector-and-cut", t, [("zero", frac(t, 0.35), 4096), ("cut", frac(t, 0.80, 1))]),
        ("text-two-adjacent", t, [("zero", frac(t, 0.62), 8192)]),
        ("text8-clean", "text8", []),
        ("text8-sector", "text8", [("zero", frac("text8", 0.40), 4096)]),
        ("mixed-clean", "mixed", []),
        ("mixed-sector", "mixed", [("zero", frac("mixed", 0.50), 4096)]),
        ("mixed-two-sectors", "mixed", [("zero", frac("mixed", 0.15), 4096), ("zero", frac("mixed", 0.70), 8192)]),
        ("members-clean", "members", []),
        ("members-sector", "members", [("zero", frac("members", 0.55), 4096)]),
        ("members-truncated", "members", [("cut", frac("members", 0.90, 1))]),
        ("fixed-clean", "fixed", []),
        ("fixed-sector", "fixed", [("zero", frac("fixed", 0.45), 4096)]),
        ("fixed-two-sectors", "fixed", [("zero", frac("fixed", 0.20), 4096), ("zero", frac("fixed", 0.70), 4096)]),
        ("fixed-flip", "fixed", [("flip", int(len(bases["fixed"]) * 0.55) * 8 + 6)]),
        ("fixed-truncated", "fixed", [("cut", frac("fixed", 0.60, 1) + 77)]),
        ("tar-clean", "tar", []),
        ("tar-sector", "tar", [("zero", frac("tar", 0.45), 4096)]),
        ("tar-three-sectors", "tar", [("zero", frac("tar", 0.20), 4096), ("zero", frac("tar", 0.50), 4096),
                                      ("zero", frac("tar", 0.80), 4096)]),
        ("tar-dup-span", "tar", [("dup", frac("tar", 0.35), 65536)]),
        ("tar-crlf-region", "tar", [("crlf_to_lf", frac("tar", 0.55), frac("tar", 0.30))]),
        ("tar-truncated", "tar", [("cut", frac("tar", 0.70, 1))]),
        ("tar-bit-flip", "tar", [("flip", frac("tar", 0.62, 1) * 8 + 3)]),
        ("text-flip-71", t, [("flip", int(len(bases[t]) * 0.71) * 8 + 3)]),
        ("text8-flip-27", "text8", [("flip", int(len(bases["text8"]) * 0.27) * 8 + 3)]),
        ("members-flip-13", "members", [("flip", int(len(bases["members"]) * 0.13) * 8 + 3)]),
        ("members-flip-27", "members", [("flip", int(len(bases["members"]) * 0.27) * 8 + 3)]),
        ("members-flip-41", "members", [("flip", int(len(bases["members"]) * 0.41) * 8 + 3)]),
        ("tar-flip-86", "tar", [("flip", int(len(bases["tar"]) * 0.86) * 8 + 3)]),
        ("raw-flip-mended-59", "raw", [("flip", 1318077)]),
        ("raw-flip-mended-84", "raw", [("flip", 1871005)]),
        ("raw-flip-25", "raw", [("flip", 564093)]),
        ("raw-clean", "raw", []),
        ("raw-sector", "raw", [("zero", frac("raw", 0.50), 4096)]),
        ("raw-no-trailer-info", "raw", [("zero", frac("raw", 0.60), 4096)]),
    ]


def tar_outcome(r):
    """The recovered-file list of a rescued tar (the oracle's restatement of gpuzip's reader)."""
    s = r["stats"] or {}
    o = tar_oracle.untar(r["data"], r["mask"], s.get("crc_check", -1), s.get("damaged", 0), s.get("hidden_damage", 0))
    o["skipped"] = [list(x) for x in o["skipped"]]
    return o


def describe(r):
    data, mask = r["data"], r["mask"]
    counts = [0, 0, 0, 0]
    for v in range(4):
        counts[v] = mask.count(bytes([v]))
    return {
        "rc": r["rc"],
        "out_len": len(data),
        "data_sha256": hashlib.sha256(data).hexdigest(),
        "mask_sha256": hashlib.sha256(mask).hexdigest(),
        "mask_counts": counts,
        "stats": r["stats"],
        "pieces": [{k: v for k, v in p.items() if k != "why"} for p in r["pieces"]],
        "notes": len(r["notes"]),
        "largest_chunk": r["largest_chunk"],
    }


def run_case(name, base_name, ops, bases, info, lib_path, no_infer=True):
    data = damage(bases[base_name], ops)
    if base_name == "raw":
        known = name != "raw-no-trailer-info"
        r = gzrescue.rescue(data, raw=True, expected_size=info["raw"]["size"] if known else None,
                            expected_crc=info["raw"]["crc"] if known else None, lib_path=lib_path, no_infer=no_infer)
    else:
        r = gzrescue.rescue(data, lib_path=lib_path, no_infer=no_infer)
    return data, r


def load_bases():
    bases = {}
    for name in ("text", "text8", "mixed", "members", "raw", "tar", "fixed"):
        with open(os.path.join(BASE_DIR, name + ".bin"), "rb") as f:
            bases[name] = f.read()
    with open(OUT) as f:
        g = json.load(f)
    return bases, g["info"], g["cases"]


def main():
    if not os.path.exists(REF_LIB):
        sys.exit(f"{REF_LIB} is missing: run `make -C oracle ref` first")
    bases, info = make_bases()
    os.makedirs(BASE_DIR, exist_ok=True)
    for name, b in bases.items():
        with open(os.path.join(BASE_DIR, name + ".bin"), "wb") as f:
            f.write(b)
    out = {"info": info, "cases": []}
    for name, base_name, ops in cases(bases):
        _, r = run_case(name, base_name, ops, bases, info, REF_LIB)
        d = describe(r)
        if base_name == "tar" and r["rc"] == 0:
            d["tar"] = tar_outcome(r)
        _, ri = run_case(name, base_name, ops, bases, info, REF_LIB, no_infer=False)
        di = describe(ri)
        out["cases"].append({"name": name, "base": base_name, "ops": [list(o) for o in ops], "reference": d,
                             "reference_infer": di})
        s = d["stats"] or {}
        if "tar" in d:
            t = d["tar"]
            print(f"    tar: intact {t['intact']} unverified {t['unverified']} suspect {len(t['suspect'])} "
                  f"inferred {len(t['inferred'])} partial {len(t['partial'])} skipped {t['skipped']} repaired {t['repaired']}")
        print(f"{name:22s} inferred {(di['stats'] or {}).get('inferred_bytes')} mask {di['mask_counts']}")
        print(f"{name:22s} rc {d['rc']} out {d['out_len']:8d} pieces {len(d['pieces']):3d} damaged {s.get('damaged')} "
              f"mask {d['mask_counts']} crc {s.get('crc_check')} hidden {s.get('hidden_damage')}")
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
