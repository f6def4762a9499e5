"""Golden summary of the reference's rescue of the full-size damaged .tar.gz (2,000 files of the
mixed workload's contents, three zeroed sectors, a span written twice, CR LF to LF in a 16 MiB
region: gpuzip_gb300.workloads.rescue_tar + rescue_damage, seed 4).

    python tests/golden/make_rescue_tar_golden.py      (needs oracle/_ref/libgzrescue_ref.so)

Records the input's SHA-256, and what gzrescue's own rescue.cpp gives, with no_infer = 1 and
again with inference on (under "infer"): SHA-256 of
the output and of the mask, the mask counts, every statistic, the SHA-256 of the piece records
(as JSON, `why` left out), and the recovered-file list the reader's restatement
(oracle/tar_oracle.py) reads from that output. Takes a few minutes of CPU."""
import hashlib
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)
import make_rescue_golden as G  # noqa: E402
from gpuzip_gb300 import gzrescue  # noqa: E402
from gpuzip_gb300 import workloads as W  # noqa: E402

OUT = os.path.join(HERE, "rescue_tar_2000.json")


def damaged_input(nfiles=2000):
    member, _ = W.rescue_tar(seed=4, nfiles=nfiles)
    return W.rescue_damage(member, seed=4)[0]


def summary(r, data):
    d = G.describe(r)
    d["pieces_sha256"] = hashlib.sha256(json.dumps(d.pop("pieces"), sort_keys=True).encode()).hexdigest()
    d["input_sha256"] = hashlib.sha256(data).hexdigest()
    d["input_len"] = len(data)
    return d


def main():
    data = damaged_input()
    t = time.time()
    r = gzrescue.rescue(data, lib_path=G.REF_LIB, no_infer=True)
    secs = time.time() - t
    d = summary(r, data)
    d["tar"] = G.tar_outcome(r)
    d["reference_seconds"] = round(secs, 1)
    del r
    # the same with the inference of lost window bytes on (the reference's default)
    t = time.time()
    ri = gzrescue.rescue(data, lib_path=G.REF_LIB, no_infer=False)
    secs_i = time.time() - t
    di = summary(ri, data)
    di["tar"] = G.tar_outcome(ri)
    di["reference_seconds"] = round(secs_i, 1)
    d["infer"] = di
    with open(OUT, "w") as f:
        json.dump(d, f, indent=1)
    print(json.dumps({k: v for k, v in d.items() if k != "tar"}, indent=1))


if __name__ == "__main__":
    main()
