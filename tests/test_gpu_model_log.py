"""GPU: the rescue model's float log (gpuzip_gb300/csrc/gi_model.h, CUDA's double log rounded to
float) equals the host C library's log rounded to float - what the reference computes
(gpuinflate/rescue.cpp:1723-1733) - over a large sample of the probabilities a model's counts give:
(uni + 1) / (n + 256), then up to five times (e + 1.5 pr) / (t + 1.5), with counts drawn as a
filled table holds them (n up to 2^20 trained bytes, context totals t up to n, e up to t). The
doubles are the device's exactly: the same IEEE operations in the same order."""
import math
import os
import struct
import subprocess
import tempfile

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "gpuzip_gb300", "csrc")


def probabilities(count, seed=23):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(rng.integers(1, 1 << 20))
        uni = int(rng.integers(0, n + 1)) if rng.random() < 0.8 else 0
        pr = (uni + 1.0) / (n + 256.0)
        for _ in range(int(rng.integers(0, 6))):
            t = int(min(n, rng.geometric(1.0 / float(rng.choice([2, 30, 1000, 50000])))))
            e = int(rng.integers(0, t + 1)) if rng.random() < 0.7 else 0
            pr = (e + 1.5 * pr) / (t + 1.5)
        out.append(pr)
    return out


def test_model_log_rounds_like_the_host():
    xs = probabilities(400_000)
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "model_log_check")
        subprocess.run(["nvcc", "-O2", "-gencode", "arch=compute_103a,code=sm_103a", "-I", CSRC,
                        os.path.join(HERE, "model_log_check.cu"), "-o", exe], check=True)
        src, dst = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
        with open(src, "wb") as f:
            f.write(struct.pack(f"<{len(xs)}d", *xs))
        subprocess.run([exe, src, dst], check=True)
        got = np.fromfile(dst, dtype=np.float32)
    want = np.array([math.log(x) for x in xs], dtype=np.float64).astype(np.float32)
    differ = np.flatnonzero(got != want)
    assert len(got) == len(xs)
    assert len(differ) == 0, [(xs[i], float(got[i]), float(want[i])) for i in differ[:5]]
