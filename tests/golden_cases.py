"""The golden fixtures (tests/golden/): base streams and the reference decoder's results."""
import json
import os

from gpuzip_gb300 import workloads as W

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load():
    with open(os.path.join(HERE, "golden.json")) as f:
        g = json.load(f)
    streams = {}
    for name in sorted({c["stream"] for c in g["cases"]}):
        with open(os.path.join(HERE, "streams", name + ".deflate"), "rb") as f:
            streams[name] = f.read()
    return g, streams


def cases():
    """(case, input bytes) for every golden case, regenerating each damaged copy from its seed."""
    g, streams = load()
    out = []
    by_stream = {}
    for c in g["cases"]:
        by_stream.setdefault(c["stream"], []).append(c)
    for name, cs in by_stream.items():
        data = streams[name]
        rng = W.SplitMix64(cs[0]["seed"])
        variants = {"base": data}
        for it in range(g["mutations_per_stream"]):
            variants[f"m{it}"] = W.mutate(data, rng)
        for c in cs:
            out.append((c, variants[c["variant"]]))
    return out
