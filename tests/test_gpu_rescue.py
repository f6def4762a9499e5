"""GPU: the rescue path (gr_rescue / gr_rescue_raw of libgpuinflate) against the reference's
own results on the same damaged inputs (tests/golden/rescue_golden.json, made by gzrescue's
rescue.cpp with no_infer = 1 and again with the inference on): the output bytes, the per-byte
mask, every statistic (hidden_damage included, which the one-flipped-bit test sets) and every
piece are the same; for the tar cases, the file list of gr_rescue_tar is the reader's."""
import os
import sys

import pytest

from gpuzip_gb300 import gzrescue

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_rescue_golden as G  # noqa: E402

BASES, INFO, CASES = G.load_bases()


def compare(name, got, ref):
    diffs = []
    for k in ("rc", "out_len", "data_sha256", "mask_sha256", "mask_counts"):
        if got[k] != ref[k]:
            diffs.append((k, got[k], ref[k]))
    if (got["stats"] is None) != (ref["stats"] is None):
        diffs.append(("stats", got["stats"], ref["stats"]))
    elif ref["stats"]:
        for k, v in ref["stats"].items():
            if got["stats"][k] != v:
                diffs.append(("stats." + k, got["stats"][k], v))
    if len(got["pieces"]) != len(ref["pieces"]):
        diffs.append(("pieces", len(got["pieces"]), len(ref["pieces"])))
    else:
        for i, (a, b) in enumerate(zip(got["pieces"], ref["pieces"])):
            for k in b:
                if a[k] != b[k]:
                    diffs.append((f"piece[{i}].{k}", a[k], b[k]))
    return diffs


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_rescue_matches_reference(case):
    _, r = G.run_case(case["name"], case["base"], [tuple(o) for o in case["ops"]], BASES, INFO, None)
    got = G.describe(r)
    diffs = compare(case["name"], got, case["reference"])
    assert not diffs, diffs[:12]
    assert got["largest_chunk"] <= 1 << 20


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_rescue_with_inference_matches_reference(case):
    """With the inference of lost window bytes on (the reference's default): the bytes it infers,
    their mask (GR_INFERRED) and every statistic as the reference's."""
    _, r = G.run_case(case["name"], case["base"], [tuple(o) for o in case["ops"]], BASES, INFO, None, no_infer=False)
    got = G.describe(r)
    diffs = compare(case["name"], got, case["reference_infer"])
    assert not diffs, diffs[:12]


TAR_CASES = [c for c in CASES if "tar" in c["reference"]]


@pytest.mark.parametrize("case", TAR_CASES, ids=[c["name"] for c in TAR_CASES])
def test_tar_walk_matches_reader(case):
    """gr_rescue_tar's file list (the walk on the GPU) is the one gpuzip's reader gives for the
    reference's rescued stream (its restatement in oracle/tar_oracle.py, recorded in the fixtures)."""
    data = G.damage(BASES[case["base"]], [tuple(o) for o in case["ops"]])
    r = gzrescue.rescue_tar(data, no_infer=True)
    assert r["rc"] == 0
    want = case["reference"]["tar"]
    got = {k: r["tar"][k] for k in want}
    assert got == want


def test_inference_model_learned_on_gpu(capfd, monkeypatch):
    """The inference cases' context models are learned on the GPU (atomic insertion, checked to
    give the ordered table's counts), not again on the host: the debug report names the learner,
    and the results are the reference's."""
    monkeypatch.setenv("GPUZIP_RESCUE_DEBUG", "1")
    for case in CASES:
        _, r = G.run_case(case["name"], case["base"], [tuple(o) for o in case["ops"]], BASES, INFO, None, no_infer=False)
        assert not compare(case["name"], G.describe(r), case["reference_infer"])
    err = capfd.readouterr().err
    assert "train(gpu)" in err and "train(host)" not in err


def test_inference_in_small_chunks_matches_reference(monkeypatch):
    """The inference's host pass over the list of unknown bytes, cut into chunks of 16 entries
    (so that even the small cases take many chunks and owners in parallel): the same results."""
    monkeypatch.setenv("GPUZIP_RESCUE_CHUNK", "16")
    for case in CASES:
        _, r = G.run_case(case["name"], case["base"], [tuple(o) for o in case["ops"]], BASES, INFO, None, no_infer=False)
        diffs = compare(case["name"], G.describe(r), case["reference_infer"])
        assert not diffs, (case["name"], diffs[:12])
