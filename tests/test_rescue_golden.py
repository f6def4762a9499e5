"""The rescue fixtures against the reference: each case's damaged input, rebuilt from its base
file and damage operations, run through gzrescue's own rescue library (built from its
gpuinflate/rescue.cpp into oracle/_ref by `make -C oracle ref`, in a tree where the reference
sources are present) gives exactly what tests/golden/rescue_golden.json holds. Without that build
the test is skipped; the fixtures' own consistency is checked either way."""
import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_rescue_golden as G  # noqa: E402


def test_fixtures_are_consistent():
    bases, info, cases = G.load_bases()
    assert len(cases) >= 20
    for c in cases:
        ref = c["reference"]
        assert c["base"] in bases
        assert ref["out_len"] == sum(ref["mask_counts"])
        if ref["stats"]:
            s = ref["stats"]
            assert s["output_size"] == ref["out_len"]
            assert s["exact_bytes"] + s["suspect_bytes"] + s["unknown_bytes"] + s["inferred_bytes"] == ref["out_len"]
            assert s["pieces"] == len(ref["pieces"])
            assert sum(p["length"] for p in ref["pieces"]) == ref["out_len"]
        assert ref["largest_chunk"] <= 1 << 20


@pytest.mark.skipif(not os.path.exists(G.REF_LIB), reason="the reference rescue library is not built here")
def test_reference_reproduces_fixtures():
    bases, info, cases = G.load_bases()
    for c in cases:
        _, r = G.run_case(c["name"], c["base"], [tuple(o) for o in c["ops"]], bases, info, G.REF_LIB)
        d = G.describe(r)
        if "tar" in c["reference"]:
            d["tar"] = G.tar_outcome(r)
        assert d == c["reference"], c["name"]
        _, ri = G.run_case(c["name"], c["base"], [tuple(o) for o in c["ops"]], bases, info, G.REF_LIB, no_infer=False)
        assert G.describe(ri) == c["reference_infer"], c["name"]
