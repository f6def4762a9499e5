"""GPU: the search for the CRs a raw Deflate stream lost to an ASCII-mode transfer (gr_rescue_raw
with the stream's size and CRC, cr_lost 1 or detected) against gzrescue's own rescue.cpp on the
same inputs (tests/golden/cr_golden.json): which CRs are put back (cr_restored), the input bytes
the search decoded (cr_decoded, also where the budget cut it short), the output, its mask, every
statistic and every piece; once with no_infer = 1 and once with the inference on."""
import os
import sys
import time

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
sys.path.insert(0, HERE)
import make_cr_golden as C  # noqa: E402
import make_rescue_golden as G  # noqa: E402
from test_gpu_rescue import compare  # noqa: E402

BASES, INFO, CASES = C.load()


@pytest.mark.parametrize("no_infer", [True, False], ids=["no_infer", "infer"])
@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_cr_search_matches_reference(case, no_infer):
    t = time.perf_counter()
    r = C.run_case(case["base"], case["strip"], case["cr_lost"], case["crs_expected"], case["cr_budget"], BASES, INFO,
                   None, no_infer)
    took = time.perf_counter() - t
    got = G.describe(r)
    want = case["reference" if no_infer else "reference_infer"]
    diffs = compare(case["name"], got, want)
    assert not diffs, diffs[:12]
    print(f"{case['name']}: restored {got['stats']['cr_restored']}, decoded {got['stats']['cr_decoded']}, {took:.2f} s")
