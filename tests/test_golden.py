"""The oracle reproduces its committed golden frames (tests/golden/)."""
import json
import os

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
import sys  # noqa: E402

sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402

CASES = json.load(open(os.path.join(HERE, "golden", "oracle_frames.json")))["cases"]


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_oracle_matches_golden(case):
    got = make_golden.render_case(case)
    for k in ("covered", "packets", "exposure", "center_pixel", "vis_sha256", "tile_lum_sha256", "rgba_sha256"):
        assert got[k] == case[k], k
