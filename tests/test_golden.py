"""CPU suite: the oracle still reproduces the committed golden digests."""
import hashlib
import json
import os

import pytest

from jp2lam_gb300._native import synth_page

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "golden.json")))


@pytest.mark.parametrize("case", GOLD["cases"], ids=[c["name"] for c in GOLD["cases"]])
def test_oracle_matches_golden(orc, case):
    px = synth_page(case["w"], case["h"], case["ncomp"], case["seed"], glyphs=case["glyphs"],
                    photo_w=case["photo_w"], photo_h=case["photo_h"])
    assert hashlib.sha256(px.tobytes()).hexdigest() == case["input_sha256"]
    data = orc.encode(px, case["w"], case["h"], case["ncomp"], case["quality"], fmt=case["format"],
                      threads=2)
    assert len(data) == case["size"]
    assert hashlib.sha256(data).hexdigest() == case["sha256"]


def test_cfg0_fixture_decodes_losslessly(orc):
    data = open(os.path.join(HERE, "golden", "cfg0.j2k"), "rb").read()
    w, h, c, dec = orc.decode(data)
    px = synth_page(512, 512, 1, 0, glyphs=400)
    assert (w, h, c) == (512, 512, 1)
    assert (dec == px).all()
