"""GPU parity: the CUDA path, called through the C ABI, against the oracle
and the golden digests. Integer/byte work, so the bar is bit-exact
(coefficients, per-block Tier-1 results, whole codestreams)."""
import hashlib
import json
import os

import numpy as np
import pytest

import jp2lam_gb300 as jl
from jp2lam_gb300._native import synth_page

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "golden.json")))


@pytest.fixture(scope="module")
def eng():
    e = jl.Engine(0)
    yield e
    e.close()


def _page(w, h, c, seed, photo=True):
    return synth_page(w, h, c, seed, photo_w=w // 3 if photo else 0, photo_h=h // 3 if photo else 0)


SMALL = [(1, 1), (2, 2), (3, 5), (5, 3), (8, 1), (1, 9), (17, 19), (33, 65), (64, 64), (65, 63),
         (100, 70), (129, 200), (300, 257)]


@pytest.mark.parametrize("w,h", SMALL)
@pytest.mark.parametrize("q", [100, 85, 20])
@pytest.mark.parametrize("c", [1, 3])
def test_coefficients_bit_exact(eng, orc, w, h, q, c):
    px = _page(w, h, c, w * 131 + h)
    for comp in range(c):
        g = eng.debug_coefficients(px, w, h, c, q, comp)
        o = orc.coefficients(px, w, h, c, q, comp)
        assert np.array_equal(g, o), (comp, np.argwhere(g != o)[:5])


@pytest.mark.parametrize("w,h", [(64, 64), (100, 70), (300, 257), (517, 389)])
@pytest.mark.parametrize("q", [100, 85, 50, 20])
@pytest.mark.parametrize("c", [1, 3])
def test_block_results_match(eng, orc, w, h, q, c):
    px = _page(w, h, c, 7 + q)
    rows = eng.debug_blocks(px, w, h, c, q)
    full = orc.block_summary(px, w, h, c, q, pcrd=False)
    kept = orc.block_summary(px, w, h, c, q, pcrd=True)
    assert len(rows) == len(full)
    assert np.array_equal(rows[:, 0], full[:, 5]), "magnitude bit-planes"
    assert np.array_equal(rows[:, 1], full[:, 6]), "zero bit-planes"
    assert np.array_equal(rows[:, 2], full[:, 7]), "pass counts"
    assert np.array_equal(rows[:, 3], full[:, 8]), "payload lengths"
    assert np.array_equal(rows[:, 6], kept[:, 7]), "retained passes"
    assert np.array_equal(rows[:, 7], kept[:, 8]), "retained bytes"


@pytest.mark.parametrize("w,h", SMALL + [(640, 480)])
@pytest.mark.parametrize("q", [100, 99, 85, 50, 29, 1])
@pytest.mark.parametrize("c", [1, 3])
def test_codestream_byte_identical(eng, orc, w, h, q, c):
    px = _page(w, h, c, w + 17 * h + q)
    fmt = (w + h + q) % 2
    assert eng.encode(px, w, h, c, q, fmt) == orc.encode(px, w, h, c, q, fmt=fmt, threads=4)


@pytest.mark.parametrize("case", GOLD["cases"], ids=[c["name"] for c in GOLD["cases"]])
def test_golden_digests(eng, case):
    px = synth_page(case["w"], case["h"], case["ncomp"], case["seed"], glyphs=case["glyphs"],
                    photo_w=case["photo_w"], photo_h=case["photo_h"])
    data = eng.encode(px, case["w"], case["h"], case["ncomp"], case["quality"], case["format"])
    assert hashlib.sha256(data).hexdigest() == case["sha256"]


def test_public_api_matches_oracle(orc):
    px = synth_page(512, 512, 1, 0, glyphs=400)
    img = jl.Image.from_gray_bytes(512, 512, px.tobytes())
    data = jl.encode(img, jl.EncodeOptions(100, jl.OutputFormat.J2K))
    assert data == open(os.path.join(HERE, "golden", "cfg0.j2k"), "rb").read()
    enc = jl.BatchEncoder(jl.EncodeOptions(85, jl.OutputFormat.JP2))
    out = enc.encode_all([img, img])
    assert out[0] == out[1] == orc.encode(px, 512, 512, 1, 85, fmt=1)
    assert enc.encoded_count() == 2


def test_planar_rgb_input_matches_interleaved(eng):
    px = _page(97, 61, 3, 3)
    planar = np.ascontiguousarray(px.reshape(-1, 3).T).ravel()
    a = eng.encode(px, 97, 61, 3, 75, 0)
    b = eng.encode(planar, 97, 61, 3, 75, 0, interleaved=False)
    assert a == b


def test_full_size_page_q85_byte_identical_and_decodes(eng, orc):
    """The 2550x3300 gray q85 JP2 page (text + 800x600 photo)."""
    w, h = 2550, 3300
    px = synth_page(w, h, 1, 1, photo_w=800, photo_h=600)
    g = eng.encode(px, w, h, 1, 85, 1)
    o = orc.encode(px, w, h, 1, 85, fmt=1, threads=16)
    assert g == o
    dw, dh, dc, dec = orc.decode(g)
    assert (dw, dh, dc) == (w, h, 1)
    mse = np.mean((dec.astype(np.float64) - px) ** 2)
    assert 10 * np.log10(255.0 ** 2 / mse) > 30.0


def test_lossless_round_trip_through_decoder(eng, orc):
    px = _page(333, 211, 1, 9)
    data = eng.encode(px, 333, 211, 1, 100, 1)
    _, _, _, dec = orc.decode(data)
    assert np.array_equal(dec, px)


def test_invalid_input_through_c_abi(eng):
    with pytest.raises(jl.InvalidInput):
        eng.encode(b"", 0, 0, 1, 85, 0)
    with pytest.raises(jl.InvalidInput):
        eng.encode(b"\x00" * 12, 2, 2, 3, 85, 7)
    with pytest.raises(jl.InvalidInput):
        eng.encode(b"\x00" * 8, 2, 2, 2, 85, 0)


def test_repeated_calls_are_deterministic(eng):
    px = _page(400, 300, 3, 21)
    a = eng.encode(px, 400, 300, 3, 62, 1)
    b = eng.encode(px, 400, 300, 3, 62, 1)
    c = eng.encode(_page(64, 64, 1, 2), 64, 64, 1, 85, 1)
    d = eng.encode(px, 400, 300, 3, 62, 1)
    assert a == b == d and len(c) > 0
