"""The device decoder (jp2g_decode) against the oracle's restatement of the
reference's decoder (src/decode/*.rs).

Every decoded sample must equal the oracle's: lossless codestreams give the
input back, lossy ones give the oracle's reconstruction byte for byte (the
f32 dequantisation, inverse 9/7 and inverse ICT are the reference's
operations in its order, without contraction). Corrupted files either fail
on the host (both decoders) or decode to the same samples. The gray
lossless 32x32 pattern is the reference's own end-to-end test
(src/decode/mod.rs:486-508)."""
import numpy as np
import pytest

import jp2lam_gb300 as jl
from jp2lam_gb300._native import synth_page

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    e = jl.Engine(0)
    yield e
    e.close()


def _pattern(w, h):
    y, x = np.mgrid[0:h, 0:w]
    return ((x * 7 + y * 11 + (x ^ y)) & 0xFF).astype(np.uint8).ravel()


@pytest.mark.parametrize("fmt", [0, 1])
def test_gray_lossless_pattern_round_trip(eng, fmt):
    px = _pattern(32, 32)
    data = eng.encode(px, 32, 32, 1, 100, fmt)
    got, w, h, c = eng.decode(data)
    assert (w, h, c) == (32, 32, 1)
    assert np.array_equal(np.frombuffer(got, np.uint8), px)
    img = jl.decode_jp2(data, engine=eng)
    assert img.colorspace is jl.ColorSpace.GRAY and img.data == px.tobytes()


CASES = [
    (64, 64, 1, 100), (7, 3, 1, 100), (333, 211, 1, 100), (1, 1, 1, 100), (5, 200, 1, 100),
    (64, 64, 1, 85), (333, 211, 1, 50), (333, 211, 3, 75), (1, 9, 3, 40), (257, 129, 3, 95),
    (1275, 1650, 1, 30), (1275, 1650, 3, 62), (2550, 3300, 1, 85), (2550, 3300, 3, 75),
]


@pytest.mark.parametrize("w,h,c,q", CASES)
def test_decode_equals_the_oracle(eng, orc, w, h, c, q):
    px = synth_page(w, h, c, 70 + w + q, photo_w=max(w // 3, 1), photo_h=max(h // 3, 1))
    data = eng.encode(px, w, h, c, q, (w + q) % 2)
    got, gw, gh, gc = eng.decode(data)
    ow, oh, oc, want = orc.decode(data)
    assert (gw, gh, gc) == (ow, oh, oc) == (w, h, c)
    got = np.frombuffer(got, np.uint8)
    if not np.array_equal(got, want):
        bad = np.flatnonzero(got != want)
        pytest.fail(f"{bad.size} samples differ, first at {bad[0]}: {got[bad[0]]} vs {want[bad[0]]}")
    if q >= 100:
        assert np.array_equal(got, px)


@pytest.mark.parametrize("w,h", [(64, 64), (7, 3), (333, 211), (1275, 1650)])
def test_rgb_lossless_needs_the_extra_chroma_bitplane(eng, orc, w, h):
    # the encoder codes RCT chroma with one more bit-plane than QCD signals;
    # the reference's decoder rejects such blocks, and so does this one
    # unless told about the extra bit-plane
    px = synth_page(w, h, 3, 5 + w, photo_w=max(w // 3, 1), photo_h=max(h // 3, 1))
    data = eng.encode(px, w, h, 3, 100, 1)
    got, _, _, _ = eng.decode(data, rct_chroma_extra_bitplane=True)
    assert np.array_equal(np.frombuffer(got, np.uint8), px)
    assert np.array_equal(orc.decode(data, rct_chroma_extra_bitplane=True)[3], px)
    try:
        orc.decode(data)
        oracle_failed = None
    except RuntimeError as e:
        oracle_failed = str(e)
    if oracle_failed is None:
        got2, _, _, _ = eng.decode(data)
        assert np.array_equal(np.frombuffer(got2, np.uint8), orc.decode(data)[3])
    else:
        with pytest.raises(jl.DecodeFailed, match="pass count exceeds maximum"):
            eng.decode(data)


def test_malformed_files_fail_on_the_host(eng):
    px = synth_page(100, 70, 3, 3, photo_w=30, photo_h=20)
    data = eng.encode(px, 100, 70, 3, 75, 1)
    for bad in (b"", b"\x00" * 16, data[:20], data[:len(data) // 2], b"\xff\x4f\xff\x51" + b"\x00" * 40):
        with pytest.raises((jl.DecodeFailed, jl.UnsupportedFeature)):
            eng.decode(bad)
    # the engine stays usable
    got, _, _, _ = eng.decode(data)
    assert len(got) == 100 * 70 * 3


@pytest.mark.parametrize("seed", range(6))
def test_corrupted_payload_decodes_like_the_oracle(eng, orc, seed):
    # flipped bytes in the tile data: both decoders fail on the host, or
    # both decode the same (garbled) samples
    w, h, c = 300, 200, 1 + 2 * (seed % 2)
    px = synth_page(w, h, c, 40 + seed, photo_w=100, photo_h=60)
    data = bytearray(eng.encode(px, w, h, c, 60 + 5 * seed, 0))
    rng = np.random.default_rng(seed)
    start = len(data) // 3
    for pos in rng.integers(start, len(data) - 2, size=4):
        data[int(pos)] ^= int(rng.integers(1, 256))
    data = bytes(data)
    try:
        want = orc.decode(data)[3]
    except RuntimeError:
        want = None
    if want is None:
        with pytest.raises((jl.DecodeFailed, jl.UnsupportedFeature)):
            eng.decode(data)
    else:
        got, _, _, _ = eng.decode(data)
        assert np.array_equal(np.frombuffer(got, np.uint8), want)
