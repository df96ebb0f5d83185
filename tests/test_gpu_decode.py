"""The device decoder (jp2g_decode) against the oracle's restatement of the
reference's decoder (src/decode/*.rs).

Every decoded sample must equal the oracle's: lossless codestreams give the
input back, lossy ones give the oracle's reconstruction byte for byte (the
f32 dequantisation, inverse 9/7 and inverse ICT are the reference's
operations in its order, without contraction). Corrupted files either fail
on the host (both decoders) or decode to the same samples. The gray
lossless 32x32 pattern is the reference's own end-to-end test
(src/decode/mod.rs:486-508)."""
import re

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


def _same_failure(eng, orc, data, **flags):
    """Decodes with both decoders; when the oracle rejects the file the
    device decoder must reject it with the same message. Returns the
    oracle's samples, or None."""
    try:
        return orc.decode(data, **flags)
    except RuntimeError as e:
        msg = re.escape(str(e).split(": ", 2)[-1])
        with pytest.raises((jl.DecodeFailed, jl.UnsupportedFeature), match=msg):
            eng.decode(data, **flags)
        return None


@pytest.mark.parametrize("w,h,c,q", CASES)
def test_decode_equals_the_oracle(eng, orc, w, h, c, q):
    px = synth_page(w, h, c, 70 + w + q, photo_w=max(w // 3, 1), photo_h=max(h // 3, 1))
    data = eng.encode(px, w, h, c, q, (w + q) % 2)
    _same_failure(eng, orc, data)
    flags = dict(accept_empty_segments=True)
    got, gw, gh, gc = eng.decode(data, **flags)
    ow, oh, oc, want = orc.decode(data, **flags)
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


def test_decode_batch_equals_the_oracle_per_file(eng, orc):
    # mixed sizes, gray/sRGB, lossless/lossy, J2K/JP2 in one call; a broken
    # file fails alone
    shapes = [(64, 64, 1, 100), (333, 211, 3, 75), (1275, 1650, 1, 85), (7, 3, 3, 40), (640, 480, 3, 100),
              (2550, 3300, 3, 62), (100, 70, 1, 50), (257, 129, 1, 95)]
    files, pxs = [], []
    for i, (w, h, c, q) in enumerate(shapes):
        px = synth_page(w, h, c, 300 + i, photo_w=max(w // 3, 1), photo_h=max(h // 3, 1))
        pxs.append(px)
        files.append(eng.encode(px, w, h, c, q, i % 2))
    files.insert(3, files[2][:len(files[2]) // 3])
    flags = dict(rct_chroma_extra_bitplane=True, accept_empty_segments=True)
    got = eng.decode_batch(files, **flags)
    assert isinstance(got[3], (jl.DecodeFailed, jl.UnsupportedFeature))
    del got[3], files[3]
    for (w, h, c, q), px, f, g in zip(shapes, pxs, files, got):
        assert not isinstance(g, Exception), g
        data, gw, gh, gc = g
        assert (gw, gh, gc) == (w, h, c)
        want = orc.decode(f, **flags)[3]
        assert np.array_equal(np.frombuffer(data, np.uint8), want)
        if q >= 100:
            assert np.array_equal(want, px)
    imgs = jl.decode_batch(files[:2], engine=eng, **flags)
    assert [im.width for im in imgs] == [64, 333]


@pytest.mark.parametrize("w,h,c,q,seed", [(7, 3, 3, 40, 303), (257, 129, 1, 95, 307)])
def test_empty_segments_fail_like_the_reference_unless_accepted(eng, orc, w, h, c, q, seed):
    # the encoder keeps a single cleanup pass whose MQ byte count is 0 for
    # some blocks; the reference's decoder rejects such a block
    # (decode/t1.rs:109-111), and so does this one unless asked to accept it
    px = synth_page(w, h, c, seed, photo_w=max(w // 3, 1), photo_h=max(h // 3, 1))
    data = eng.encode(px, w, h, c, q, 0)
    assert data == orc.encode(px, w, h, c, q, fmt=0)
    assert _same_failure(eng, orc, data) is None
    got = eng.decode(data, accept_empty_segments=True)[0]
    assert np.array_equal(np.frombuffer(got, np.uint8), orc.decode(data, accept_empty_segments=True)[3])


def test_decode_batch_splits_rounds_under_a_small_budget(eng, orc):
    # 6 files of about 8.3 MB of device state each under a 24 MiB budget:
    # rounds of two, retried smaller when a pool cannot grow
    pages = [synth_page(640, 480, 3, 900 + i, photo_w=200, photo_h=150) for i in range(6)]
    files = [eng.encode(p, 640, 480, 3, 70, 0) for p in pages]
    small = jl.Engine(0, hbm_budget_bytes=24 << 20)
    try:
        got = small.decode_batch(files)
        for f, g in zip(files, got):
            assert not isinstance(g, Exception), g
            assert np.array_equal(np.frombuffer(g[0], np.uint8), orc.decode(f)[3])
    finally:
        small.close()


def test_large_decode_batch_two_decoders_per_warp(eng, orc):
    # over 9,728 code-blocks in one call: the decoders run two per warp;
    # every file must equal its own single-file decode and the oracle
    pages = [(2550, 3300, 3, 75), (2550, 3300, 3, 50), (1275, 1650, 1, 85)]
    files = []
    for i, (w, h, c, q) in enumerate(pages):
        px = synth_page(w, h, c, 500 + i, photo_w=w // 3, photo_h=h // 3)
        files.append(eng.encode(px, w, h, c, q, 1))
    flags = dict(accept_empty_segments=True)
    got = eng.decode_batch(files, **flags)
    for f, g in zip(files, got):
        assert not isinstance(g, Exception), g
        assert np.array_equal(np.asarray(g[0]), np.asarray(eng.decode(f, **flags)[0]))
    assert np.array_equal(np.asarray(got[1][0]), orc.decode(files[1], **flags)[3])
