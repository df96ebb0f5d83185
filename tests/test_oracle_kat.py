"""Pins the oracle against the reference's own known-answer and
cross-implementation tests (ported from the reference's #[test] functions;
each test names the one it follows)."""
import json
import os

import numpy as np
import pytest

from tests.golden import reference_tables as rt

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


# ---------------------------------------------------------------- tables ----
def test_context_and_probability_tables_match_reference(orc):
    """Tables generated from ISO 15444-1 Annex C/D rules equal the literal
    tables in src/tier1/luts.rs and src/mq/mod.rs (digests recorded by
    tests/golden/reference_tables.py)."""
    ref = json.load(open(os.path.join(GOLDEN, "reference_tables.json")))
    zc, sc, spb, mq = orc.tables()
    assert rt.digest(zc) == ref["zc_sha256"]
    assert rt.digest(sc) == ref["sc_sha256"]
    assert rt.digest(spb) == ref["spb_sha256"]
    assert rt.digest(mq) == ref["mq_states_sha256"]
    norms = [orc.lib.orc_norm97(l, o) if (o == 0 or l < 9) else 0.0
             for o in range(4) for l in range(10)]
    assert rt.digest(norms, "float") == ref["norms97_sha256"]


# ------------------------------------------------------------ plan/norms ----
def test_stepsize_packing_is_stable(orc):
    """src/dwt/norms.rs:122-129"""
    import ctypes
    e, m = ctypes.c_int(), ctypes.c_int()
    orc.lib.orc_encode_stepsize(8096, 8, ctypes.byref(e), ctypes.byref(m))
    assert (e.value, m.value) == (9, 2000)
    orc.lib.orc_irreversible_quant(8, 6, 0, 0, ctypes.byref(e), ctypes.byref(m))
    assert (e.value, m.value) == (14, 1824)


def test_norm_tables_match_reference_values(orc):
    """src/dwt/norms.rs:131-134"""
    assert orc.lib.orc_norm97(1, 1) == 3.989


@pytest.mark.parametrize("w,h,nres", [(2, 2, 2), (3, 2, 2), (3, 3, 2), (5, 3, 2), (17, 19, 5)])
def test_tiny_gray_plan_is_bounded(orc, w, h, nres):
    """src/plan/mod.rs:258-301"""
    p = orc.plan(w, h, 1, 85)
    assert p["levels"] + 1 == nres


def test_plan_caps_resolution_count(orc):
    """src/plan/mod.rs:222-256"""
    p = orc.plan(8, 8, 1, 85)
    assert p["levels"] + 1 <= 4
    assert p["cbw"] == 64


def test_lossy_rgb_plan_uses_scalar_expounded(orc):
    """src/plan/mod.rs:303-347"""
    p = orc.plan(32, 32, 3, 42)
    assert p["quants"][0][3] > 0


def test_code_block_size_follows_quality(orc):
    """src/plan/derive.rs:159-165"""
    assert orc.plan(256, 256, 1, 29)["cbw"] == 32
    assert orc.plan(256, 256, 1, 30)["cbw"] == 64


# ------------------------------------------------------------------- DWT ----
def test_53_known_2x2_case(orc):
    """src/dwt/rev53.rs:944-949"""
    assert orc.dwt([1, 2, 3, 4], 2, 2, 1, 53).tolist() == [3, 1, 2, 0]


def test_53_known_1d_row_case(orc):
    """src/dwt/rev53.rs:951-956"""
    assert orc.dwt([10, 20, 30, 40], 4, 1, 1, 53).tolist() == [10, 33, 0, 10]


def _max_dec(w, h):
    m = min(w, h)
    return 0 if m <= 1 else m.bit_length() - 1


def _tiny_patterns(w, h):
    pats = [np.zeros(w * h, np.int32), np.ones(w * h, np.int32),
            np.tile(np.arange(w, dtype=np.int32), h),
            np.repeat(np.arange(h, dtype=np.int32), w),
            np.array([(x + y) & 1 for y in range(h) for x in range(w)], np.int32)]
    for i in range(w * h):
        d = np.zeros(w * h, np.int32)
        d[i] = 255
        pats.append(d)
    return pats


def test_53_roundtrips_exactly_for_small_images(orc):
    """src/dwt/rev53.rs:1079-1096"""
    for h in range(1, 9):
        for w in range(1, 9):
            lv = min(_max_dec(w, h), 3)
            for p in _tiny_patterns(w, h):
                f = orc.dwt(p, w, h, lv, 53)
                assert np.array_equal(orc.dwt(f, w, h, lv, 53, inverse=True), p), (w, h)


@pytest.mark.parametrize("w,h,lv", [(48, 40, 5), (64, 48, 5), (32, 32, 5)])
def test_53_roundtrips_at_5_levels_non_pow2(orc, w, h, lv):
    """src/dwt/rev53.rs:1098-1112"""
    for p in _tiny_patterns(w, h)[:40]:
        f = orc.dwt(p, w, h, lv, 53)
        assert np.array_equal(orc.dwt(f, w, h, lv, 53, inverse=True), p)


def test_97_roundtrips_within_tolerance(orc):
    """src/dwt/irrev97.rs:882-905"""
    for h in range(1, 9):
        for w in range(1, 9):
            lv = min(_max_dec(w, h), 3)
            for p in _tiny_patterns(w, h):
                f = orc.dwt(p.astype(np.float32), w, h, lv, 97)
                r = orc.dwt(f, w, h, lv, 97, inverse=True)
                assert np.max(np.abs(r - p)) < 1e-3


def test_97_constant_concentrates_into_ll(orc):
    """src/dwt/irrev97.rs:907-923"""
    d = orc.dwt(np.full(64, 128.0, np.float32), 8, 8, 3, 97)
    assert abs(d[0]) > 1.0
    assert np.all(np.abs(d[1:]) < 1e-2)


def test_97_length_one_is_scaled_by_inv_k(orc):
    """src/dwt/irrev97.rs:925-930 (via a 1x1 one-level transform, which the
    reference reduces to the same x/K rule on each axis: vertical n=1 and
    horizontal n=1 each scale by 1/K)."""
    k = np.float32(1.230174104914001)
    d = orc.dwt(np.array([100.0], np.float32), 1, 1, 1, 97)
    assert abs(d[0] - np.float32(np.float32(100.0) / k) / k) < 1e-4


# -------------------------------------------------------------------- MQ ----
CTX_ZC, CTX_SC, CTX_MAG, CTX_AGG, CTX_UNI = 0, 9, 14, 17, 18


def _syms(pairs):
    return np.array([(c << 1) | b for c, b in pairs], np.uint8)


def _xorshift(s):
    s ^= (s << 13) & 0xFFFFFFFFFFFFFFFF
    s ^= s >> 7
    s ^= (s << 17) & 0xFFFFFFFFFFFFFFFF
    return s & 0xFFFFFFFFFFFFFFFF


def _cross(orc, pairs):
    s = _syms(pairs)
    a, b = orc.mq_encode(s, 0), orc.mq_encode(s, 1)
    assert a == b
    # decode round trip (src/mq/mod.rs:773-784)
    ctxs = np.array([c for c, _ in pairs], np.uint8)
    bits = orc.mq_decode(a, ctxs)
    assert bits.tolist() == [b for _, b in pairs]
    return a


def test_mq_matches_alt_uni_all_zero(orc):
    """src/mq/mod.rs:786-791"""
    _cross(orc, [(CTX_UNI, 0)] * 256)


def test_mq_matches_alt_uni_all_one(orc):
    """src/mq/mod.rs:793-798"""
    _cross(orc, [(CTX_UNI, 1)] * 256)


def test_mq_matches_alt_alternating(orc):
    """src/mq/mod.rs:800-805"""
    _cross(orc, [(CTX_AGG, i & 1) for i in range(512)])


def test_mq_matches_alt_mixed_contexts(orc):
    """src/mq/mod.rs:807-825"""
    ctxs = [CTX_ZC, CTX_SC, CTX_MAG, CTX_AGG, CTX_UNI]
    _cross(orc, [(ctxs[i % 5], ((i * 2654435761) & 0xFFFFFFFF) >> 30 & 1) for i in range(400)])


def test_mq_matches_alt_randomized(orc):
    """src/mq/mod.rs:827-851"""
    ctxs = [CTX_ZC, CTX_SC, CTX_MAG, CTX_AGG, CTX_UNI]
    for seed in range(32):
        s = (seed + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF or 1
        s = _xorshift(s)
        n = 100 + s % 1500
        pairs = []
        for _ in range(n):
            s = _xorshift(s)
            pairs.append((ctxs[s % 5], (s >> 32) & 1))
        _cross(orc, pairs)


def test_mq_matches_alt_skewed_mps(orc):
    """src/mq/mod.rs:877-890"""
    s = 0xDEADBEEFCAFEBABE
    pairs = []
    for _ in range(5000):
        s = _xorshift(s)
        pairs.append((CTX_AGG, 1 if (s & 0xFF) < 8 else 0))
    _cross(orc, pairs)


def test_mq_every_context_all_states(orc):
    """Long streams on every context drive all 47 states and carry paths."""
    rng = np.random.default_rng(7)
    for p1 in (0.01, 0.2, 0.5, 0.9):
        pairs = [(int(c), int(b)) for c, b in zip(rng.integers(0, 19, 20000),
                                                  rng.random(20000) < p1)]
        _cross(orc, pairs)


def test_mq_erterm_decodes(orc):
    """src/mq/mod.rs:923-948: ERTERM flush output decodes to the input."""
    pairs = [(CTX_ZC, 1), (CTX_AGG, 0), (CTX_UNI, 1), (CTX_AGG, 1), (CTX_UNI, 0), (CTX_ZC, 0), (CTX_UNI, 1)]
    data = orc.mq_encode(_syms(pairs), 2)
    bits = orc.mq_decode(data, np.array([c for c, _ in pairs], np.uint8))
    assert bits.tolist() == [b for _, b in pairs]


# ---------------------------------------------------------------- Tier-1 ----
BAND_LL, BAND_HL, BAND_LH, BAND_HH = 0, 1, 2, 3


def test_tier1_analysis_bitplane_metadata(orc):
    """src/encode/backend/native/t1.rs:1339-1394: 4x4, 2 levels; the LL block
    is the single coefficient -38 (Mb = 2-1+8 = 9)."""
    r = orc.t1_block([-38], 1, 1, BAND_LL, 9)
    assert r["mbp"] == 6 and r["zbp"] == 3
    assert len(r["passes"]) == 16
    assert r["passes"][0][0] == 2 and r["passes"][0][1] == 5 and r["passes"][0][2] == 1
    hh = orc.t1_block([0, 0, 0, 0], 2, 2, BAND_HH, 11)
    assert hh["mbp"] == 0 and hh["zbp"] == 11 and len(hh["passes"]) == 0


def test_tier1_codeblock_split_metadata(orc):
    """t1.rs:1396-1438 / layout.rs:223-247: 6x6 ramp, 1 level, 2x2 blocks;
    first HH block is [21, 22, 27, 28]."""
    r = orc.t1_block([21, 22, 27, 28], 2, 2, BAND_HH, 11)
    assert r["mbp"] == 5
    assert len(r["passes"]) == 13
    assert int((r["passes"][:, 0] == 0).sum()) == 4


def test_tier1_cumulative_lengths_and_single_payload(orc):
    """t1.rs:1440-1494"""
    r = orc.t1_block([-38], 1, 1, BAND_LL, 9)
    lengths = r["passes"][:, 4]
    cum = r["passes"][:, 5]
    assert lengths.sum() == len(r["payload"]) > 0
    assert np.array_equal(np.cumsum(lengths), cum)


@pytest.mark.parametrize("seed", range(12))
def test_tier1_decoder_roundtrip(orc, seed):
    """t1.rs:1496-1546: encode -> decode recovers the coefficients, for
    random blocks of every band and ragged sizes."""
    rng = np.random.default_rng(seed)
    w, h = [(64, 64), (33, 17), (1, 1), (5, 64), (64, 3), (31, 31)][seed % 6]
    band = seed % 4
    scale = [3, 40, 700, 5000][seed % 4]
    c = (rng.laplace(0, scale, w * h)).astype(np.int32)
    c[rng.random(w * h) < 0.5] = 0
    r = orc.t1_block(c, w, h, band, 16)
    if r["mbp"] == 0:
        return
    dec = orc.t1_decode(r["payload"], w, h, band, 16, r["zbp"], len(r["passes"]))
    assert np.array_equal(dec, c)


def test_tier1_is_deterministic(orc):
    """t1.rs:1548-1580"""
    rng = np.random.default_rng(3)
    c = rng.integers(-300, 300, 64 * 64).astype(np.int32)
    a = orc.t1_block(c, 64, 64, BAND_HL, 12)
    b = orc.t1_block(c, 64, 64, BAND_HL, 12)
    assert a["payload"] == b["payload"]


# ------------------------------------------------------------------- T2 -----
@pytest.mark.parametrize("n,width,code", [(1, 1, 0), (2, 2, 0b10), (3, 4, 0b1100), (5, 4, 0b1110),
                                          (6, 9, 0b1111_00000), (36, 9, 0b1111_11110),
                                          (37, 16, 0b11111111_10000000), (164, 16, 0xFFFF)])
def test_numpasses_codewords_follow_table_b4(orc, n, width, code):
    """src/encode/backend/native/t2.rs:608-627"""
    import ctypes
    c, w = ctypes.c_uint32(), ctypes.c_int()
    orc.lib.orc_t2_numpasses_bits(ctypes.c_uint32(n), ctypes.byref(c), ctypes.byref(w))
    assert (c.value, w.value) == (code, width)


def test_b1072_segment_partition(orc):
    """t2.rs:629-649 (ISO 15444-1 B.10.7.2 note)."""
    import ctypes
    lengths = np.array([6, 31, 44, 134, 192], np.uint32)
    term = np.array([1, 0, 1, 1, 1], np.int32)
    sl = np.zeros(8, np.uint32)
    sn = np.zeros(8, np.uint32)
    n = ctypes.c_int()
    inc = ctypes.c_uint32()
    orc.lib.orc_t2_segments(lengths.ctypes.data_as(ctypes.c_void_p), term.ctypes.data_as(ctypes.c_void_p),
                            5, sl.ctypes.data_as(ctypes.c_void_p), sn.ctypes.data_as(ctypes.c_void_p),
                            ctypes.byref(n), ctypes.byref(inc))
    assert list(zip(sl[:n.value], sn[:n.value])) == [(6, 1), (75, 2), (134, 1), (192, 1)]
    assert inc.value == 5
    lengths = np.array([6], np.uint32)
    term = np.array([1], np.int32)
    orc.lib.orc_t2_segments(lengths.ctypes.data_as(ctypes.c_void_p), term.ctypes.data_as(ctypes.c_void_p),
                            1, sl.ctypes.data_as(ctypes.c_void_p), sn.ctypes.data_as(ctypes.c_void_p),
                            ctypes.byref(n), ctypes.byref(inc))
    assert inc.value == 0


def _tagtree_parents_reference_walk(nw, nh):
    """Restatement of the reference's parent-linking walk
    (t2.rs:121-162) for comparison with the standard (i/2, j/2) rule."""
    nplh, nplv = [nw], [nh]
    numnodes = 0
    while True:
        n = nplh[-1] * nplv[-1]
        nplh.append((nplh[-1] + 1) // 2)
        nplv.append((nplv[-1] + 1) // 2)
        numnodes += n
        if n <= 1:
            break
    numlvls = len(nplh) - 1
    parent = [-1] * numnodes
    node = 0
    pidx = nw * nh
    pidx0 = pidx
    for i in range(numlvls - 1):
        j = 0
        while j < nplv[i]:
            k = nplh[i]
            while True:
                k -= 1
                if k < 0:
                    break
                parent[node] = pidx
                node += 1
                k -= 1
                if k >= 0:
                    parent[node] = pidx
                    node += 1
                pidx += 1
            if j & 1 or j == nplv[i] - 1:
                pidx0 = pidx
            else:
                pidx = pidx0
                pidx0 = pidx0 + nplh[i]
            j += 1
    return parent


def _tagtree_parents_standard(nw, nh):
    dims = []
    w, h = nw, nh
    while True:
        dims.append((w, h))
        if w * h <= 1:
            break
        w, h = (w + 1) // 2, (h + 1) // 2
    base = [0]
    for d in dims:
        base.append(base[-1] + d[0] * d[1])
    parent = [-1] * base[-1]
    for l in range(len(dims) - 1):
        for j in range(dims[l][1]):
            for i in range(dims[l][0]):
                parent[base[l] + j * dims[l][0] + i] = base[l + 1] + (j // 2) * dims[l + 1][0] + i // 2
    return parent


def test_tag_tree_parent_rule_matches_reference_walk():
    for nw in range(1, 40):
        for nh in range(1, 40):
            assert _tagtree_parents_reference_walk(nw, nh) == _tagtree_parents_standard(nw, nh)


# ------------------------------------------------------------------ PCRD ----
def _pcrd(orc, cum, dist, lam):
    import ctypes
    cum = np.array(cum, np.uint32)
    dist = np.array(dist, np.float64)
    hp = np.zeros(64, np.int32)
    hs = np.zeros(64, np.float64)
    n = ctypes.c_int()
    keep = orc.lib.orc_pcrd_select(cum.ctypes.data_as(ctypes.c_void_p), dist.ctypes.data_as(ctypes.c_void_p),
                                   len(cum), ctypes.c_double(lam), hp.ctypes.data_as(ctypes.c_void_p),
                                   hs.ctypes.data_as(ctypes.c_void_p), ctypes.byref(n))
    return keep, hp[:n.value], hs[:n.value]


@pytest.mark.parametrize("lam,keep", [(20.0, 0), (6.0, 1), (3.0, 2), (0.75, 3), (0.1, 4)])
def test_choose_block_point_obeys_lambda(orc, lam, keep):
    """src/dwt/pcrd.rs:1080-1095"""
    k, _, _ = _pcrd(orc, [10, 20, 30, 40], [100.0, 50.0, 20.0, 5.0], lam)
    assert k == keep


def test_hull_prunes_non_convex_and_equal_slopes(orc):
    """pcrd.rs:1054-1078 and pcrd.rs:1232-1260"""
    _, hp, hs = _pcrd(orc, [10, 20, 30], [100.0, 120.0, 10.0], 0.0)
    assert len(hp) < 4
    assert all(hs[i] < hs[i - 1] for i in range(2, len(hs)))
    _, hp, hs = _pcrd(orc, [10, 20, 30], [100.0, 100.0, 20.0], 0.0)
    assert len(hp) < 4
    assert all(hs[i] < hs[i - 1] for i in range(2, len(hs)))


def test_quality_to_lambda_shape(orc):
    """pcrd.rs:1425-1456: decreasing in quality, 0 at 100."""
    f = orc.lib.orc_quality_to_lambda
    vals = [f(q, 12_000_000) for q in range(1, 100)]
    assert all(b <= a for a, b in zip(vals, vals[1:]))
    assert f(100, 12_000_000) == 0.0


# ----------------------------------------------------------- end to end ----
def test_gray_lossless_jp2_roundtrip(orc):
    """src/decode/mod.rs:486-508"""
    w = h = 32
    px = np.array([((x * 7 + y * 11 + (x ^ y)) & 0xFF) for y in range(h) for x in range(w)], np.uint8)
    data = orc.encode(px, w, h, 1, 100, fmt=1)
    dw, dh, dc, dec = orc.decode(data)
    assert (dw, dh, dc) == (w, h, 1)
    assert np.array_equal(dec, px)


# The reference's literal codestream-writer vectors (src/j2k/mod.rs:44-133),
# under the plan of a 1x1 gray page at Preset::DocumentHigh's quality (the
# plan only matters for SIZ/COD/QCD segments of its own lengths, which these
# opaque segments are not). The oracle's encoder frames every codestream
# with this same writer (build_codestream -> frame_codestream).
_DOCUMENT_HIGH = 85  # Preset::DocumentHigh.quality() (src/model.rs:54-61)
_LITERAL_PARSED = bytes([
    0xff, 0x4f, 0xff, 0x51, 0x00, 0x04, 0x12, 0x34, 0xff, 0x52, 0x00, 0x05, 0xaa, 0xbb,
    0xcc, 0xff, 0x90, 0x00, 0x0a, 0x00, 0x00, 0x00, 0x00, 0x00, 0x17, 0x00, 0x00, 0xff,
    0x64, 0x00, 0x03, 0x01, 0xff, 0x93, 0xde, 0xad, 0xbe, 0xef, 0xff, 0xd9,
])
_LITERAL_WRITTEN = bytes([
    0xff, 0x4f, 0xff, 0x51, 0x00, 0x04, 0x12, 0x34, 0xff, 0x52, 0x00, 0x05, 0xaa, 0xbb,
    0xcc, 0xff, 0x90, 0x00, 0x0a, 0x00, 0x00, 0x00, 0x00, 0x00, 0x18, 0x00, 0x00, 0xff,
    0x64, 0x00, 0x03, 0x01, 0xff, 0x93, 0x10, 0x20, 0x30, 0x40, 0x50, 0xff, 0xd9,
])


def test_parser_reemits_single_tile_codestream(orc):
    """j2k/mod.rs:44-76: parse a single-tile codestream and write it again."""
    assert orc.reframe(_LITERAL_PARSED, 1, 1, 1, _DOCUMENT_HIGH) == _LITERAL_PARSED


def test_writer_accepts_locally_constructed_packet_sequence(orc):
    """j2k/mod.rs:78-133: two opaque main-header segments, one tile-part
    (tile 0, part 0, 0 parts) with a COM segment and a payload of a
    header+body packet (10 20 | 30) and an opaque packet (40 50)."""
    main = bytes([0xff, 0x51, 0x00, 0x04, 0x12, 0x34, 0xff, 0x52, 0x00, 0x05, 0xaa, 0xbb, 0xcc])
    tile_hdr = bytes([0xff, 0x64, 0x00, 0x03, 0x01])
    payload = bytes([0x10, 0x20, 0x30, 0x40, 0x50])
    assert orc.frame(1, 1, 1, _DOCUMENT_HIGH, main, tile_hdr, payload, 0, 0, 0) == _LITERAL_WRITTEN


def test_encoder_codestream_is_the_writer_framing(orc):
    """An encoded codestream re-frames to itself: its SIZ/COD/QCD are the
    plan's own segments and its SOT carries tile 0, part 0 of 1 with
    Psot = 12 + 2 + payload (backend.rs:275-290)."""
    px = np.arange(64, dtype=np.uint8)
    for q in (85, 100):
        cs = orc.encode(px, 8, 8, 1, q, fmt=0)
        assert orc.reframe(cs, 8, 8, 1, q) == cs
        sot = cs.index(b"\xff\x90")
        psot = int.from_bytes(cs[sot + 6:sot + 10], "big")
        assert sot + psot == len(cs) - 2
        assert cs[sot + 10:sot + 14] == b"\x00\x01\xff\x93"


def test_synthetic_rgb_quality_sweep_is_valid_jp2(orc):
    """tests/visual_output.rs:140-176: valid JP2 >= 64 bytes at every quality."""
    w = h = 64
    y, x = np.mgrid[0:h, 0:w]
    px = np.stack([(x * 4) & 255, (y * 4) & 255, ((x + y) * 2) & 255], -1).astype(np.uint8).ravel()
    for q in (1, 10, 25, 50, 75, 90, 99):
        data = orc.encode(px, w, h, 3, q, fmt=1)
        assert data[4:8] == b"jP  " and len(data) >= 64
        dw, dh, dc, _ = orc.decode(data)
        assert (dw, dh, dc) == (w, h, 3)


def test_lossy_quality_ladder_sizes_increase(orc):
    """tests/lossy_quality.rs:100-196 on a synthetic page (lear.png is not in
    the mount): sizes strictly increase over q1 < q10 < q25 < q50 < q75."""
    rng = np.random.default_rng(0)
    w, h = 128, 96
    base = np.clip(128 + 60 * np.sin(np.arange(w * h) / 37.0) + rng.normal(0, 20, w * h), 0, 255)
    px = base.astype(np.uint8)
    sizes = [len(orc.encode(px, w, h, 1, q, fmt=1)) for q in (1, 10, 25, 50, 75)]
    assert all(b > a for a, b in zip(sizes, sizes[1:])), sizes


def test_lossy_decode_psnr_near_encoder_estimate(orc):
    """encode_with_psnr's internal estimate (backend.rs:305-433) and a real
    decode of the same stream land close together; they are not identical by
    design (the estimate truncates whole bit-planes, the decoder stops at the
    retained pass)."""
    rng = np.random.default_rng(1)
    w, h = 96, 80
    px = np.clip(rng.normal(128, 40, w * h), 0, 255).astype(np.uint8)
    data = orc.encode(px, w, h, 1, 75, fmt=1)
    _, _, _, dec = orc.decode(data)
    mse = np.mean((dec.astype(np.float64) - px) ** 2)
    psnr_dec = 10 * np.log10(255.0 ** 2 / mse)
    psnr_est, ssim = orc.quality_metrics(px, w, h, 1, 75)
    assert psnr_dec > 20.0 and 0.0 < ssim <= 1.0
    assert abs(psnr_dec - psnr_est) < 2.0


def test_rgb_lossless_chroma_needs_the_extra_bitplane_to_decode(orc):
    """At q >= 100 with RCT the encoder codes chroma with precision + 1
    (backend.rs:179-189) while QCD carries component 0's exponents
    (plan/mod.rs:141-145); the reference's decoder takes Mb from QCD
    (decode/t1.rs:56) and rejects more passes than 1 + 3 (Mb - 1)
    (decode/t1.rs:121-126). So its own sRGB lossless output does not decode
    with its own decoder, and reads back exactly once chroma is given the
    extra bit-plane. Byte identity with the reference stays the parity mode."""
    for w, h in ((64, 64), (7, 3), (333, 211)):
        y, x = np.mgrid[0:h, 0:w]
        px = np.stack([(x * 5 + y) & 255, (y * 3) & 255, ((x ^ y) * 7) & 255], -1).astype(np.uint8).ravel()
        data = orc.encode(px, w, h, 3, 100, fmt=1)
        with pytest.raises(RuntimeError, match="pass count exceeds maximum"):
            orc.decode(data)
        dw, dh, dc, dec = orc.decode(data, rct_chroma_extra_bitplane=True)
        assert (dw, dh, dc) == (w, h, 3)
        assert np.array_equal(dec, px)
    gray = np.arange(64 * 64, dtype=np.uint32).astype(np.uint8)
    assert np.array_equal(orc.decode(orc.encode(gray, 64, 64, 1, 100, fmt=1))[3], gray)


def test_empty_segment_blocks_are_rejected_by_the_reference_decoder(orc):
    """Some lossy outputs keep a single cleanup pass whose MQ byte count is 0
    (the pass's rate in the R-D curve), so the packet carries a code-block
    with one pass and no bytes. The reference's decoder rejects it
    (decode/t1.rs:109-111); decoded from an all-0xFF stream (C.3.4) it reads
    back like its neighbours."""
    from jp2lam_gb300._native import synth_page
    for w, h, c, q, seed in ((7, 3, 3, 40, 303), (257, 129, 1, 95, 307)):
        px = synth_page(w, h, c, seed, photo_w=max(w // 3, 1), photo_h=max(h // 3, 1))
        rows = orc.block_summary(px, w, h, c, q)
        assert ((rows[:, 7] == 1) & (rows[:, 8] == 0)).any()
        data = orc.encode(px, w, h, c, q, fmt=0)
        with pytest.raises(RuntimeError, match="no compressed bytes"):
            orc.decode(data)
        dw, dh, dc, dec = orc.decode(data, accept_empty_segments=True)
        assert (dw, dh, dc) == (w, h, c)
        err = np.abs(dec.astype(int) - px.astype(int))
        assert err.mean() < 16
